// Per-step model set-up on the device: the eigen system of a reversible rate
// matrix and the discretised Gamma rates, both in FP64.
//
// tt_reversible_eigen replaces the eigendecomposition in
// SymmetricSubstitutionModel.p_t (torchtree/evolution/substitution_model/
// abstract.py:57-79): with Pi = diag(pi), the symmetric matrix
// A = Pi^1/2 Q Pi^-1/2 is diagonalised as A = V diag(lambda) V^T (torch's
// eigh reads the lower triangle; so does this kernel), and
// Q = U diag(lambda) W with U = Pi^-1/2 V, W = V^T Pi^1/2 (V is orthogonal,
// so W is the inverse of U without a matrix inverse).
//
// FP64 arithmetic is scarce on this GPU (a few FP64 FMAs per cycle per SM),
// so the solver does most of its sweeps in FP32 and spreads the FP64 matrix
// products over many CTAs:
//  1. eigen_start_kernel, one CTA per matrix: cyclic Jacobi in FP32 (parallel
//     round-robin ordering of Brent and Luk, 1985; each rotation Golub & Van
//     Loan, Algorithm 8.4.2 "sym.schur2"): eigenvectors X0 good to ~1e-5;
//  2. two Newton-Schulz steps X <- X (3I - X^T X) / 2 (Higham, "Functions of
//     Matrices", 8.3) in FP64, each squaring X's distance from orthonormal
//     (eigen_gram_kernel forms R = I - X^T X, eigen_orth_kernel X <- X + X R/2),
//     kEigRows rows of the products per CTA;
//  3. eigen_gram_kernel forms S = X^T A X (off-diagonal ~1e-5 of its norm) and
//     eigen_finish_kernel, one CTA per matrix, diagonalises S by FP64 Jacobi
//     sweeps accumulated into X (quadratic convergence from there: two or
//     three sweeps) to 1e-14 of the Frobenius norm.
// A matrix whose FP64 sweeps do not converge (30 of them) sets the status
// word to TT_ERR_UNSUPPORTED.  Eigenvalues are returned in ascending order,
// as eigh returns them.  The buffers u, w and eigenvalues hold X, S / R and
// R's diagonal between the steps, so the call needs no workspace.
#include <math.h>

#include <cooperative_groups.h>

#include <algorithm>
#include <string>

#include "../../include/torchtree_gb300.h"
#include "tt_gamma.cuh"
#include "tt_launch.h"

namespace tt {

namespace {

constexpr int kEigMax = 64;      // largest state count
constexpr int kEigLd = kEigMax + 1;
constexpr int kEigThreads = 256;
constexpr int kEigRows = 4;  // rows of the FP64 products per CTA

// pair i of round r in the round-robin over m players (m even): player m-1
// stays, the others rotate
__device__ __forceinline__ void rr_pair(int r, int i, int m, int &p, int &q) {
  if (i == 0) {
    p = r;
    q = m - 1;
  } else {
    p = (r + i) % (m - 1);
    q = (r - i + (m - 1)) % (m - 1);
  }
  if (p > q) {
    const int t = p;
    p = q;
    q = t;
  }
}

// The Jacobi rotation (c, s) that zeroes a_pq of [[a_pp, a_pq], [a_pq, a_qq]]
// in FP64.  FP64 division and square root are long dependency chains on this
// GPU, and every round waits for its rotations: the angle to FP32 accuracy (a
// slightly inexact angle leaves a residual the next sweep removes), then
// c = (1 + t^2)^-1/2 from an FP32 seed by two Newton steps y <- y (3 - x y^2) / 2
// in FP64, so that c^2 + s^2 = 1 to FP64 rounding and the rotation stays
// orthogonal.  a_pq != 0.
__device__ __forceinline__ void jacobi_rotation_f64(double app, double aqq, double apq, double &c, double &s) {
  c = 1.0;
  s = 0.0;
  if (apq == 0.0) return;
  const float tf = float(aqq - app) / float(2.0 * apq);
  float t32;
  if (!(fabsf(tf) <= 1e18f)) t32 = 0.5f / tf;
  else t32 = (tf >= 0.0f ? 1.0f : -1.0f) / (fabsf(tf) + sqrtf(1.0f + tf * tf));
  const double t = double(t32), x = 1.0 + t * t;
  double y = double(rsqrtf(float(x)));
  y = y * (1.5 - 0.5 * x * y * y);
  y = y * (1.5 - 0.5 * x * y * y);
  c = y;
  s = t * y;
}

// Cyclic Jacobi sweeps on A (n x n, leading dimension kEigLd) accumulating
// the rotations into V, in T arithmetic, until the off-diagonal norm squared
// is at most tol2 times the Frobenius norm squared; true when converged within
// max_sweeps.  cs and pq hold a round's rotations and pairs.  Called by the
// whole CTA.
template <typename T>
__device__ bool jacobi_sweeps(T *A, T *V, T *cs, int *pq, double *red, int *flag, int n, double tol2,
                              int max_sweeps) {
  constexpr int NW = kEigThreads / 32;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int m = n + (n & 1);  // an odd n gets a dummy player that never rotates
  const int npairs = m / 2;
  for (int sweep = 0; sweep <= max_sweeps; ++sweep) {
    // convergence: off-diagonal norm against the Frobenius norm
    double off = 0.0, tot = 0.0;
    for (int i = warp; i < n; i += NW)
      for (int j = lane; j < n; j += 32) {
        const double v = double(A[i * kEigLd + j]);
        tot += v * v;
        if (i != j) off += v * v;
      }
    for (int o = 16; o; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      tot += __shfl_xor_sync(0xffffffffu, tot, o);
    }
    if (lane == 0) {
      red[warp] = off;
      red[NW + warp] = tot;
    }
    __syncthreads();
    if (tid == 0) {
      double so = 0.0, st = 0.0;
      for (int w = 0; w < NW; ++w) {
        so += red[w];
        st += red[NW + w];
      }
      *flag = !(so > tol2 * st) || n == 1;
    }
    __syncthreads();
    if (*flag) return true;
    if (sweep == max_sweeps) return false;
    for (int r = 0; r < m - 1; ++r) {
      // this round's pairs and rotations
      if (tid < npairs) {
        int p, qq;
        rr_pair(r, tid, m, p, qq);
        T c = T(1), s = T(0);
        if (qq < n) {
          const T apq = A[p * kEigLd + qq];
          if (apq != T(0)) {
            if constexpr (sizeof(T) == 4) {
              const T tau = (A[qq * kEigLd + qq] - A[p * kEigLd + p]) / (T(2) * apq);
              T t;
              if (fabs(tau) > T(1e18)) t = T(0.5) / tau;
              else t = (tau >= T(0) ? T(1) : T(-1)) / (fabs(tau) + sqrt(T(1) + tau * tau));
              c = T(1) / sqrt(T(1) + t * t);
              s = t * c;
            } else {
              double cd, sd;
              jacobi_rotation_f64(A[p * kEigLd + p], A[qq * kEigLd + qq], apq, cd, sd);
              c = T(cd);
              s = T(sd);
            }
          }
        }
        cs[2 * tid] = c;
        cs[2 * tid + 1] = s;
        pq[2 * tid] = p;
        pq[2 * tid + 1] = qq;
      }
      __syncthreads();
      // rows: A <- J^T A (rows p, q of every pair), a warp per pair, lanes
      // along the row.  Distinct pairs touch distinct rows, so all of a
      // thread's loads go first (independent shared-memory latencies).
      {
        constexpr int PK = (kEigMax / 2 + NW - 1) / NW;  // pairs per warp
        T ap[PK][2], aq[PK][2], cr[PK], sr[PK];
        int pr[PK], qr[PK];
#pragma unroll
        for (int k = 0; k < PK; ++k) {
          const int i = warp + k * NW;
          pr[k] = i < npairs ? pq[2 * i] : 0;
          qr[k] = i < npairs ? pq[2 * i + 1] : n;
          cr[k] = i < npairs ? cs[2 * i] : T(1);
          sr[k] = i < npairs ? cs[2 * i + 1] : T(0);
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int j = lane + 32 * h;
            const bool go = qr[k] < n && sr[k] != T(0) && j < n;  // not the dummy player nor the identity
            ap[k][h] = go ? A[pr[k] * kEigLd + j] : T(0);
            aq[k][h] = go ? A[qr[k] * kEigLd + j] : T(0);
          }
        }
#pragma unroll
        for (int k = 0; k < PK; ++k)
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int j = lane + 32 * h;
            if (qr[k] < n && sr[k] != T(0) && j < n) {
              A[pr[k] * kEigLd + j] = cr[k] * ap[k][h] - sr[k] * aq[k][h];
              A[qr[k] * kEigLd + j] = sr[k] * ap[k][h] + cr[k] * aq[k][h];
            }
          }
      }
      __syncthreads();
      // columns: A <- A J, V <- V J, a warp per row, lanes over the pairs
      {
        constexpr int RK = (kEigMax + NW - 1) / NW;  // rows per warp
        const int i = lane;                           // npairs <= 32
        const int pc = i < npairs ? pq[2 * i] : 0, qc = i < npairs ? pq[2 * i + 1] : n;
        const T c = i < npairs ? cs[2 * i] : T(1), s = i < npairs ? cs[2 * i + 1] : T(0);
        const bool go = qc < n && s != T(0);
        T a0[RK], a1[RK], v0[RK], v1[RK];
#pragma unroll
        for (int k = 0; k < RK; ++k) {
          const int row = warp + k * NW;
          const bool g = go && row < n;
          a0[k] = g ? A[row * kEigLd + pc] : T(0);
          a1[k] = g ? A[row * kEigLd + qc] : T(0);
          v0[k] = g ? V[row * kEigLd + pc] : T(0);
          v1[k] = g ? V[row * kEigLd + qc] : T(0);
        }
#pragma unroll
        for (int k = 0; k < RK; ++k) {
          const int row = warp + k * NW;
          if (go && row < n) {
            A[row * kEigLd + pc] = c * a0[k] - s * a1[k];
            A[row * kEigLd + qc] = s * a0[k] + c * a1[k];
            V[row * kEigLd + pc] = c * v0[k] - s * v1[k];
            V[row * kEigLd + qc] = s * v0[k] + c * v1[k];
          }
        }
      }
      __syncthreads();
    }
  }
  return false;
}

// sqrt(pi) of matrix b into sq, then A = Pi^1/2 Q Pi^-1/2 from the lower
// triangle (mirrored) into A (leading dimension kEigLd) as T; whole CTA.
template <typename T>
__device__ void load_symmetrised(const double *q, const double *pi, int b, int n, double *sq, T *A) {
  constexpr int NW = kEigThreads / 32;
  const double *qb = q + size_t(b) * n * n;
  for (int i = threadIdx.x; i < n; i += kEigThreads) sq[i] = sqrt(pi[size_t(b) * n + i]);
  __syncthreads();
  for (int i = threadIdx.x >> 5; i < n; i += NW)
    for (int j = threadIdx.x & 31; j < n; j += 32) {
      const int r = i >= j ? i : j, c = i >= j ? j : i;
      A[i * kEigLd + j] = T(sq[r] * qb[r * n + c] / sq[c]);
    }
  __syncthreads();
}

// Step 1, one CTA per matrix: FP32 Jacobi sweeps on A until the off-diagonal
// norm is below 1e-6 of the Frobenius norm (at most 6 sweeps: FP32 rounding
// may stop short of that); the eigenvector matrix X0, in FP64, into x.
__global__ void __launch_bounds__(kEigThreads) eigen_start_kernel(const double *q, const double *pi, int n,
                                                                  double *x) {
  constexpr int NW = kEigThreads / 32;
  __shared__ float A[kEigMax * kEigLd], V[kEigMax * kEigLd], cs[kEigMax];
  __shared__ int pq[kEigMax];
  __shared__ double red[2 * NW], sq[kEigMax];
  __shared__ int flag;
  const int b = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  load_symmetrised(q, pi, b, n, sq, A);
  for (int i = warp; i < n; i += NW)
    for (int j = lane; j < n; j += 32) V[i * kEigLd + j] = i == j ? 1.0f : 0.0f;
  __syncthreads();
  jacobi_sweeps<float>(A, V, cs, pq, red, &flag, n, 1e-12, 6);
  double *xb = x + size_t(b) * n * n;
  for (int i = warp; i < n; i += NW)
    for (int j = lane; j < n; j += 32) xb[i * n + j] = double(V[i * kEigLd + j]);
}

// Step 2 / 3, kEigRows rows per CTA (grid: row blocks x matrices), FP64: for
// the current eigenvector estimate X (x),
//   R = I - X^T X   (strict lower triangle into w, diagonal into lam),
//   S = X^T A X     (upper triangle with the diagonal into w; with_s only).
// Both are symmetric, so one n x n buffer holds the two.
__global__ void __launch_bounds__(kEigThreads) eigen_gram_kernel(const double *q, const double *pi, int n,
                                                                 const double *x, double *w, double *lam,
                                                                 int with_s) {
  constexpr int NW = kEigThreads / 32;
  extern __shared__ __align__(16) double gsm[];
  double *A = gsm;                      // [n][kEigLd]
  double *X = A + kEigMax * kEigLd;     // [n][kEigLd]
  double *M = X + kEigMax * kEigLd;     // [kEigRows][kEigLd]: rows of X^T A
  double *sq = M + kEigRows * kEigLd;   // [n]
  const int b = blockIdx.y, i0 = blockIdx.x * kEigRows, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int rows = min(kEigRows, n - i0);
  const double *xb = x + size_t(b) * n * n;
  for (int i = warp; i < n; i += NW)
    for (int j = lane; j < n; j += 32) X[i * kEigLd + j] = xb[i * n + j];
  if (with_s) load_symmetrised(q, pi, b, n, sq, A);
  else __syncthreads();
  double *wb = w + size_t(b) * n * n;
  // R rows i0 .. i0 + rows - 1, columns j <= i; two warps per row
  for (int t = warp; t < 2 * rows; t += NW) {
    const int r = t >> 1, i = i0 + r;
    for (int j = (t & 1) * 32 + lane; j <= i; j += 64) {
      double s = 0.0;
      for (int k = 0; k < n; ++k) s = fma(X[k * kEigLd + i], X[k * kEigLd + j], s);
      if (j < i) wb[i * n + j] = -s;
      else lam[size_t(b) * n + i] = 1.0 - s;
    }
  }
  if (!with_s) return;
  for (int t = warp; t < 2 * rows; t += NW) {
    const int r = t >> 1, i = i0 + r;
    for (int j = (t & 1) * 32 + lane; j < n; j += 64) {
      double s = 0.0;
      for (int k = 0; k < n; ++k) s = fma(X[k * kEigLd + i], A[k * kEigLd + j], s);
      M[r * kEigLd + j] = s;
    }
  }
  __syncthreads();
  for (int t = warp; t < 2 * rows; t += NW) {
    const int r = t >> 1, i = i0 + r;
    for (int j = i + (t & 1) * 32 + lane; j < n; j += 64) {
      double s = 0.0;
      for (int k = 0; k < n; ++k) s = fma(M[r * kEigLd + k], X[k * kEigLd + j], s);
      wb[i * n + j] = s;
    }
  }
}

// Step 2, kEigRows rows per CTA, FP64: one Newton-Schulz step
// X <- X + X R / 2 = X (3I - X^T X) / 2 with R = I - X^T X from the last
// eigen_gram_kernel.  A row of the result needs only that row of X, so each
// CTA updates its own rows in place.
__global__ void __launch_bounds__(kEigThreads) eigen_orth_kernel(int n, double *x, const double *w,
                                                                 const double *lam) {
  constexpr int NW = kEigThreads / 32;
  extern __shared__ __align__(16) double osm[];
  double *R = osm;                      // [n][kEigLd], halved
  double *Xr = R + kEigMax * kEigLd;    // [kEigRows][kEigLd]
  const int b = blockIdx.y, i0 = blockIdx.x * kEigRows, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int rows = min(kEigRows, n - i0);
  const double *wb = w + size_t(b) * n * n, *rd = lam + size_t(b) * n;
  double *xb = x + size_t(b) * n * n;
  for (int i = warp; i < n; i += NW)
    for (int j = lane; j < n; j += 32)
      R[i * kEigLd + j] = 0.5 * (i == j ? rd[i] : wb[max(i, j) * n + min(i, j)]);
  for (int r = warp; r < rows; r += NW)
    for (int j = lane; j < n; j += 32) Xr[r * kEigLd + j] = xb[(i0 + r) * n + j];
  __syncthreads();
  for (int t = warp; t < 2 * rows; t += NW) {
    const int r = t >> 1;
    for (int j = (t & 1) * 32 + lane; j < n; j += 64) {
      double s = Xr[r * kEigLd + j];
      for (int k = 0; k < n; ++k) s = fma(Xr[r * kEigLd + k], R[k * kEigLd + j], s);
      xb[(i0 + r) * n + j] = s;
    }
  }
}

// Step 3, one CTA per matrix, FP64: S = X^T A X (in W, upper triangle) and X
// (in U); FP64 Jacobi sweeps on S, accumulated into X, to 1e-14 of the
// Frobenius norm; a matrix that does not converge in 30 sweeps sets the
// status word.  Eigenvalues ascending, with U = Pi^-1/2 X and W = X^T Pi^1/2.
__global__ void __launch_bounds__(kEigThreads) eigen_finish_kernel(const double *pi, int n, double *lam, double *U,
                                                                   double *W, int *status) {
  constexpr int NW = kEigThreads / 32;
  extern __shared__ __align__(16) double fsm[];
  double *A = fsm;                       // [n][kEigLd] S, symmetric
  double *V = A + kEigMax * kEigLd;      // [n][kEigLd] X
  double *cs = V + kEigMax * kEigLd;     // [kEigMax/2][2]
  double *red = cs + kEigMax;            // [2 * NW]
  double *sq = red + 2 * NW;             // [n]
  int *pq = reinterpret_cast<int *>(sq + kEigMax);  // [kEigMax/2][2]
  __shared__ int flag;
  const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const size_t mo = size_t(b) * n * n;
  for (int i = tid; i < n; i += kEigThreads) sq[i] = sqrt(pi[size_t(b) * n + i]);
  for (int i = warp; i < n; i += NW)
    for (int j = lane; j < n; j += 32) {
      A[i * kEigLd + j] = W[mo + size_t(min(i, j)) * n + max(i, j)];
      V[i * kEigLd + j] = U[mo + size_t(i) * n + j];
    }
  __syncthreads();
  // (every thread's reads of U and W are done: the sweeps begin with a barrier)
  const bool ok = jacobi_sweeps<double>(A, V, cs, pq, red, &flag, n, 1e-28, 30);
  if (tid == 0 && !ok) atomicExch(status, TT_ERR_UNSUPPORTED);
  // ascending order: the rank of each eigenvalue (ties by index)
  for (int k = tid; k < n; k += kEigThreads) {
    const double lk = A[k * kEigLd + k];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const double lj = A[j * kEigLd + j];
      rank += lj < lk || (lj == lk && j < k);
    }
    lam[size_t(b) * n + rank] = lk;
    for (int i = 0; i < n; ++i) {
      U[(size_t(b) * n + i) * n + rank] = V[i * kEigLd + k] / sq[i];  // U = Pi^-1/2 V
      W[(size_t(b) * n + rank) * n + i] = V[i * kEigLd + k] * sq[i];  // W = V^T Pi^1/2
    }
  }
}

// Step 3 for matrices of more than 32 states: the same FP64 Jacobi sweeps on
// a cluster of kEigCluster CTAs per matrix (FP64 arithmetic on one SM bounds
// the single-CTA sweeps).  Every CTA keeps a copy of A; each round, all CTAs
// form the same rotations from their identical copies, a CTA updates the rows
// p, q of its share of the pairs (pairs i = rank mod kEigCluster) and writes
// them into every copy through distributed shared memory, then, after a
// cluster barrier, updates columns p, q of its share of the rows (rows = rank
// mod kEigCluster) in every copy of A and in its own rows of V.  The
// convergence test runs on each CTA's (identical) copy, so every CTA leaves
// the sweeps together.  Each CTA writes its rows of U and W.
constexpr int kEigCluster = 4;

__global__ void __cluster_dims__(kEigCluster, 1, 1) __launch_bounds__(kEigThreads)
    eigen_finish_cluster_kernel(const double *pi, int n, double *lam, double *U, double *W, int *status) {
  namespace cg = cooperative_groups;
  constexpr int NW = kEigThreads / 32, C = kEigCluster;
  extern __shared__ __align__(16) double csm[];
  double *A = csm;                       // [n][kEigLd] S, symmetric (a copy per CTA)
  double *V = A + kEigMax * kEigLd;      // [n][kEigLd] X (rows = rank mod C are this CTA's)
  double *cs = V + kEigMax * kEigLd;     // [kEigMax/2][2]
  double *red = cs + kEigMax;            // [2 * NW]
  double *sq = red + 2 * NW;             // [n]
  int *pq = reinterpret_cast<int *>(sq + kEigMax);  // [kEigMax/2][2]
  __shared__ int flag;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = int(cluster.block_rank());
  const int b = blockIdx.x / C, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  double *Ac[C];
#pragma unroll
  for (int q = 0; q < C; ++q) Ac[q] = cluster.map_shared_rank(A, q);
  const size_t mo = size_t(b) * n * n;
  for (int i = tid; i < n; i += kEigThreads) sq[i] = sqrt(pi[size_t(b) * n + i]);
  for (int i = warp; i < n; i += NW)
    for (int j = lane; j < n; j += 32) {
      A[i * kEigLd + j] = W[mo + size_t(min(i, j)) * n + max(i, j)];
      if (i % C == rank) V[i * kEigLd + j] = U[mo + size_t(i) * n + j];
    }
  cluster.sync();  // every CTA has read U and W before any writes its outputs
  const int m = n + (n & 1), npairs = m / 2;
  bool ok = false;
  for (int sweep = 0; sweep <= 30; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = warp; i < n; i += NW)
      for (int j = lane; j < n; j += 32) {
        const double v = A[i * kEigLd + j];
        tot += v * v;
        if (i != j) off += v * v;
      }
    for (int o = 16; o; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      tot += __shfl_xor_sync(0xffffffffu, tot, o);
    }
    if (lane == 0) {
      red[warp] = off;
      red[NW + warp] = tot;
    }
    __syncthreads();
    if (tid == 0) {
      double so = 0.0, st = 0.0;
      for (int w = 0; w < NW; ++w) {
        so += red[w];
        st += red[NW + w];
      }
      flag = !(so > 1e-28 * st) || n == 1;
    }
    __syncthreads();
    if (flag) {
      ok = true;
      break;
    }
    if (sweep == 30) break;
    for (int r = 0; r < m - 1; ++r) {
      if (tid < npairs) {  // the round's rotations, the same in every CTA
        int p, qq;
        rr_pair(r, tid, m, p, qq);
        double c = 1.0, sn = 0.0;
        if (qq < n) jacobi_rotation_f64(A[p * kEigLd + p], A[qq * kEigLd + qq], A[p * kEigLd + qq], c, sn);
        cs[2 * tid] = c;
        cs[2 * tid + 1] = sn;
        pq[2 * tid] = p;
        pq[2 * tid + 1] = qq;
      }
      __syncthreads();
      // rows p, q of this CTA's pairs (a warp per pair), into every copy
      for (int i = rank + C * warp; i < npairs; i += C * NW) {
        const int p = pq[2 * i], qq = pq[2 * i + 1];
        const double c = cs[2 * i], sn = cs[2 * i + 1];
        if (qq >= n || sn == 0.0) continue;
        double np_[2], nq_[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int j = lane + 32 * h;
          const double ap = j < n ? A[p * kEigLd + j] : 0.0, aq = j < n ? A[qq * kEigLd + j] : 0.0;
          np_[h] = c * ap - sn * aq;
          nq_[h] = sn * ap + c * aq;
        }
#pragma unroll
        for (int q = 0; q < C; ++q)
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int j = lane + 32 * h;
            if (j < n) {
              Ac[q][p * kEigLd + j] = np_[h];
              Ac[q][qq * kEigLd + j] = nq_[h];
            }
          }
      }
      cluster.sync();
      // columns p, q of this CTA's rows (a warp per row, lanes over the pairs), into every copy of
      // A and this CTA's rows of V
      for (int row = rank + C * warp; row < n; row += C * NW) {
        const int i = lane;
        if (i >= npairs) continue;
        const int p = pq[2 * i], qq = pq[2 * i + 1];
        const double c = cs[2 * i], sn = cs[2 * i + 1];
        if (qq >= n || sn == 0.0) continue;
        const double ap = A[row * kEigLd + p], aq = A[row * kEigLd + qq];
        const double np_ = c * ap - sn * aq, nq_ = sn * ap + c * aq;
#pragma unroll
        for (int q = 0; q < C; ++q) {
          Ac[q][row * kEigLd + p] = np_;
          Ac[q][row * kEigLd + qq] = nq_;
        }
        const double vp = V[row * kEigLd + p], vq = V[row * kEigLd + qq];
        V[row * kEigLd + p] = c * vp - sn * vq;
        V[row * kEigLd + qq] = sn * vp + c * vq;
      }
      cluster.sync();
    }
  }
  if (tid == 0 && rank == 0 && !ok) atomicExch(status, TT_ERR_UNSUPPORTED);
  // ascending order: the rank of each eigenvalue (ties by index); this CTA's rows of U and W
  for (int k = tid; k < n; k += kEigThreads) {
    const double lk = A[k * kEigLd + k];
    int rk = 0;
    for (int j = 0; j < n; ++j) {
      const double lj = A[j * kEigLd + j];
      rk += lj < lk || (lj == lk && j < k);
    }
    if (rank == 0) lam[size_t(b) * n + rk] = lk;
    for (int i = rank; i < n; i += C) {
      U[(size_t(b) * n + i) * n + rk] = V[i * kEigLd + k] / sq[i];  // U = Pi^-1/2 V
      W[(size_t(b) * n + rk) * n + i] = V[i * kEigLd + k] * sq[i];  // W = V^T Pi^1/2
    }
  }
  cluster.sync();  // no CTA leaves while another may still write into its shared memory
}

__global__ void gamma_quantiles_kernel(const double *shape, int batch, int K, double *x, double *dxda) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= batch * K) return;
  const int b = e / K, k = e - b * K;
  const double q = (2.0 * k + 1.0) / (2.0 * K);
  double xv = 0.0, dv = 0.0;
  if (!gamma_quantile(shape[b], q, xv, dv)) xv = dv = __longlong_as_double(0x7ff8000000000000ll);  // NaN
  x[e] = xv;
  dxda[e] = dv;
}

int efail(int code, const std::string &msg) { return record_error(code, msg.c_str()); }

}  // namespace

}  // namespace tt

extern "C" {

int tt_reversible_eigen(int32_t batch, int32_t state_count, const double *q, const double *frequencies,
                        double *eigenvalues, double *u, double *w, int32_t *status, void *stream) {
  if (!q || !frequencies || !eigenvalues || !u || !w || !status)
    return tt::efail(TT_ERR_INVALID_ARGUMENT, "NULL argument");
  if (batch < 1 || state_count < 1 || state_count > tt::kEigMax)
    return tt::efail(TT_ERR_INVALID_ARGUMENT, "tt_reversible_eigen: batch >= 1 and 1 <= state_count <= 64");
  using namespace tt;
  const int n = state_count;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t gram_smem = (2 * size_t(kEigMax) * kEigLd + kEigRows * kEigLd + kEigMax) * sizeof(double);
  const size_t orth_smem = (size_t(kEigMax) * kEigLd + kEigRows * kEigLd) * sizeof(double);
  const size_t finish_smem =
      (2 * size_t(kEigMax) * kEigLd + kEigMax + 2 * (kEigThreads / 32) + kEigMax) * sizeof(double) +
      kEigMax * sizeof(int);
  cudaError_t e = kernel_smem(eigen_gram_kernel, gram_smem);
  if (e == cudaSuccess) e = kernel_smem(eigen_orth_kernel, orth_smem);
  if (e == cudaSuccess) e = kernel_smem(eigen_finish_kernel, finish_smem);
  if (e == cudaSuccess) e = kernel_smem(eigen_finish_cluster_kernel, finish_smem);
  // matrices in groups of at most 65,535 (the grid's y extent of the row-block kernels)
  for (int b0 = 0; e == cudaSuccess && b0 < batch; b0 += 65535) {
    const int nb = std::min(batch - b0, 65535);
    const size_t mo = size_t(b0) * n * n, vo = size_t(b0) * n;
    const double *qb = q + mo, *pib = frequencies + vo;
    double *ub = u + mo, *wb = w + mo, *lb = eigenvalues + vo;
    const dim3 rows_grid((n + kEigRows - 1) / kEigRows, nb);
    eigen_start_kernel<<<nb, kEigThreads, 0, s>>>(qb, pib, n, ub);
    for (int it = 0; it < 2; ++it) {
      eigen_gram_kernel<<<rows_grid, kEigThreads, gram_smem, s>>>(qb, pib, n, ub, wb, lb, 0);
      eigen_orth_kernel<<<rows_grid, kEigThreads, orth_smem, s>>>(n, ub, wb, lb);
    }
    eigen_gram_kernel<<<rows_grid, kEigThreads, gram_smem, s>>>(qb, pib, n, ub, wb, lb, 1);
    if (n > 32)  // FP64 sweeps on a cluster of CTAs per matrix
      eigen_finish_cluster_kernel<<<nb * kEigCluster, kEigThreads, finish_smem, s>>>(pib, n, lb, ub, wb, status);
    else
      eigen_finish_kernel<<<nb, kEigThreads, finish_smem, s>>>(pib, n, lb, ub, wb, status);
    e = cudaGetLastError();
  }
  return e == cudaSuccess ? TT_OK : tt::efail(TT_ERR_CUDA, std::string("eigen launch: ") + cudaGetErrorString(e));
}

int tt_gamma_quantiles(int32_t batch, int32_t category_count, const double *shape, double *x, double *dx_dshape,
                       void *stream) {
  if (!shape || !x || !dx_dshape) return tt::efail(TT_ERR_INVALID_ARGUMENT, "NULL argument");
  if (batch < 1 || category_count < 1) return tt::efail(TT_ERR_INVALID_ARGUMENT, "batch and categories must be >= 1");
  const int n = batch * category_count;
  // one warp per CTA: the quantiles' FP64 work spreads over as many SMs as warps
  tt::gamma_quantiles_kernel<<<(n + 31) / 32, 32, 0, static_cast<cudaStream_t>(stream)>>>(
      shape, batch, category_count, x, dx_dshape);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? TT_OK
                          : tt::efail(TT_ERR_CUDA, std::string("gamma quantile launch: ") + cudaGetErrorString(e));
}

int tt_gamma_quantiles_host(int32_t batch, int32_t category_count, const double *shape, double *x,
                            double *dx_dshape) {
  if (!shape || !x || !dx_dshape) return tt::efail(TT_ERR_INVALID_ARGUMENT, "NULL argument");
  if (batch < 1 || category_count < 1) return tt::efail(TT_ERR_INVALID_ARGUMENT, "batch and categories must be >= 1");
  for (int b = 0; b < batch; ++b)
    for (int k = 0; k < category_count; ++k) {
      const double q = (2.0 * k + 1.0) / (2.0 * category_count);
      if (!tt::gamma_quantile(shape[b], q, x[b * category_count + k], dx_dshape[b * category_count + k]))
        return tt::efail(TT_ERR_INVALID_ARGUMENT, "Gamma quantile: the shape must be finite and > 0");
    }
  return TT_OK;
}

}  // extern "C"
