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
// The eigensolver is the cyclic Jacobi method with the parallel
// (round-robin) ordering of Brent and Luk (1985): one CTA per matrix, A and V
// in shared memory; each round rotates n/2 disjoint (p, q) pairs at once
// (Golub & Van Loan, Algorithm 8.4.2 "sym.schur2" for each rotation), so that
// every pair is met once per sweep; sweeps stop when the off-diagonal norm is
// below 1e-14 of the Frobenius norm (at most 40 sweeps; a matrix that does
// not get there sets the status word to TT_ERR_UNSUPPORTED).  Eigenvalues are
// returned in ascending order, as eigh returns them.
#include <math.h>

#include <string>

#include "../../include/torchtree_gb300.h"
#include "tt_gamma.cuh"
#include "tt_launch.h"

namespace tt {

namespace {

constexpr int kEigMax = 64;      // largest state count
constexpr int kEigLd = kEigMax + 1;
constexpr int kEigThreads = 256;

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

__global__ void __launch_bounds__(kEigThreads) reversible_eigen_kernel(const double *q, const double *pi, int n,
                                                                       double *lam, double *U, double *W,
                                                                       int *status) {
  extern __shared__ __align__(16) double esm[];
  double *A = esm;                     // [n][kEigLd]
  double *V = A + kEigMax * kEigLd;    // [n][kEigLd]
  double *cs = V + kEigMax * kEigLd;   // [kEigMax/2][2] rotation (c, s) per pair
  double *red = cs + kEigMax;          // [kEigThreads/32] reduction
  double *sq = red + kEigThreads / 32; // [n] sqrt(pi)
  __shared__ int flag;
  const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const double *qb = q + size_t(b) * n * n;
  for (int i = tid; i < n; i += kEigThreads) sq[i] = sqrt(pi[size_t(b) * n + i]);
  __syncthreads();
  // A = Pi^1/2 Q Pi^-1/2 from the lower triangle (mirrored), V = I
  for (int e = tid; e < n * n; e += kEigThreads) {
    const int i = e / n, j = e - i * n;
    const int r = i >= j ? i : j, c = i >= j ? j : i;
    A[i * kEigLd + j] = sq[r] * qb[r * n + c] / sq[c];
    V[i * kEigLd + j] = i == j ? 1.0 : 0.0;
  }
  __syncthreads();
  const int m = n + (n & 1);  // an odd n gets a dummy player that never rotates
  const int npairs = m / 2;
  int sweep = 0;
  for (; sweep < 40; ++sweep) {
    // convergence: off-diagonal norm against the Frobenius norm
    double off = 0.0, tot = 0.0;
    for (int e = tid; e < n * n; e += kEigThreads) {
      const int i = e / n, j = e - i * n;
      const double v = A[i * kEigLd + j];
      tot += v * v;
      if (i != j) off += v * v;
    }
    for (int o = 16; o; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      tot += __shfl_xor_sync(0xffffffffu, tot, o);
    }
    if (lane == 0) red[warp] = off;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int w = 0; w < kEigThreads / 32; ++w) s += red[w];
      off = s;
    }
    __syncthreads();
    if (lane == 0) red[warp] = tot;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int w = 0; w < kEigThreads / 32; ++w) s += red[w];
      flag = !(off > 1e-28 * s) || n == 1;
    }
    __syncthreads();
    if (flag) break;
    for (int r = 0; r < m - 1; ++r) {
      // rotations of this round's pairs
      if (tid < npairs) {
        int p, qq;
        rr_pair(r, tid, m, p, qq);
        double c = 1.0, s = 0.0;
        if (qq < n) {
          const double apq = A[p * kEigLd + qq];
          if (apq != 0.0) {
            const double tau = (A[qq * kEigLd + qq] - A[p * kEigLd + p]) / (2.0 * apq);
            double t;
            if (fabs(tau) > 1e150) t = 0.5 / tau;
            else t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
            c = 1.0 / sqrt(1.0 + t * t);
            s = t * c;
          }
        }
        cs[2 * tid] = c;
        cs[2 * tid + 1] = s;
      }
      __syncthreads();
      // rows: A <- J^T A  (rows p, q of every pair)
      for (int e = tid; e < npairs * n; e += kEigThreads) {
        const int i = e / n, j = e - i * n;
        int p, qq;
        rr_pair(r, i, m, p, qq);
        if (qq >= n) continue;
        const double c = cs[2 * i], s = cs[2 * i + 1];
        const double ap = A[p * kEigLd + j], aq = A[qq * kEigLd + j];
        A[p * kEigLd + j] = c * ap - s * aq;
        A[qq * kEigLd + j] = s * ap + c * aq;
      }
      __syncthreads();
      // columns: A <- A J, V <- V J
      for (int e = tid; e < npairs * n; e += kEigThreads) {
        const int i = e / n, row = e - i * n;
        int p, qq;
        rr_pair(r, i, m, p, qq);
        if (qq >= n) continue;
        const double c = cs[2 * i], s = cs[2 * i + 1];
        const double ap = A[row * kEigLd + p], aq = A[row * kEigLd + qq];
        A[row * kEigLd + p] = c * ap - s * aq;
        A[row * kEigLd + qq] = s * ap + c * aq;
        const double vp = V[row * kEigLd + p], vq = V[row * kEigLd + qq];
        V[row * kEigLd + p] = c * vp - s * vq;
        V[row * kEigLd + qq] = s * vp + c * vq;
      }
      __syncthreads();
    }
  }
  if (tid == 0 && sweep == 40) atomicExch(status, TT_ERR_UNSUPPORTED);
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
  const size_t smem = (2 * size_t(tt::kEigMax) * tt::kEigLd + tt::kEigMax + tt::kEigThreads / 32 + tt::kEigMax) *
                      sizeof(double);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaFuncSetAttribute(tt::reversible_eigen_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(smem));
  if (e == cudaSuccess) {
    tt::reversible_eigen_kernel<<<batch, tt::kEigThreads, smem, s>>>(q, frequencies, state_count, eigenvalues, u, w,
                                                                      status);
    e = cudaGetLastError();
  }
  return e == cudaSuccess ? TT_OK : tt::efail(TT_ERR_CUDA, std::string("eigen launch: ") + cudaGetErrorString(e));
}

int tt_gamma_quantiles(int32_t batch, int32_t category_count, const double *shape, double *x, double *dx_dshape,
                       void *stream) {
  if (!shape || !x || !dx_dshape) return tt::efail(TT_ERR_INVALID_ARGUMENT, "NULL argument");
  if (batch < 1 || category_count < 1) return tt::efail(TT_ERR_INVALID_ARGUMENT, "batch and categories must be >= 1");
  const int n = batch * category_count;
  tt::gamma_quantiles_kernel<<<(n + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(
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
