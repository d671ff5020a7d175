// Transition matrices of non-reversible rate matrices on the device, FP64:
// P = exp(Q t r) for every (sample, branch, category) in one launch, and
// the adjoint that turns dlnL/dP into dlnL/dQ and dlnL/d(t r).
//
// Replaces NonSymmetricSubstitutionModel.p_t
// (torchtree/evolution/substitution_model/abstract.py:86-94, torch.matrix_exp
// of the normalised Q times each branch length and rate; the models are the
// general non-reversible ones of general.py:203-300) and autograd through it.
//
// The exponential is the scaling-and-squaring method with the [13/13] Pade
// approximant of Higham (SIAM J. Matrix Anal. Appl. 26(4), 2005): with
// s = max(0, ceil(log2(||A||_1 / theta_13))), theta_13 = 5.371920351148152
// (Higham's Table 2.3), A is scaled by 2^-s,
//   U = A [A6 (b13 A6 + b11 A4 + b9 A2) + b7 A6 + b5 A4 + b3 A2 + b1 I],
//   V =    A6 (b12 A6 + b10 A4 + b8 A2) + b6 A6 + b4 A4 + b2 A2 + b0 I,
// (V - U) R = (V + U) is solved by Gaussian elimination with partial
// pivoting, and R is squared s times.  The Pade coefficients are
// b_j = (2m-j)! m! / ((2m)! j! (m-j)!), m = 13, built by their recurrence.
//
// The adjoint uses the Frechet derivative L(A, E) of the exponential:
// d tr(G^T exp(A)) = tr(L(A^T, G)^T dA), and L(A^T, G) is the upper-right
// block of exp([[A^T, G], [0, A^T]]) (Mathias 1996; Higham, "Functions of
// Matrices", 2008, section 3.2), computed by the same routine on a matrix of
// twice the size.  With A = Q tau: dlnL/dQ = tau L(tau Q^T, G) and
// dlnL/dtau = tr(G^T Q P).
//
// One CTA per matrix; the matrices live in shared memory (six n x (n+1)
// FP64 buffers), so n = S <= 64 for the exponential and n = 2S <= 64 (S <= 32)
// for the adjoint.
#include <math.h>

#include <string>

#include "../../include/torchtree_gb300.h"
#include "tt_launch.h"

namespace tt {

namespace {

constexpr int kExpmThreads = 128;
constexpr int kExpmMax = 64;

__host__ __device__ constexpr size_t expm_smem_bytes(int n) {
  return size_t(6) * n * (n + 1) * sizeof(double) + size_t(n) * sizeof(int) + 64;
}

// C = A B (n x n, leading dimension ld), all in shared memory; C distinct
// from A and B
__device__ void mm(double *C, const double *A, const double *B, int n, int ld) {
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e - i * n;
    double acc = 0.0;
    for (int k = 0; k < n; ++k) acc = fma(A[i * ld + k], B[k * ld + j], acc);
    C[i * ld + j] = acc;
  }
  __syncthreads();
}

// exp(M) for the n x n matrix in buffer 0 of `w` (six n x ld buffers); the
// result is left in buffer `*out` (an index into the six buffers)
__device__ void expm_smem(double *w, int n, int *piv, int &out) {
  const int ld = n + 1, sz = n * ld;
  double *A = w, *A2 = w + sz, *A4 = w + 2 * sz, *A6 = w + 3 * sz, *Ub = w + 4 * sz, *Vb = w + 5 * sz;
  __shared__ double s_norm;
  __shared__ int s_scale;
  // 1-norm (largest absolute column sum) and the scaling
  if (threadIdx.x == 0) {
    double nrm = 0.0;
    for (int j = 0; j < n; ++j) {
      double c = 0.0;
      for (int i = 0; i < n; ++i) c += fabs(A[i * ld + j]);
      nrm = fmax(nrm, c);
    }
    s_norm = nrm;
    int s = 0;
    if (nrm > 5.371920351148152) s = int(ceil(log2(nrm / 5.371920351148152)));
    s_scale = s > 0 ? s : 0;
  }
  __syncthreads();
  const int s = s_scale;
  if (s > 0) {
    const double f = ldexp(1.0, -s);
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) A[(e / n) * ld + e % n] *= f;
    __syncthreads();
  }
  // Pade [13/13] coefficients
  double b[14];
  b[0] = 1.0;
  for (int j = 0; j < 13; ++j) b[j + 1] = b[j] * double(13 - j) / (double(j + 1) * double(26 - j));
  mm(A2, A, A, n, ld);
  mm(A4, A2, A2, n, ld);
  mm(A6, A4, A2, n, ld);
  // Ub = b13 A6 + b11 A4 + b9 A2
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int x = (e / n) * ld + e % n;
    Ub[x] = b[13] * A6[x] + b[11] * A4[x] + b[9] * A2[x];
  }
  __syncthreads();
  mm(Vb, A6, Ub, n, ld);  // Vb = A6 Ub
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e - i * n, x = i * ld + j;
    Vb[x] += b[7] * A6[x] + b[5] * A4[x] + b[3] * A2[x] + (i == j ? b[1] : 0.0);
  }
  __syncthreads();
  mm(Ub, A, Vb, n, ld);  // U = A (...)
  // Vb = b12 A6 + b10 A4 + b8 A2, then V = A6 Vb (into A, no longer needed)
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int x = (e / n) * ld + e % n;
    Vb[x] = b[12] * A6[x] + b[10] * A4[x] + b[8] * A2[x];
  }
  __syncthreads();
  mm(A, A6, Vb, n, ld);
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e - i * n, x = i * ld + j;
    const double v = A[x] + b[6] * A6[x] + b[4] * A4[x] + b[2] * A2[x] + (i == j ? b[0] : 0.0);
    A2[x] = v - Ub[x];  // M = V - U
    A4[x] = v + Ub[x];  // R = V + U
  }
  __syncthreads();
  // Gaussian elimination with partial pivoting on M, applied to R
  __shared__ int s_p;
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x == 0) {
      int p = k;
      double best = fabs(A2[k * ld + k]);
      for (int i = k + 1; i < n; ++i)
        if (fabs(A2[i * ld + k]) > best) {
          best = fabs(A2[i * ld + k]);
          p = i;
        }
      s_p = p;
      piv[k] = p;
    }
    __syncthreads();
    const int p = s_p;
    if (p != k)
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double t1 = A2[k * ld + j];
        A2[k * ld + j] = A2[p * ld + j];
        A2[p * ld + j] = t1;
        const double t2 = A4[k * ld + j];
        A4[k * ld + j] = A4[p * ld + j];
        A4[p * ld + j] = t2;
      }
    __syncthreads();
    const double inv = 1.0 / A2[k * ld + k];
    // rows below k: subtract l_ik times row k (in M's trailing columns and in R)
    const int rows = n - k - 1;
    for (int e = threadIdx.x; e < rows * (2 * n); e += blockDim.x) {
      const int i = k + 1 + e / (2 * n), c = e % (2 * n);
      const double l = A2[i * ld + k] * inv;
      if (c < n) {
        if (c > k) A2[i * ld + c] -= l * A2[k * ld + c];
      } else {
        A4[i * ld + (c - n)] -= l * A4[k * ld + (c - n)];
      }
    }
    __syncthreads();
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) A2[i * ld + k] = 0.0;
    __syncthreads();
  }
  // back substitution, one thread per right-hand-side column
  for (int j = threadIdx.x; j < n; j += blockDim.x)
    for (int i = n - 1; i >= 0; --i) {
      double acc = A4[i * ld + j];
      for (int c = i + 1; c < n; ++c) acc -= A2[i * ld + c] * A4[c * ld + j];
      A4[i * ld + j] = acc / A2[i * ld + i];
    }
  __syncthreads();
  // squaring: ping-pong between A4 and A6
  double *cur = A4, *nxt = A6;
  for (int r = 0; r < s; ++r) {
    mm(nxt, cur, cur, n, ld);
    double *t = cur;
    cur = nxt;
    nxt = t;
  }
  out = int((cur - w) / sz);
}

// grid (B*K, b): P[b][br][k] = exp(Q_b * bl[b][br] * rate[b][k])
__global__ void __launch_bounds__(kExpmThreads) expm_pmatrix_kernel(const double *q, const double *bl,
                                                                    const double *rates, int S, int B, int K,
                                                                    double *P) {
  extern __shared__ __align__(16) double xsm[];
  const int n = S, ld = n + 1, sz = n * ld;
  int *piv = reinterpret_cast<int *>(xsm + 6 * sz);
  const int bk = blockIdx.x, b = blockIdx.y, br = bk / K, k = bk - br * K;
  const double tau = bl[size_t(b) * B + br] * rates[size_t(b) * K + k];
  const double *qb = q + size_t(b) * S * S;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) xsm[(e / n) * ld + e % n] = qb[e] * tau;
  __syncthreads();
  int out = 0;
  expm_smem(xsm, n, piv, out);
  const double *R = xsm + out * sz;
  double *dst = P + ((size_t(b) * B + br) * K + k) * S * S;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) dst[e] = R[(e / n) * ld + e % n];
}

// grid (B*K, b): the Frechet adjoint of P = exp(Q tau) for G = dlnL/dP:
// dq_part[b][br][k] = tau L(tau Q^T, G) and dtau[b][br][k] = tr(G^T Q P)
__global__ void __launch_bounds__(kExpmThreads) expm_adjoint_kernel(const double *q, const double *bl,
                                                                    const double *rates, const double *G, int S,
                                                                    int B, int K, double *dq_part,
                                                                    double *dtau) {
  extern __shared__ __align__(16) double xsm[];
  const int n = 2 * S, ld = n + 1, sz = n * ld;
  int *piv = reinterpret_cast<int *>(xsm + 6 * sz);
  const int bk = blockIdx.x, b = blockIdx.y, br = bk / K, k = bk - br * K;
  const double tau = bl[size_t(b) * B + br] * rates[size_t(b) * K + k];
  const double *qb = q + size_t(b) * S * S;
  const size_t mat = ((size_t(b) * B + br) * K + k) * S * S;
  const double *g = G + mat;
  // [[tau Q^T, G], [0, tau Q^T]]
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e - i * n;
    double v = 0.0;
    if (i < S && j < S) v = qb[j * S + i] * tau;
    else if (i < S && j >= S) v = g[i * S + (j - S)];
    else if (i >= S && j >= S) v = qb[(j - S) * S + (i - S)] * tau;
    xsm[i * ld + j] = v;
  }
  __syncthreads();
  int out = 0;
  expm_smem(xsm, n, piv, out);
  const double *R = xsm + out * sz;
  // upper-right block: L(tau Q^T, G); upper-left block: exp(tau Q^T) = P^T
  for (int e = threadIdx.x; e < S * S; e += blockDim.x) {
    const int i = e / S, j = e - i * S;
    dq_part[mat + e] = tau * R[i * ld + S + j];
  }
  // dtau = sum_ij G_ij (Q P)_ij, (Q P)_ij = sum_c Q_ic P_cj = sum_c Q_ic R[j][c]
  __shared__ double red[kExpmThreads / 32];
  double acc = 0.0;
  for (int e = threadIdx.x; e < S * S; e += blockDim.x) {
    const int i = e / S, j = e - i * S;
    double qp = 0.0;
    for (int c = 0; c < S; ++c) qp = fma(qb[i * S + c], R[j * ld + c], qp);
    acc = fma(g[e], qp, acc);
  }
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kExpmThreads / 32; ++w) t += red[w];
    dtau[(size_t(b) * B + br) * K + k] = t;
  }
}

int xfail(int code, const std::string &msg) { return record_error(code, msg.c_str()); }

}  // namespace

}  // namespace tt

extern "C" {

int tt_transition_matrices_expm(int32_t batch, int32_t state_count, int32_t branch_count, int32_t category_count,
                                const double *q, const double *branch_lengths, const double *category_rates,
                                double *matrices, void *stream) {
  if (!q || !branch_lengths || !category_rates || !matrices) return tt::xfail(TT_ERR_INVALID_ARGUMENT, "NULL argument");
  if (batch < 1 || branch_count < 1 || category_count < 1 || state_count < 1 || state_count > tt::kExpmMax)
    return tt::xfail(TT_ERR_INVALID_ARGUMENT, "tt_transition_matrices_expm: sizes >= 1 and state_count <= 64");
  if (size_t(branch_count) * category_count > 0x7fffffffu || batch > 65535)
    return tt::xfail(TT_ERR_INVALID_ARGUMENT, "too many matrices for one launch");
  const size_t smem = tt::expm_smem_bytes(state_count);
  cudaError_t e = tt::kernel_smem(tt::expm_pmatrix_kernel, smem);
  if (e == cudaSuccess) {
    tt::expm_pmatrix_kernel<<<dim3(branch_count * category_count, batch), tt::kExpmThreads, smem,
                              static_cast<cudaStream_t>(stream)>>>(q, branch_lengths, category_rates, state_count,
                                                                   branch_count, category_count, matrices);
    e = cudaGetLastError();
  }
  return e == cudaSuccess ? TT_OK : tt::xfail(TT_ERR_CUDA, std::string("expm launch: ") + cudaGetErrorString(e));
}

int tt_transition_matrices_expm_adjoint(int32_t batch, int32_t state_count, int32_t branch_count,
                                        int32_t category_count, const double *q, const double *branch_lengths,
                                        const double *category_rates, const double *grad_matrices,
                                        double *grad_q_parts, double *grad_times, void *stream) {
  if (!q || !branch_lengths || !category_rates || !grad_matrices || !grad_q_parts || !grad_times)
    return tt::xfail(TT_ERR_INVALID_ARGUMENT, "NULL argument");
  if (batch < 1 || branch_count < 1 || category_count < 1 || state_count < 1 || 2 * state_count > tt::kExpmMax)
    return tt::xfail(TT_ERR_INVALID_ARGUMENT, "tt_transition_matrices_expm_adjoint: sizes >= 1 and state_count <= 32");
  if (size_t(branch_count) * category_count > 0x7fffffffu || batch > 65535)
    return tt::xfail(TT_ERR_INVALID_ARGUMENT, "too many matrices for one launch");
  const size_t smem = tt::expm_smem_bytes(2 * state_count);
  cudaError_t e = tt::kernel_smem(tt::expm_adjoint_kernel, smem);
  if (e == cudaSuccess) {
    tt::expm_adjoint_kernel<<<dim3(branch_count * category_count, batch), tt::kExpmThreads, smem,
                              static_cast<cudaStream_t>(stream)>>>(q, branch_lengths, category_rates, grad_matrices,
                                                                   state_count, branch_count, category_count,
                                                                   grad_q_parts, grad_times);
    e = cudaGetLastError();
  }
  return e == cudaSuccess ? TT_OK
                          : tt::xfail(TT_ERR_CUDA, std::string("expm adjoint launch: ") + cudaGetErrorString(e));
}

}  // extern "C"
