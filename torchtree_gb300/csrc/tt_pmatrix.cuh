// Transition-matrix kernels.
//
// Forward (replaces torchtree/evolution/substitution_model/abstract.py:67-76):
//   P[b][i][k] = U[b] diag(exp(lambda[b] * t[b][i] * r[b][k])) W[b]
// for every sample, branch and rate category in one launch, in FP64, stored
// at the pruning precision in step order [b][step][side][K][mstride] (each
// S x S matrix padded to mstride elements) so the pruning kernels stage one
// contiguous block per step.
//
// Backward: chains dlnL/dP through the same product to the eigen system,
// the branch lengths and the category rates (what autograd does through
// abstract.py:67-76 in the reference).
#pragma once

#include "tt_common.cuh"

namespace tt {

template <typename T, int S>
__global__ void pmatrix_from_eigen_kernel(const double *__restrict__ lam,
                                          const double *__restrict__ U,
                                          const double *__restrict__ W,
                                          const double *__restrict__ bl,
                                          const double *__restrict__ rates,
                                          const int *__restrict__ branch_pos, T *__restrict__ pmat,
                                          int B, int K, int n_steps, int batch, int mstride) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long total = (long long)batch * B * K;
  if (idx >= total) return;
  const int k = int(idx % K);
  const int br = int((idx / K) % B);
  const int b = int(idx / ((long long)K * B));
  const int pos = branch_pos[br];
  if (pos < 0) return;
  const double t = bl[size_t(b) * B + br] * rates[size_t(b) * K + k];
  const double *Ub = U + size_t(b) * S * S;
  const double *Wb = W + size_t(b) * S * S;
  double e[S];
#pragma unroll
  for (int m = 0; m < S; ++m) e[m] = exp(lam[size_t(b) * S + m] * t);
  T *dst = pmat + ((size_t(b) * n_steps * 2 + pos) * K + k) * mstride;
#pragma unroll
  for (int i = 0; i < S; ++i) {
    double ue[S];
#pragma unroll
    for (int m = 0; m < S; ++m) ue[m] = Ub[i * S + m] * e[m];
    T row[S];
#pragma unroll
    for (int j = 0; j < S; ++j) {
      double acc = 0.0;
#pragma unroll
      for (int m = 0; m < S; ++m) acc = fma(ue[m], Wb[m * S + j], acc);
      row[j] = T(acc);
    }
    store_vec<T, S>(dst + i * S, row);
  }
}

// Matrices given by the caller ([b][B][K][S][S], FP64) -> step order, each
// S x S matrix at a stride of `mstride` elements.
template <typename T>
__global__ void pmatrix_scatter_kernel(const double *__restrict__ src,
                                       const int *__restrict__ branch_pos, T *__restrict__ pmat,
                                       int B, int KSS, int n_steps, int batch, int SS, int mstride) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long total = (long long)batch * B * KSS;
  if (idx >= total) return;
  const int e = int(idx % KSS);
  const int br = int((idx / KSS) % B);
  const int b = int(idx / ((long long)KSS * B));
  const int pos = branch_pos[br];
  if (pos < 0) return;
  pmat[(size_t(b) * n_steps * 2 + pos) * (KSS / SS) * mstride + (e / SS) * mstride + e % SS] = T(src[idx]);
}

// FP32 plans: the same matrices stored as category pairs,
// [b][step][side][KQ][4][4] float2 with (category 2q, category 2q+1); slots of
// padded categories are never written (the buffer is zeroed once).
static __global__ void pmatrix_pairs_from_eigen_kernel(const double *__restrict__ lam, const double *__restrict__ U,
                                                const double *__restrict__ W, const double *__restrict__ bl,
                                                const double *__restrict__ rates,
                                                const int *__restrict__ branch_pos, float *__restrict__ pmat,
                                                int B, int K, int KQ, int n_steps, int batch) {
  constexpr int S = 4;
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long total = (long long)batch * B * K;
  if (idx >= total) return;
  const int k = int(idx % K);
  const int br = int((idx / K) % B);
  const int b = int(idx / ((long long)K * B));
  const int pos = branch_pos[br];
  if (pos < 0) return;
  const double t = bl[size_t(b) * B + br] * rates[size_t(b) * K + k];
  const double *Ub = U + size_t(b) * S * S;
  const double *Wb = W + size_t(b) * S * S;
  double e[S];
#pragma unroll
  for (int m = 0; m < S; ++m) e[m] = exp(lam[size_t(b) * S + m] * t);
  float *dst = pmat + ((size_t(b) * n_steps * 2 + pos) * KQ + (k >> 1)) * 32 + (k & 1);
#pragma unroll
  for (int i = 0; i < S; ++i) {
    double ue[S];
#pragma unroll
    for (int m = 0; m < S; ++m) ue[m] = Ub[i * S + m] * e[m];
#pragma unroll
    for (int j = 0; j < S; ++j) {
      double acc = 0.0;
#pragma unroll
      for (int m = 0; m < S; ++m) acc = fma(ue[m], Wb[m * S + j], acc);
      dst[(i * S + j) * 2] = float(acc);
    }
  }
}

static __global__ void pmatrix_pairs_scatter_kernel(const double *__restrict__ src, const int *__restrict__ branch_pos,
                                             float *__restrict__ pmat, int B, int K, int KQ, int n_steps,
                                             int batch) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long total = (long long)batch * B * K * 16;
  if (idx >= total) return;
  const int e = int(idx % 16);
  const int k = int((idx / 16) % K);
  const int br = int((idx / (16 * K)) % B);
  const int b = int(idx / ((long long)16 * K * B));
  const int pos = branch_pos[br];
  if (pos < 0) return;
  pmat[((size_t(b) * n_steps * 2 + pos) * KQ + (k >> 1)) * 32 + e * 2 + (k & 1)] = float(src[idx]);
}

// Gradient of sum_b lnL[b] through P = U diag(exp(lambda t r)) W.
// One CTA per sample; a thread owns whole branches (all categories), so
// dlnL/dt is written directly and the rest is a fixed-order block sum.
template <int S, int KMAX, int THREADS>
__global__ void __launch_bounds__(THREADS)
    pmatrix_backward_kernel(const double *__restrict__ G, const double *__restrict__ lam,
                            const double *__restrict__ U, const double *__restrict__ W,
                            const double *__restrict__ bl, const double *__restrict__ rates, int B,
                            int K, double *dlam, double *dU, double *dW, double *dbl,
                            double *drates) {
  constexpr int NV = 2 * S * S + S + KMAX;
  __shared__ double part[THREADS / 32][NV];
  const int b = blockIdx.x;
  const int tid = threadIdx.x;
  double u[S][S], w[S][S], l[S], r[KMAX];
#pragma unroll
  for (int i = 0; i < S; ++i) {
    l[i] = lam[size_t(b) * S + i];
#pragma unroll
    for (int j = 0; j < S; ++j) {
      u[i][j] = U[(size_t(b) * S + i) * S + j];
      w[i][j] = W[(size_t(b) * S + i) * S + j];
    }
  }
#pragma unroll
  for (int k = 0; k < KMAX; ++k) r[k] = k < K ? rates[size_t(b) * K + k] : 0.0;
  double acc[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) acc[v] = 0.0;

  for (int br = tid; br < B; br += THREADS) {
    const double t0 = bl[size_t(b) * B + br];
    double dt = 0.0;
#pragma unroll
    for (int k = 0; k < KMAX; ++k) {
      if (k >= K) continue;
      const double t = t0 * r[k];
      const double *g = G + ((size_t(b) * B + br) * K + k) * S * S;
      double gk[S][S];
#pragma unroll
      for (int i = 0; i < S; ++i)
#pragma unroll
        for (int j = 0; j < S; ++j) gk[i][j] = g[i * S + j];
      double e[S], de[S];
#pragma unroll
      for (int m = 0; m < S; ++m) e[m] = exp(l[m] * t);
      // (G W^T)[i][m] and (U^T G)[m][j]
#pragma unroll
      for (int m = 0; m < S; ++m) {
        double dsum = 0.0;
#pragma unroll
        for (int i = 0; i < S; ++i) {
          double gw = 0.0;
#pragma unroll
          for (int j = 0; j < S; ++j) gw = fma(gk[i][j], w[m][j], gw);
          acc[i * S + m] = fma(e[m], gw, acc[i * S + m]);  // dU[i][m]
          dsum = fma(u[i][m], gw, dsum);
        }
        de[m] = dsum;
#pragma unroll
        for (int j = 0; j < S; ++j) {
          double ug = 0.0;
#pragma unroll
          for (int i = 0; i < S; ++i) ug = fma(u[i][m], gk[i][j], ug);
          acc[S * S + m * S + j] = fma(e[m], ug, acc[S * S + m * S + j]);  // dW[m][j]
        }
      }
      double slam = 0.0;
#pragma unroll
      for (int m = 0; m < S; ++m) {
        const double q = de[m] * e[m];
        acc[2 * S * S + m] = fma(q, t, acc[2 * S * S + m]);  // dlambda[m]
        slam = fma(q, l[m], slam);
      }
      dt = fma(slam, r[k], dt);
      acc[2 * S * S + S + k] = fma(slam, t0, acc[2 * S * S + S + k]);  // d rate[k]
    }
    if (dbl) dbl[size_t(b) * B + br] = dt;
  }
  const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const double s = warp_sum(acc[v]);
    if (lane == 0) part[warp][v] = s;
  }
  __syncthreads();
  for (int v = tid; v < NV; v += THREADS) {
    double s = 0.0;
#pragma unroll
    for (int ww = 0; ww < THREADS / 32; ++ww) s += part[ww][v];
    if (v < S * S) {
      if (dU) dU[size_t(b) * S * S + v] = s;
    } else if (v < 2 * S * S) {
      if (dW) dW[size_t(b) * S * S + v - S * S] = s;
    } else if (v < 2 * S * S + S) {
      if (dlam) dlam[size_t(b) * S + v - 2 * S * S] = s;
    } else if (v - 2 * S * S - S < K) {
      if (drates) drates[size_t(b) * K + v - 2 * S * S - S] = s;
    }
  }
}

}  // namespace tt
