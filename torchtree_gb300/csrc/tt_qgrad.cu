// dlnL/dQ: the plan's dlnL/dP chained through P = exp(Q t r) in the eigenbasis
// of Q = U diag(lambda) W (the Frechet derivative of the matrix exponential):
//
//   M = U^T G W^T,   X = sum_(branch, k) F(t r) .* M,   dlnL/dQ = W^T X U^T,
//   F_mn = (e^(lambda_m tau) - e^(lambda_n tau)) / (lambda_m - lambda_n)
//        = tau e^(max) phi(-|lambda_m - lambda_n| tau),  phi(z) = expm1(z) / z,
//   dlnL/dtau = sum_m lambda_m e^(lambda_m tau) M_mm  (-> branch lengths, rates).
//
// Unlike the chain through dU, dW (tt_pmatrix.cuh, tt_wide.cuh) nothing here
// differentiates eigenvectors, so the result is well conditioned at any
// working precision: FP32 plans of the wide path run these products in FP32.
#include <string>

#include "../../include/torchtree_gb300.h"
#include "tt_plan.h"
#include "tt_wide.cuh"

namespace tt {

namespace {

template <typename T>
__device__ __forceinline__ T exp_t(T x);
template <>
__device__ __forceinline__ double exp_t(double x) { return exp(x); }
template <>
__device__ __forceinline__ float exp_t(float x) { return expf(x); }

template <typename T>
__device__ __forceinline__ T frechet(T lm, T ln, T tau) {
  const T a = lm * tau, c = ln * tau;
  const T d = a > c ? c - a : a - c;  // -|a - c|
  T phi = T(1);
  if (d != T(0)) {
    if constexpr (sizeof(T) == 8) phi = expm1(d) / d;
    else phi = expm1f(d) / d;
  }
  return tau * exp_t(a > c ? a : c) * phi;
}

// The same divided difference from the states' exponentials em = exp(am),
// en = exp(an) (am = lambda_m tau, an = lambda_n tau), FP32: far apart,
// tau (em - en) / (am - an) has no cancellation; within 0.5, the Taylor
// series of expm1(x) / x to x^7 (remainder below 1.1e-8 for |x| <= 0.5).
__device__ __forceinline__ float frechet_e(float am, float an, float em, float en, float tau) {
  const float d = am - an;
  if (fabsf(d) > 0.5f) return tau * (em - en) / d;
  const float x = -fabsf(d);
  float phi = 1.0f / 40320.0f;
  phi = fmaf(phi, x, 1.0f / 5040.0f);
  phi = fmaf(phi, x, 1.0f / 720.0f);
  phi = fmaf(phi, x, 1.0f / 120.0f);
  phi = fmaf(phi, x, 1.0f / 24.0f);
  phi = fmaf(phi, x, 1.0f / 6.0f);
  phi = fmaf(phi, x, 0.5f);
  phi = fmaf(phi, x, 1.0f);
  return tau * fmaxf(em, en) * phi;
}

}  // namespace

// 4 states: one CTA per (chunk of 128 branches, sample), one branch per
// thread, products in T (the plan's precision: FP64 arithmetic is scarce on
// this GPU), sums over a thread's branches in T and across the CTA in FP64;
// X and the rate sums reduced in a fixed order through shared memory.
template <typename T>
__global__ void __launch_bounds__(128) qgrad_small_kernel(const double *G, const double *lam, const double *U,
                                                          const double *W, const double *bl, const double *rates,
                                                          int B, int K, double *part, double *dbl) {
  constexpr int S = 4;
  __shared__ double red[128][S * S + 8];
  const int chunk = blockIdx.x, b = blockIdx.y, tid = threadIdx.x;
  T u[S][S], w[S][S], l[S];
#pragma unroll
  for (int i = 0; i < S; ++i) {
    l[i] = T(lam[b * S + i]);
#pragma unroll
    for (int j = 0; j < S; ++j) {
      u[i][j] = T(U[(size_t(b) * S + i) * S + j]);
      w[i][j] = T(W[(size_t(b) * S + i) * S + j]);
    }
  }
  T X[S][S];
  double dr[8];
#pragma unroll
  for (int i = 0; i < S; ++i)
#pragma unroll
    for (int j = 0; j < S; ++j) X[i][j] = T(0);
#pragma unroll
  for (int k = 0; k < 8; ++k) dr[k] = 0.0;
  for (int br = chunk * 128 + tid; br < min(B, chunk * 128 + 128); br += 128) {
    const double t = bl[size_t(b) * B + br];
    double dt = 0.0;
    for (int k = 0; k < K; ++k) {
      const T tau = T(t * rates[b * K + k]);
      const double *g = G + ((size_t(b) * B + br) * K + k) * S * S;
      T h[S][S], M[S][S];
#pragma unroll
      for (int i = 0; i < S; ++i)
#pragma unroll
        for (int n = 0; n < S; ++n) {
          T acc = T(0);
#pragma unroll
          for (int j = 0; j < S; ++j) acc = fma(T(g[i * S + j]), w[n][j], acc);
          h[i][n] = acc;
        }
#pragma unroll
      for (int m = 0; m < S; ++m)
#pragma unroll
        for (int n = 0; n < S; ++n) {
          T acc = T(0);
#pragma unroll
          for (int i = 0; i < S; ++i) acc = fma(u[i][m], h[i][n], acc);
          M[m][n] = acc;
        }
      T sk = T(0);
      if constexpr (sizeof(T) == 4) {  // the states' exponentials once, the divided differences from them
        T lt[S], es[S];
#pragma unroll
        for (int m = 0; m < S; ++m) {
          lt[m] = l[m] * tau;
          es[m] = exp_t(lt[m]);
        }
#pragma unroll
        for (int m = 0; m < S; ++m) {
          sk = fma(l[m] * es[m], M[m][m], sk);
#pragma unroll
          for (int n = 0; n < S; ++n) X[m][n] = fma(frechet_e(lt[m], lt[n], es[m], es[n], tau), M[m][n], X[m][n]);
        }
      } else {
#pragma unroll
        for (int m = 0; m < S; ++m) {
          sk = fma(l[m] * exp_t(l[m] * tau), M[m][m], sk);
#pragma unroll
          for (int n = 0; n < S; ++n) X[m][n] = fma(frechet(l[m], l[n], tau), M[m][n], X[m][n]);
        }
      }
      const double s = double(sk);
      dt = fma(s, rates[b * K + k], dt);
      if (k < 8) dr[k] = fma(s, t, dr[k]);
    }
    if (dbl) dbl[size_t(b) * B + br] = dt;
  }
#pragma unroll
  for (int i = 0; i < S; ++i)
#pragma unroll
    for (int j = 0; j < S; ++j) red[tid][i * S + j] = double(X[i][j]);
#pragma unroll
  for (int k = 0; k < 8; ++k) red[tid][S * S + k] = dr[k];
  __syncthreads();
  for (int e = tid; e < S * S + K; e += 128) {
    double acc = 0.0;
    for (int r = 0; r < 128; ++r) acc += red[r][e];
    part[(size_t(b) * gridDim.x + chunk) * (S * S + K) + e] = acc;
  }
}

// 20 / 61 states: one CTA per (chunk of branches, sample); per (branch, k)
// H = G W^T and M = U^T H as 4 x 4 register tiles (rows ib + IB x), then
// X += F .* M in the thread's tile.  Chunk partials [S*S + K] in FP64.
template <typename T, int SP>
__global__ void __launch_bounds__(256) wide_qgrad_kernel(const double *G, const double *lam, const double *U,
                                                         const double *W, const double *bl, const double *rates,
                                                         int S, int B, int K, int bchunk, double *dbl, double *part) {
  constexpr int IB = SP / 4;
  constexpr int NB = (IB * IB + 255) / 256;
  extern __shared__ __align__(128) unsigned char smem[];
  T *ug = reinterpret_cast<T *>(smem);  // [i][perm m] = U[i][m]
  T *wt = ug + SP * SP;                  // [j][perm n] = W[n][j]
  T *gt = wt + SP * SP;                  // [j][perm i] = G[i][j]
  T *hs = gt + SP * SP;                  // [i][perm n] = H[i][n]
  T *ls = hs + SP * SP;                  // lambda [SP]
  T *lt = ls + SP;                       // lambda tau [SP] (FP32 plans)
  T *es = lt + SP;                       // exp(lambda tau) [SP] (FP32 plans)
  double *dred = reinterpret_cast<double *>(es + SP);  // [IB] diagonal sums
  const int chunk = blockIdx.x, b = blockIdx.y, tid = threadIdx.x;
  for (int e = tid; e < SP * SP; e += 256) {
    const int x = e / SP, y = e - x * SP;
    const bool in = x < S && y < S;
    ug[x * SP + wperm<IB>(y)] = in ? T(U[(size_t(b) * S + x) * S + y]) : T(0);
    wt[y * SP + wperm<IB>(x)] = in ? T(W[(size_t(b) * S + x) * S + y]) : T(0);
  }
  for (int m = tid; m < SP; m += 256) ls[m] = m < S ? T(lam[size_t(b) * S + m]) : T(0);
  T X[NB][4][4];
#pragma unroll
  for (int nb = 0; nb < NB; ++nb)
#pragma unroll
    for (int x = 0; x < 4; ++x)
#pragma unroll
      for (int y = 0; y < 4; ++y) X[nb][x][y] = T(0);
  double drs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  const int br0 = chunk * bchunk, br1 = min(B, br0 + bchunk);
  for (int br = br0; br < br1; ++br) {
    const double t = bl[size_t(b) * B + br];
    double dt = 0.0;
    for (int k = 0; k < K; ++k) {
      const T tau = T(t * rates[size_t(b) * K + k]);
      __syncthreads();  // previous products done with gt / hs / es
      if constexpr (sizeof(T) == 4)
        for (int m = tid; m < SP; m += 256) {
          lt[m] = ls[m] * tau;
          es[m] = m < S ? exp_t(ls[m] * tau) : T(0);
        }
      const double *g = G + ((size_t(b) * B + br) * K + k) * S * S;
      for (int e = tid; e < SP * SP; e += 256) {
        const int i = e / SP, j = e - i * SP;
        gt[j * SP + wperm<IB>(i)] = (i < S && j < S) ? T(g[i * S + j]) : T(0);
      }
      __syncthreads();
#pragma unroll
      for (int nb = 0; nb < NB; ++nb) {  // H block: rows i = bi + IB x, cols n = bn + IB y
        const int blk = tid + nb * 256;
        if (blk < IB * IB) {
          const int bi = blk / IB, bn = blk - bi * IB;
          T h[4][4];
#pragma unroll
          for (int x = 0; x < 4; ++x)
#pragma unroll
            for (int y = 0; y < 4; ++y) h[x][y] = T(0);
          for (int j = 0; j < SP; ++j) {
            T ga[4], wa[4];
            V4<T>::ld(gt + j * SP + bi * 4, ga);
            V4<T>::ld(wt + j * SP + bn * 4, wa);
            outer4(h, ga, wa);
          }
#pragma unroll
          for (int x = 0; x < 4; ++x) V4<T>::st(hs + (bi + IB * x) * SP + bn * 4, h[x]);
        }
      }
      __syncthreads();
      double dsum = 0.0;
#pragma unroll
      for (int nb = 0; nb < NB; ++nb) {  // M block: rows m = bm + IB x, cols n = bn + IB y
        const int blk = tid + nb * 256;
        if (blk < IB * IB) {
          const int bm = blk / IB, bn = blk - bm * IB;
          T M[4][4];
#pragma unroll
          for (int x = 0; x < 4; ++x)
#pragma unroll
            for (int y = 0; y < 4; ++y) M[x][y] = T(0);
          for (int i = 0; i < SP; ++i) {
            T ua[4], ha[4];
            V4<T>::ld(ug + i * SP + bm * 4, ua);
            V4<T>::ld(hs + i * SP + bn * 4, ha);
            outer4(M, ua, ha);
          }
#pragma unroll
          for (int x = 0; x < 4; ++x) {
            const int m = bm + IB * x;
#pragma unroll
            for (int y = 0; y < 4; ++y) {
              const int n = bn + IB * y;
              if constexpr (sizeof(T) == 4)
                X[nb][x][y] += frechet_e(lt[m], lt[n], es[m], es[n], tau) * M[x][y];
              else
                X[nb][x][y] += frechet(ls[m], ls[n], tau) * M[x][y];
            }
          }
          if (bm == bn)
#pragma unroll
            for (int x = 0; x < 4; ++x) {
              const int m = bm + IB * x;
              // in the plan's type (an FP64 exp costs thousands of cycles of this GPU's FP64 pipe)
              if constexpr (sizeof(T) == 4) {
                if (m < S) dsum += double(ls[m] * es[m] * M[x][x]);
              } else {
                if (m < S) dsum += double(ls[m] * exp_t(ls[m] * tau) * M[x][x]);
              }
            }
        }
      }
      // the IB diagonal blocks' sums, fixed order
      if (tid < IB * IB && (tid / IB) == (tid - (tid / IB) * IB)) dred[tid / IB] = dsum;
      __syncthreads();
      if (tid == 0) {
        double s = 0.0;
        for (int x = 0; x < IB; ++x) s += dred[x];
        dt += s * rates[size_t(b) * K + k];
        if (k < 8) drs[k] += s * t;
      }
    }
    if (tid == 0 && dbl) dbl[size_t(b) * B + br] = dt;
  }
  const int width = S * S + K;
  double *dst = part + (size_t(b) * gridDim.x + chunk) * width;
#pragma unroll
  for (int nb = 0; nb < NB; ++nb) {
    const int blk = tid + nb * 256;
    if (blk < IB * IB) {
      const int bm = blk / IB, bn = blk - bm * IB;
#pragma unroll
      for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y) {
          const int m = bm + IB * x, n = bn + IB * y;
          if (m < S && n < S) dst[m * S + n] = double(X[nb][x][y]);
        }
    }
  }
  if (tid == 0)
    for (int k = 0; k < K; ++k) dst[S * S + k] = drs[k];
}

// per sample, kQRows rows per CTA (grid: row blocks x samples), FP64:
// X rows = sums of the chunk partials, then Z rows = X rows U^T; the first
// row block also sums the rate terms.  Spreading the rows over CTAs keeps the
// FP64 work off a single SM per sample.
constexpr int kQRows = 4;

__global__ void __launch_bounds__(256) qgrad_sum_rows_kernel(const double *part, int nchunks, const double *U, int S,
                                                             int K, double *Z, double *drates) {
  __shared__ double X[kQRows][64];
  const int b = blockIdx.y, r0 = blockIdx.x * kQRows, tid = threadIdx.x, width = S * S + K;
  const int rows = min(kQRows, S - r0);
  for (int e = tid; e < rows * S; e += blockDim.x) {
    const int r = e / S, c = e - r * S;
    double s = 0.0;
    for (int ch = 0; ch < nchunks; ++ch) s += part[(size_t(b) * nchunks + ch) * width + (r0 + r) * S + c];
    X[r][c] = s;
  }
  if (blockIdx.x == 0 && drates)
    for (int k = tid; k < K; k += blockDim.x) {
      double s = 0.0;
      for (int ch = 0; ch < nchunks; ++ch) s += part[(size_t(b) * nchunks + ch) * width + S * S + k];
      drates[size_t(b) * K + k] = s;
    }
  __syncthreads();
  const double *u = U + size_t(b) * S * S;
  for (int e = tid; e < rows * S; e += blockDim.x) {  // Z[m][j] = sum_n X[m][n] U[j][n]
    const int r = e / S, j = e - r * S;
    double acc = 0.0;
    for (int n = 0; n < S; ++n) acc = fma(X[r][n], u[j * S + n], acc);
    Z[(size_t(b) * S + r0 + r) * S + j] = acc;
  }
}

// dQ rows i = sum_m W[m][i] Z[m][j], kQRows rows per CTA, FP64.
__global__ void __launch_bounds__(256) qgrad_dq_rows_kernel(const double *Z, const double *W, int S, double *dQ) {
  const int b = blockIdx.y, r0 = blockIdx.x * kQRows, tid = threadIdx.x;
  const int rows = min(kQRows, S - r0);
  const double *w = W + size_t(b) * S * S, *z = Z + size_t(b) * S * S;
  for (int e = tid; e < rows * S; e += blockDim.x) {
    const int i = r0 + e / S, j = e - (e / S) * S;
    double acc = 0.0;
    for (int m = 0; m < S; ++m) acc = fma(w[m * S + i], z[m * S + j], acc);
    dQ[size_t(b) * S * S + size_t(i) * S + j] = acc;
  }
}

namespace {

template <typename T, int SP>
cudaError_t launch_wide_qgrad(tt_plan *p, const double *lam, const double *U, const double *W, const double *bl,
                              const double *rates, double *dbl, double *part, int bchunk, int nchunks,
                              cudaStream_t s) {
  const size_t smem = 4 * SP * SP * sizeof(T) + 3 * SP * sizeof(T) + (SP / 4 + 2) * sizeof(double) + 16;
  cudaError_t e = kernel_smem(wide_qgrad_kernel<T, SP>, smem);
  if (e != cudaSuccess) return e;
  wide_qgrad_kernel<T, SP><<<dim3(nchunks, p->batch), 256, smem, s>>>(p->d_G, lam, U, W, bl, rates, p->S, p->B,
                                                                      p->K, bchunk, dbl, part);
  return cudaGetLastError();
}

}  // namespace

int rate_matrix_gradient(tt_plan *p, const double *lam, const double *U, const double *W, const double *bl,
                         const double *rates, double *dQ, double *dbl, double *drates, cudaStream_t s) {
  const int S = p->S, K = p->K;
  const int width = S * S + K;
  int nchunks = 1;
  cudaError_t e = cudaSuccess;
  if (!p->d_qpart) {  // chunk partials, allocated on first use
    const int bchunk = 8;
    const size_t chunks = S == 4 ? size_t((p->B + 127) / 128) : size_t((p->B + bchunk - 1) / bchunk);
    // the chunk partials, then Z [b][S][S] of the finishing step
    e = cudaMalloc(reinterpret_cast<void **>(&p->d_qpart),
                   (size_t(p->batch) * chunks * width + size_t(p->batch) * S * S) * sizeof(double));
    if (e != cudaSuccess) {
      cudaGetLastError();
      return record_error(TT_ERR_OUT_OF_MEMORY, "cudaMalloc of the rate-matrix gradient chunks failed");
    }
    p->bytes += (size_t(p->batch) * chunks * width + size_t(p->batch) * S * S) * sizeof(double);
    p->qpart_chunks = int(chunks);
  }
  if (S == 4) {
    nchunks = (p->B + 127) / 128;
    if (p->precision == TT_PRECISION_F32)
      qgrad_small_kernel<float><<<dim3(nchunks, p->batch), 128, 0, s>>>(p->d_G, lam, U, W, bl, rates, p->B, K,
                                                                        p->d_qpart, dbl);
    else
      qgrad_small_kernel<double><<<dim3(nchunks, p->batch), 128, 0, s>>>(p->d_G, lam, U, W, bl, rates, p->B, K,
                                                                         p->d_qpart, dbl);
    e = cudaGetLastError();
  } else {
    const int bchunk = 8;
    nchunks = (p->B + bchunk - 1) / bchunk;
    const bool f32 = p->precision == TT_PRECISION_F32;
    if (S <= 20)
      e = f32 ? launch_wide_qgrad<float, 20>(p, lam, U, W, bl, rates, dbl, p->d_qpart, bchunk, nchunks, s)
              : launch_wide_qgrad<double, 20>(p, lam, U, W, bl, rates, dbl, p->d_qpart, bchunk, nchunks, s);
    else
      e = f32 ? launch_wide_qgrad<float, 64>(p, lam, U, W, bl, rates, dbl, p->d_qpart, bchunk, nchunks, s)
              : launch_wide_qgrad<double, 64>(p, lam, U, W, bl, rates, dbl, p->d_qpart, bchunk, nchunks, s);
  }
  if (e == cudaSuccess) {
    double *Z = p->d_qpart + size_t(p->batch) * p->qpart_chunks * width;
    const dim3 grid((S + kQRows - 1) / kQRows, p->batch);
    qgrad_sum_rows_kernel<<<grid, 256, 0, s>>>(p->d_qpart, nchunks, U, S, K, Z, drates);
    if (dQ) qgrad_dq_rows_kernel<<<grid, 256, 0, s>>>(Z, W, S, dQ);
    e = cudaGetLastError();
  }
  p->launches += dQ ? 3 : 2;
  if (e != cudaSuccess)
    return record_error(e == cudaErrorMemoryAllocation ? TT_ERR_OUT_OF_MEMORY : TT_ERR_CUDA,
                        (std::string("rate-matrix gradient launch: ") + cudaGetErrorString(e)).c_str());
  return TT_OK;
}

}  // namespace tt
