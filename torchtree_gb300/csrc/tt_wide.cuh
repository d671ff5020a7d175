// Wide-state pruning kernels: amino-acid (S = 20) and codon (S = 61, padded
// to 64) models, FP32 (rescaled) and FP64.
//
// Level-scheduled: one launch per tree level (forward: by height above the
// tips; adjoint: by depth below the root), each CTA one (node, pattern tile
// or chunk, sample, category).  At these state counts a node's work is
// S x S matrix times S x P pattern tile products, so partials live in HBM
// and every CTA runs register-tiled products out of shared memory:
//
//   forward   L_v[k]   = (P_l[k] x_l[k]) .* (P_r[k] x_r[k])            (GEMM1)
//   adjoint   u_l      = pre_v .* (P_r x_r),  pre_l = P_l^T u_l        (GEMM1, GEMM2)
//             dlnL/dP_l[k][i][j] += sum_p c_p u_l[i][p] x_l[j][p]     (GEMM3)
//
// Rescaling is per (node, category, pattern) by exact powers of two; the
// integer exponents are kept per node (cumulative over the subtree in the
// forward, along the path from the root in the adjoint), so the adjoint's
// per-pattern coefficient is c_p = w_p 2^(E_pre + E_l + E_r - log2 L_p) and
// each category is independent of the others.
//
// Thread tiles: a thread owns 4 rows {ib, ib+IB, ib+2IB, ib+3IB} (IB = SP/4)
// and 4 consecutive patterns.  Staged matrices are stored with those four
// rows adjacent (wperm), so every operand fetch is one 16-byte shared load.
//
// Layouts: matrices [b][branch][K][SP][SP] (zero outside S x S); partials
// [b][internal node][K][SP][Npad] with Npad a multiple of 128; exponents
// [b][internal node][K][Npad].  The adjoint overwrites a node's forward
// partial and exponent with its outside partial and exponent once its
// parent's step has consumed them (each (node, category, tile) region is
// touched by one CTA only).
#pragma once

#include <climits>

#include "tt_common.cuh"

namespace tt {

template <typename T, int SP, int PT>
struct WideCfg {
  static_assert(SP % 4 == 0 && PT % 4 == 0, "tiles are 4 x 4");
  static constexpr int IB = SP / 4;                                 // row blocks
  static constexpr int PB = PT / 4;                                 // pattern blocks
  static constexpr int NT = IB * PB;                                // threads
  static constexpr int XS = PT + 16 / int(sizeof(T));               // padded tile row stride
  static constexpr int NG = NT >= IB * IB ? NT / (IB * IB) : 1;    // GEMM3 pattern groups
  static constexpr int GB = NT >= IB * IB ? 1 : (IB * IB) / NT;    // GEMM3 blocks per thread
  static_assert(NT >= IB * IB || (IB * IB) % NT == 0, "GEMM3 blocks must divide evenly");
};

// shared-memory bytes of the two kernels
template <typename T, int SP, int PT>
constexpr size_t wide_fwd_smem() {
  using C = WideCfg<T, SP, PT>;
  return sizeof(T) * (2 * SP * SP + 2 * SP * C::XS) + sizeof(double) * C::IB * PT + sizeof(int) * PT;
}
// (stored_products: the adjoint reads the post-order's products and keeps no P^T)
template <typename T, int SP, int PT>
constexpr size_t wide_bwd_smem(bool stored_products = false) {
  using C = WideCfg<T, SP, PT>;
  return sizeof(T) * ((stored_products ? 2 : 4) * SP * SP + 3 * SP * C::XS + PT) + sizeof(double) * C::IB * PT +
         sizeof(int) * 4 * PT;
}

template <int IB>
__device__ __forceinline__ int wperm(int i) {
  return (i % IB) * 4 + i / IB;
}

template <typename T>
struct V4;
template <>
struct V4<float> {
  static __device__ __forceinline__ void ld(const float *p, float (&v)[4]) {
    const float4 f = *reinterpret_cast<const float4 *>(p);
    v[0] = f.x, v[1] = f.y, v[2] = f.z, v[3] = f.w;
  }
  static __device__ __forceinline__ void ldg(const float *p, float (&v)[4]) {
    const float4 f = __ldg(reinterpret_cast<const float4 *>(p));
    v[0] = f.x, v[1] = f.y, v[2] = f.z, v[3] = f.w;
  }
  static __device__ __forceinline__ void st(float *p, const float (&v)[4]) {
    *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
  }
};
template <>
struct V4<double> {
  static __device__ __forceinline__ void ld(const double *p, double (&v)[4]) {
    const double2 a = reinterpret_cast<const double2 *>(p)[0], b = reinterpret_cast<const double2 *>(p)[1];
    v[0] = a.x, v[1] = a.y, v[2] = b.x, v[3] = b.y;
  }
  static __device__ __forceinline__ void ldg(const double *p, double (&v)[4]) {
    const double2 a = __ldg(reinterpret_cast<const double2 *>(p)), b = __ldg(reinterpret_cast<const double2 *>(p) + 1);
    v[0] = a.x, v[1] = a.y, v[2] = b.x, v[3] = b.y;
  }
  static __device__ __forceinline__ void st(double *p, const double (&v)[4]) {
    reinterpret_cast<double2 *>(p)[0] = make_double2(v[0], v[1]);
    reinterpret_cast<double2 *>(p)[1] = make_double2(v[2], v[3]);
  }
};

// acc[i][j] += a[i] b[j] over a 4 x 4 register tile; FP32 runs as packed
// FP32x2 FMAs (pairs along j), FP64 as scalar FMAs
__device__ __forceinline__ void outer4(double (&acc)[4][4], const double (&a)[4], const double (&b)[4]) {
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
}

__device__ __forceinline__ void outer4(float (&acc)[4][4], const float (&a)[4], const float (&b)[4]) {
  const float2 b01 = make_float2(b[0], b[1]), b23 = make_float2(b[2], b[3]);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float2 ai = make_float2(a[i], a[i]);
    const float2 lo = __ffma2_rn(ai, b01, make_float2(acc[i][0], acc[i][1]));
    const float2 hi = __ffma2_rn(ai, b23, make_float2(acc[i][2], acc[i][3]));
    acc[i][0] = lo.x, acc[i][1] = lo.y, acc[i][2] = hi.x, acc[i][3] = hi.y;
  }
}

// Gradient tile: acc[i][s] += sum_q u[i][q] x[s][q]; FP32 keeps the even and
// odd q in the two halves of a float2 accumulator (packed FMAs along q)
template <typename T>
struct GradTile {
  T v[4][4];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int s = 0; s < 4; ++s) v[i][s] = T(0);
  }
  __device__ __forceinline__ void add(const T (&u)[4][4], const T (&x)[4][4]) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int s = 0; s < 4; ++s)
#pragma unroll
        for (int q = 0; q < 4; ++q) v[i][s] = fma(u[i][q], x[s][q], v[i][s]);
  }
  __device__ __forceinline__ T get(int i, int s) const { return v[i][s]; }
};

template <>
struct GradTile<float> {
  float2 v[4][4];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int s = 0; s < 4; ++s) v[i][s] = make_float2(0.0f, 0.0f);
  }
  __device__ __forceinline__ void add(const float (&u)[4][4], const float (&x)[4][4]) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        v[i][s] = __ffma2_rn(make_float2(u[i][0], u[i][1]), make_float2(x[s][0], x[s][1]), v[i][s]);
        v[i][s] = __ffma2_rn(make_float2(u[i][2], u[i][3]), make_float2(x[s][2], x[s][3]), v[i][s]);
      }
  }
  __device__ __forceinline__ float get(int i, int s) const { return v[i][s].x + v[i][s].y; }
};

template <typename T>
struct WideArgs {
  int tips, N, Npad, K, B, I, S, code_stride, rescale, nchunks, tiles_per_chunk, ntiles;
  const int *nodes;         // this level's node indices
  const int *left, *right;  // [I] children of internal node v - tips
  const uint8_t *codes;     // [tips][code_stride]
  const T *table;           // [C][SP]
  const T *pmat;            // [b][B][K][SP][SP]
  T *part;                  // [b][I][K][SP][Npad]
  int *expo;                // [b][I][K][Npad]
  const double *props;      // [b][K]
  const double *freqs;      // [b][S]
  const double *weights;    // [N]
  double *root_site;        // [b][K][Npad]: sum_i pi_i L_root[k][i] at exponent root_expo
  int *root_expo;           // [b][K][Npad]
  const double *log2L;      // [b][Npad] site log2-likelihoods (adjoint)
  T *gpart;                 // [b][B][nchunks][K][SP][SP]
  T *rootpart;              // [b][nchunks][K][SP + 1]
  // the children's products P_l x_l, P_r x_r of every internal node as the
  // post-order formed them, [b][I][K][2][SP][Npad], or nullptr: the adjoint
  // reads them instead of recomputing them
  T *prod;
};

// Stage a child's tile [SP][PT] (row stride XS): stored partial rows, or the
// code table rows of a tip's codes.
template <typename T, int SP, int PT>
__device__ __forceinline__ void wide_stage_child(const WideArgs<T> &a, int child, int b, int k, int n0, T *dst) {
  using C = WideCfg<T, SP, PT>;
  if (child < a.tips) {
    const uint8_t *cd = a.codes + size_t(child) * a.code_stride + n0;
    for (int e = threadIdx.x; e < SP * PT; e += C::NT) {
      const int j = e / PT, p = e - j * PT;
      dst[j * C::XS + p] = a.table[int(cd[p]) * SP + j];
    }
  } else {
    const T *src = a.part + ((size_t(b) * a.I + (child - a.tips)) * a.K + k) * SP * size_t(a.Npad) + n0;
    constexpr int Q = PT / 4;
    for (int e = threadIdx.x; e < SP * Q; e += C::NT) {
      const int j = e / Q, c4 = e - j * Q;
      T v[4];
      V4<T>::ldg(src + size_t(j) * a.Npad + 4 * c4, v);
      V4<T>::st(dst + j * C::XS + 4 * c4, v);
    }
  }
}

template <typename T>
__device__ __forceinline__ int wide_child_expo(const WideArgs<T> &a, int child, int b, int k, int n) {
  return child < a.tips ? 0 : a.expo[((size_t(b) * a.I + (child - a.tips)) * a.K + k) * a.Npad + n];
}

// --------------------------------------------------------------- forward
template <typename T, int SP, int PT>
__global__ void __launch_bounds__(WideCfg<T, SP, PT>::NT) wide_forward_kernel(const WideArgs<T> a) {
  using C = WideCfg<T, SP, PT>;
  constexpr int IB = C::IB, NT = C::NT, XS = C::XS;
  extern __shared__ __align__(128) unsigned char smem[];
  T *plt = reinterpret_cast<T *>(smem);                          // [2][SP j][SP perm i]
  T *xs = plt + 2 * SP * SP;                                      // [2][SP][XS]
  double *red = reinterpret_cast<double *>(xs + 2 * SP * XS);     // [IB][PT]
  int *ex = reinterpret_cast<int *>(red + IB * PT);               // [PT]
  const int tid = threadIdx.x, ib = tid % IB, pb = tid / IB;
  const int v = a.nodes[blockIdx.y];
  const int b = blockIdx.z / a.K, k = blockIdx.z - (blockIdx.z / a.K) * a.K;
  const int n0 = blockIdx.x * PT;
  const int l = a.left[v - a.tips], r = a.right[v - a.tips];
  const bool is_root = v == 2 * a.tips - 2;

  for (int e = tid; e < 2 * SP * SP; e += NT) {
    const int c = e / (SP * SP), ij = e - c * SP * SP, i = ij / SP, j = ij - i * SP;
    plt[c * SP * SP + j * SP + wperm<IB>(i)] = a.pmat[((size_t(b) * a.B + (c ? r : l)) * a.K + k) * SP * SP + ij];
  }
  wide_stage_child<T, SP, PT>(a, l, b, k, n0, xs);
  wide_stage_child<T, SP, PT>(a, r, b, k, n0, xs + SP * XS);
  __syncthreads();

  T al[4][4], ar[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int q = 0; q < 4; ++q) al[i][q] = ar[i][q] = T(0);
#pragma unroll 4
  for (int j = 0; j < SP; ++j) {
    T pa[4], pc[4], xa[4], xc[4];
    V4<T>::ld(plt + j * SP + ib * 4, pa);
    V4<T>::ld(plt + SP * SP + j * SP + ib * 4, pc);
    V4<T>::ld(xs + j * XS + pb * 4, xa);
    V4<T>::ld(xs + SP * XS + j * XS + pb * 4, xc);
    outer4(al, pa, xa);
    outer4(ar, pc, xc);
  }
  if (sizeof(T) == 4 && SP == 64 && a.prod) {
    T *pd = a.prod + ((size_t(b) * a.I + (v - a.tips)) * a.K + k) * 2 * SP * size_t(a.Npad) + n0 + pb * 4;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      V4<T>::st(pd + size_t(ib + IB * i) * a.Npad, al[i]);
      V4<T>::st(pd + size_t(SP + ib + IB * i) * a.Npad, ar[i]);
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int q = 0; q < 4; ++q) al[i][q] *= ar[i][q];

  if (is_root) {  // sum_i pi_i L[k][i] per pattern, FP64
    double f[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int row = ib + IB * i;
      f[i] = row < a.S ? a.freqs[size_t(b) * a.S + row] : 0.0;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      double s = 0.0;
#pragma unroll
      for (int i = 0; i < 4; ++i) s = fma(f[i], double(al[i][q]), s);
      red[ib * PT + pb * 4 + q] = s;
    }
    __syncthreads();
    if (tid < PT) {
      double s = 0.0;
      for (int u = 0; u < IB; ++u) s += red[u * PT + tid];
      const int n = n0 + tid;
      const size_t o = (size_t(b) * a.K + k) * a.Npad + n;
      a.root_site[o] = s;
      a.root_expo[o] = wide_child_expo(a, l, b, k, n) + wide_child_expo(a, r, b, k, n);
    }
    return;
  }
  if (a.rescale) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      T m = T(0);
#pragma unroll
      for (int i = 0; i < 4; ++i) m = fmax(m, al[i][q]);
      red[ib * PT + pb * 4 + q] = double(m);
    }
    __syncthreads();
    if (tid < PT) {
      double m = 0.0;
      for (int u = 0; u < IB; ++u) m = fmax(m, red[u * PT + tid]);
      ex[tid] = scale_exponent(T(m));
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = ex[pb * 4 + q];
#pragma unroll
      for (int i = 0; i < 4; ++i) al[i][q] = times_pow2_neg(al[i][q], e);
    }
  }
  T *dst = a.part + ((size_t(b) * a.I + (v - a.tips)) * a.K + k) * SP * size_t(a.Npad) + n0 + pb * 4;
#pragma unroll
  for (int i = 0; i < 4; ++i) V4<T>::st(dst + size_t(ib + IB * i) * a.Npad, al[i]);
  if (tid < PT) {
    const int n = n0 + tid;
    a.expo[((size_t(b) * a.I + (v - a.tips)) * a.K + k) * a.Npad + n] =
        wide_child_expo(a, l, b, k, n) + wide_child_expo(a, r, b, k, n) + (a.rescale ? ex[tid] : 0);
  }
}

// Root combination: site log-likelihoods, log2 L_p for the adjoint and the
// pattern-weighted per-block sums (FP64).  256 patterns per block.
__global__ void wide_root_kernel(const double *root_site, const int *root_expo, const double *props,
                                 const double *weights, double *site_lnl, double *log2L, double *block_lnl,
                                 int K, int N, int Npad);

// --------------------------------------------------------------- adjoint
// CTAs per SM the adjoint's registers are sized for: two for FP32 plans
// (codon plans read the stored products and keep no transposed matrices, so
// two fit the shared memory too)
template <typename T, int SP>
__host__ __device__ constexpr int wide_bwd_min_blocks() {
  return sizeof(T) == 4 ? (SP == 64 ? 2 : 3) : 1;
}

template <typename T, int SP, int PT>
__global__ void __launch_bounds__(WideCfg<T, SP, PT>::NT, wide_bwd_min_blocks<T, SP>())
    wide_backward_kernel(const WideArgs<T> a) {
  using C = WideCfg<T, SP, PT>;
  constexpr int IB = C::IB, NT = C::NT, XS = C::XS, NG = C::NG, GB = C::GB;
  extern __shared__ __align__(128) unsigned char smem[];
  // stored products: FP32 codon plans only (the other instantiations keep GEMM1)
  constexpr bool kProd = sizeof(T) == 4 && SP == 64;
  const bool prod = kProd && a.prod != nullptr;
  T *plt = reinterpret_cast<T *>(smem);       // [2][SP j][SP perm i]   P^T (GEMM1, absent with stored products)
  T *pl = prod ? plt : plt + 2 * SP * SP;     // [2][SP i][SP perm j]   P   (GEMM2)
  T *xs = pl + 2 * SP * SP;              // [2][SP][XS] child tiles
  T *us = xs + 2 * SP * XS;              // [SP][XS]    u of the current side
  T *cf = us + SP * XS;                  // [PT]        coefficients
  double *red = reinterpret_cast<double *>(cf + PT);  // [IB][PT]
  int *ex = reinterpret_cast<int *>(red + IB * PT);   // [PT]
  int *el = ex + PT, *er = el + PT, *ep = er + PT;    // [PT] exponents of x_l, x_r, pre
  const int tid = threadIdx.x, ib = tid % IB, pb = tid / IB;
  const int v = a.nodes[blockIdx.y];
  const int b = blockIdx.z / a.K, k = blockIdx.z - (blockIdx.z / a.K) * a.K;
  const int chunk = blockIdx.x;
  const int l = a.left[v - a.tips], r = a.right[v - a.tips];
  const bool is_root = v == 2 * a.tips - 2;
  const double wk = a.props[size_t(b) * a.K + k];

  for (int e = tid; e < 2 * SP * SP; e += NT) {
    const int c = e / (SP * SP), ij = e - c * SP * SP, i = ij / SP, j = ij - i * SP;
    const T val = a.pmat[((size_t(b) * a.B + (c ? r : l)) * a.K + k) * SP * SP + ij];
    if (!prod) plt[c * SP * SP + j * SP + wperm<IB>(i)] = val;
    pl[c * SP * SP + i * SP + wperm<IB>(j)] = val;
  }
  // GEMM3 ownership: block (gi, gj) of the SP x SP gradient, pattern quads grp, grp + NG, ...
  const int grp = NT >= IB * IB ? tid / (IB * IB) : 0;
  const bool g3 = grp < NG;
  GradTile<T> gacc[2][GB];
#pragma unroll
  for (int c = 0; c < 2; ++c)
#pragma unroll
    for (int m = 0; m < GB; ++m) gacc[c][m].zero();
  T rp[4] = {T(0), T(0), T(0), T(0)}, rw = T(0);  // root: dlnL/dpi rows, dlnL/dw_k
  double fr[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int row = ib + IB * i;
    fr[i] = row < a.S ? a.freqs[size_t(b) * a.S + row] : 0.0;
  }

  const int t0 = chunk * a.tiles_per_chunk, t1 = min(a.ntiles, t0 + a.tiles_per_chunk);
  for (int tile = t0; tile < t1; ++tile) {
    const int n0 = tile * PT;
    __syncthreads();  // previous tile's readers are done
    if (tile + 1 < t1) {  // the next tile's rows into L2 while this one computes
      constexpr int LPR = PT * int(sizeof(T)) / 128;  // 128-byte lines per tile row
      const int rows_l = l >= a.tips ? SP : 0, rows_r = r >= a.tips ? SP : 0, rows_p = is_root ? 0 : SP;
      const int rows_q = (kProd && a.prod) ? 2 * SP : 0;
      const int nrows = rows_l + rows_r + rows_p + rows_q;
      for (int e = tid; e < nrows * LPR; e += NT) {
        int row = e / LPR;
        const int seg = e - row * LPR;
        const T *base;
        if (row < rows_l) {
          base = a.part + ((size_t(b) * a.I + (l - a.tips)) * a.K + k) * SP * size_t(a.Npad);
        } else if ((row -= rows_l) < rows_r) {
          base = a.part + ((size_t(b) * a.I + (r - a.tips)) * a.K + k) * SP * size_t(a.Npad);
        } else if ((row -= rows_r) < rows_p) {
          base = a.part + ((size_t(b) * a.I + (v - a.tips)) * a.K + k) * SP * size_t(a.Npad);
        } else {
          row -= rows_p;
          base = a.prod + ((size_t(b) * a.I + (v - a.tips)) * a.K + k) * 2 * SP * size_t(a.Npad);
        }
        asm volatile("prefetch.global.L2 [%0];" ::"l"(base + size_t(row) * a.Npad + n0 + PT + seg * (128 / int(sizeof(T)))));
      }
    }
    wide_stage_child<T, SP, PT>(a, l, b, k, n0, xs);
    wide_stage_child<T, SP, PT>(a, r, b, k, n0, xs + SP * XS);
    if (tid < PT) {
      const int n = n0 + tid;
      const int El = wide_child_expo(a, l, b, k, n), Er = wide_child_expo(a, r, b, k, n);
      const int Ep = is_root ? 0 : a.expo[((size_t(b) * a.I + (v - a.tips)) * a.K + k) * a.Npad + n];
      el[tid] = El;
      er[tid] = Er;
      ep[tid] = Ep;
      T c = T(0);
      if (n < a.N) {
        const double dd = double(Ep + El + Er) - a.log2L[size_t(b) * a.Npad + n];
        if constexpr (sizeof(T) == 8) {
          c = a.weights[n] * exp2(dd);
        } else {  // the fraction's power in FP32 (an FP64 exp2 costs thousands of FP64-pipe cycles per warp)
          const double fl = floor(dd);
          c = ldexpf(float(a.weights[n]) * exp2f(float(dd - fl)), int(fl));
        }
      }
      cf[tid] = c;
    }
    // this thread's block of the outside partial of v
    T pre[4][4];
    if (is_root) {
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int q = 0; q < 4; ++q) pre[i][q] = T(wk * fr[i]);
    } else {
      const T *src = a.part + ((size_t(b) * a.I + (v - a.tips)) * a.K + k) * SP * size_t(a.Npad) + n0 + pb * 4;
#pragma unroll
      for (int i = 0; i < 4; ++i) V4<T>::ldg(src + size_t(ib + IB * i) * a.Npad, pre[i]);
    }
    __syncthreads();

    T al[4][4], ar[4][4];
    if (prod) {  // the post-order's products
      const T *pd =
          a.prod + ((size_t(b) * a.I + (v - a.tips)) * a.K + k) * 2 * SP * size_t(a.Npad) + n0 + pb * 4;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        V4<T>::ldg(pd + size_t(ib + IB * i) * a.Npad, al[i]);
        V4<T>::ldg(pd + size_t(SP + ib + IB * i) * a.Npad, ar[i]);
      }
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int q = 0; q < 4; ++q) al[i][q] = ar[i][q] = T(0);
#pragma unroll 4
      for (int j = 0; j < SP; ++j) {
        T pa[4], pc[4], xa[4], xc[4];
        V4<T>::ld(plt + j * SP + ib * 4, pa);
        V4<T>::ld(plt + SP * SP + j * SP + ib * 4, pc);
        V4<T>::ld(xs + j * XS + pb * 4, xa);
        V4<T>::ld(xs + SP * XS + j * XS + pb * 4, xc);
        outer4(al, pa, xa);
        outer4(ar, pc, xc);
      }
    }
    if (is_root) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const T c = cf[pb * 4 + q];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const T R = c * al[i][q] * ar[i][q];
          rp[i] = fma(T(wk), R, rp[i]);
          rw = fma(T(fr[i]), R, rw);
        }
      }
    }

#pragma unroll
    for (int side = 0; side < 2; ++side) {
      const int child = side ? r : l;
      // u = pre .* (product of the other side)
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        T u4[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) u4[q] = pre[i][q] * (side ? al[i][q] : ar[i][q]);
        V4<T>::st(us + (ib + IB * i) * XS + pb * 4, u4);
      }
      __syncthreads();
      if (child >= a.tips) {  // GEMM2: outside partial of the child, rescaled, in place of its forward partial
        const T *pm = pl + side * SP * SP;
        T o[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int q = 0; q < 4; ++q) o[i][q] = T(0);
#pragma unroll 4
        for (int i = 0; i < SP; ++i) {
          T pa[4], ua[4];
          V4<T>::ld(pm + i * SP + ib * 4, pa);
          V4<T>::ld(us + i * XS + pb * 4, ua);
          outer4(o, pa, ua);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          T m = T(0);
#pragma unroll
          for (int s = 0; s < 4; ++s) m = fmax(m, o[s][q]);
          red[ib * PT + pb * 4 + q] = double(m);
        }
        __syncthreads();
        if (tid < PT) {
          double m = 0.0;
          for (int u = 0; u < IB; ++u) m = fmax(m, red[u * PT + tid]);
          const int e = scale_exponent(T(m));
          ex[tid] = e;
          const int n = n0 + tid;
          a.expo[((size_t(b) * a.I + (child - a.tips)) * a.K + k) * a.Npad + n] =
              ep[tid] + (side ? el[tid] : er[tid]) + e;
        }
        __syncthreads();
        T *dst = a.part + ((size_t(b) * a.I + (child - a.tips)) * a.K + k) * SP * size_t(a.Npad) + n0 + pb * 4;
#pragma unroll
        for (int s = 0; s < 4; ++s) {
          T o4[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) o4[q] = times_pow2_neg(o[s][q], ex[pb * 4 + q]);
          V4<T>::st(dst + size_t(ib + IB * s) * a.Npad, o4);
        }
      }
      // GEMM3: dlnL/dP_child += sum_p c_p u[i][p] x_child[j][p]
      if (g3) {
        const T *xc = xs + side * SP * XS;
#pragma unroll
        for (int m = 0; m < GB; ++m) {
          const int blk = NT >= IB * IB ? tid % (IB * IB) : tid + m * NT;
          const int gi = blk / IB, gj = blk - gi * IB;
          for (int qd = grp; qd < PT / 4; qd += NG) {
            T c4[4], uu[4][4], xx[4][4];
            V4<T>::ld(cf + qd * 4, c4);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              V4<T>::ld(us + (gi + IB * i) * XS + qd * 4, uu[i]);
#pragma unroll
              for (int q = 0; q < 4; ++q) uu[i][q] *= c4[q];
            }
#pragma unroll
            for (int s = 0; s < 4; ++s) V4<T>::ld(xc + (gj + IB * s) * XS + qd * 4, xx[s]);
            gacc[side][m].add(uu, xx);
          }
        }
      }
      __syncthreads();  // us is rewritten by the next side / tile
    }
  }

  // per-chunk gradient blocks (groups summed in fixed order through shared memory)
  T *gsum = xs;  // reuse: [NG][SP*SP] for NG > 1
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const int child = side ? r : l;
    T *dst = a.gpart + (((size_t(b) * a.B + child) * a.nchunks + chunk) * a.K + k) * SP * SP;
    if (NG == 1) {
      if (g3) {
#pragma unroll
        for (int m = 0; m < GB; ++m) {
          const int blk = NT >= IB * IB ? tid % (IB * IB) : tid + m * NT;
          const int gi = blk / IB, gj = blk - gi * IB;
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int s = 0; s < 4; ++s) dst[(gi + IB * i) * SP + gj + IB * s] = gacc[side][m].get(i, s);
        }
      }
    } else {
      __syncthreads();
      if (g3) {
        const int blk = tid % (IB * IB);
        const int gi = blk / IB, gj = blk - gi * IB;
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int s = 0; s < 4; ++s) gsum[grp * SP * SP + (gi + IB * i) * SP + gj + IB * s] = gacc[side][0].get(i, s);
      }
      __syncthreads();
      for (int e = tid; e < SP * SP; e += NT) {
        T s = T(0);
        for (int g = 0; g < NG; ++g) s += gsum[g * SP * SP + e];
        dst[e] = s;
      }
    }
  }
  if (is_root) {  // block sums of the root gradients, fixed order
    __syncthreads();
    T *rs = xs;  // [NT][5]
#pragma unroll
    for (int i = 0; i < 4; ++i) rs[tid * 5 + i] = rp[i];
    rs[tid * 5 + 4] = rw;
    __syncthreads();
    T *dst = a.rootpart + ((size_t(b) * a.nchunks + chunk) * a.K + k) * (SP + 1);
    for (int row = tid; row <= SP; row += NT) {
      T s = T(0);
      if (row < SP) {
        const int bi = row % IB, i = row / IB;
        for (int p = 0; p < C::PB; ++p) s += rs[(p * IB + bi) * 5 + i];
      } else {
        for (int t = 0; t < NT; ++t) s += rs[t * 5 + 4];
      }
      dst[row] = s;
    }
  }
}

// Chunks of pattern tiles of one level launch of a wide-state adjoint: about
// target CTAs (eight waves at the kernel's CTAs per SM) over the level's
// nodes x samples x categories (bk), at most cmax chunks of the ntc tiles.
// Levels with many nodes get few long chunks: fewer CTAs, so less per-CTA
// set-up and fewer gradient blocks to write and sum.
__host__ __device__ inline int tc_level_chunks(int nodes, int bk, int ntc, int cmax, int target = 8 * 152) {
  const long long want = ((long long)target + (long long)nodes * bk - 1) / ((long long)nodes * bk);
  const int c = int(want < 1 ? 1 : (want > cmax ? cmax : want));
  const int tpc = (ntc + c - 1) / c;
  return (ntc + tpc - 1) / tpc;
}

// Fixed-order sums over chunks: G[b][branch][k][S][S] (FP64, unpadded) and
// the root gradients dfreq[b][S], dprop[b][K]; accumulate = 1 adds to what
// is there (pattern slabs after the first).  nchunks is the chunk stride of
// gpart; with branch_lvn (the node count of each branch's parent level) a
// branch sums only the chunks its level launched, tc_level_chunks(lvn, bk,
// ntc, cmax).
template <typename T>
__global__ void wide_grad_reduce_kernel(const T *gpart, double *G, int B, int nchunks, int K, int S, int SP,
                                        int accumulate, const int *branch_lvn = nullptr, int bk = 0, int ntc = 0,
                                        int cmax = 0, int target = 8 * 152) {
  // four consecutive columns per thread, threads along the row: 16-byte (FP32) or 2 x 16-byte
  // (FP64) loads of every chunk's block, the chunk sum in the plan's precision and a fixed
  // order, then FP64 (FP64 arithmetic is scarce on this GPU and the chunk blocks themselves are
  // in the plan's precision).  SP is a multiple of 4, so every load is aligned.
  const int br = blockIdx.x, b = blockIdx.y;
  const int kss = K * S * S, q4 = SP / 4;
  const size_t cstride = size_t(K) * SP * SP;  // between chunks
  const T *base = gpart + (size_t(b) * B + br) * nchunks * cstride;
  const int used = branch_lvn ? tc_level_chunks(branch_lvn[br], bk, ntc, cmax, target) : nchunks;
  double *gb = G + (size_t(b) * B + br) * kss;
  for (int e = threadIdx.x; e < K * S * q4; e += blockDim.x) {
    const int kr = e / q4, j0 = (e - kr * q4) * 4;
    if (j0 >= S) continue;
    const int k = kr / S, i = kr - k * S;
    const T *src = base + size_t(k) * SP * SP + i * SP + j0;
    T s0 = T(0), s1 = T(0), s2 = T(0), s3 = T(0);
#pragma unroll 4
    for (int c = 0; c < used; ++c) {
      const T *cs = src + c * cstride;
      if constexpr (sizeof(T) == 4) {
        const float4 v = *reinterpret_cast<const float4 *>(cs);
        s0 += v.x;
        s1 += v.y;
        s2 += v.z;
        s3 += v.w;
      } else {
        const double2 v0 = reinterpret_cast<const double2 *>(cs)[0], v1 = reinterpret_cast<const double2 *>(cs)[1];
        s0 += v0.x;
        s1 += v0.y;
        s2 += v1.x;
        s3 += v1.y;
      }
    }
    const T sv[4] = {s0, s1, s2, s3};
    double *g = gb + (size_t(k) * S + i) * S + j0;
#pragma unroll
    for (int t = 0; t < 4; ++t)
      if (j0 + t < S) g[t] = accumulate ? g[t] + double(sv[t]) : double(sv[t]);
  }
}

template <typename T>
__global__ void wide_root_reduce_kernel(const T *rootpart, double *dfreq, double *dprop, int nchunks, int K, int S,
                                        int SP, int accumulate) {
  const int b = blockIdx.x;
  for (int e = threadIdx.x; e < S + K; e += blockDim.x) {
    double s = 0.0;
    if (e < S) {
      for (int c = 0; c < nchunks; ++c)
        for (int k = 0; k < K; ++k) s += double(rootpart[((size_t(b) * nchunks + c) * K + k) * (SP + 1) + e]);
      double *d = dfreq + size_t(b) * S + e;
      *d = accumulate ? *d + s : s;
    } else {
      const int k = e - S;
      for (int c = 0; c < nchunks; ++c) s += double(rootpart[((size_t(b) * nchunks + c) * K + k) * (SP + 1) + SP]);
      double *d = dprop + size_t(b) * K + k;
      *d = accumulate ? *d + s : s;
    }
  }
}

// ------------------------------------------------------ transition matrices
// P[b][br][k] = I + U diag(expm1(lambda t r_k)) W over the padded SP x SP
// block (zero outside S x S), products in T, exponentials in FP64.  One CTA
// per (branch, sample), all categories; 4 x 4 register tiles.  U and W are
// converted to T once per CTA, and U diag(d) is formed in T: FP64 arithmetic
// (and conversions from FP64) run at a small fraction of the FP32 rate here.
template <typename T, int SP>
__global__ void __launch_bounds__(256) wide_pmatrix_kernel(const double *lam, const double *U, const double *W,
                                                           const double *bl, const double *rates, T *pmat, int S,
                                                           int B, int K) {
  constexpr int IB = SP / 4;
  extern __shared__ __align__(128) unsigned char smem[];
  T *ut = reinterpret_cast<T *>(smem);  // [m][perm i] = U[i][m] * d_m
  T *wm = ut + SP * SP;                 // [m][perm j] = W[m][j]
  T *u0 = wm + SP * SP;                 // [m][perm i] = U[i][m]
  T *dt = u0 + SP * SP;                 // [SP] d_m in T
  const int br = blockIdx.x, b = blockIdx.y, tid = threadIdx.x;
  const double t = bl[size_t(b) * B + br];
  for (int e = tid; e < SP * SP; e += 256) {
    const int m = e / SP, j = e - m * SP;
    wm[m * SP + wperm<IB>(j)] = (m < S && j < S) ? T(W[(size_t(b) * S + m) * S + j]) : T(0);
    const int i = m, mm = j;  // u0[mm][perm i] = U[i][mm]
    u0[mm * SP + wperm<IB>(i)] = (mm < S && i < S) ? T(U[(size_t(b) * S + i) * S + mm]) : T(0);
  }
  for (int k = 0; k < K; ++k) {
    const double tr = t * rates[size_t(b) * K + k];
    __syncthreads();
    for (int m = tid; m < SP; m += 256) dt[m] = m < S ? T(expm1(lam[size_t(b) * S + m] * tr)) : T(0);
    __syncthreads();
    for (int e = tid; e < SP * SP; e += 256) ut[e] = u0[e] * dt[e / SP];
    __syncthreads();
    T *dst = pmat + ((size_t(b) * B + br) * K + k) * SP * SP;
    for (int blk = tid; blk < IB * IB; blk += 256) {
      const int bi = blk / IB, bj = blk - bi * IB;
      T acc[4][4];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
      for (int m = 0; m < SP; ++m) {
        T ua[4], wa[4];
        V4<T>::ld(ut + m * SP + bi * 4, ua);
        V4<T>::ld(wm + m * SP + bj * 4, wa);
        outer4(acc, ua, wa);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int gi = bi + IB * i, gj = bj + IB * j;
          dst[gi * SP + gj] = (gi == gj && gi < S) ? acc[i][j] + T(1) : acc[i][j];
        }
    }
  }
}

// Caller-given matrices [b][B][K][S][S] (FP64) -> padded [b][B][K][SP][SP].
template <typename T>
__global__ void wide_pmatrix_copy_kernel(const double *src, T *pmat, int S, int SP, long long count) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= count) return;  // count = b * B * K * SP * SP
  const int jj = int(idx % SP), ii = int((idx / SP) % SP);
  const long long mat = idx / (SP * SP);
  pmat[idx] = (ii < S && jj < S) ? T(src[(mat * S + ii) * S + jj]) : T(0);
}

// Gradient through P = I + U D W, D = diag(expm1(lambda t r_k)):
//   dU += G W^T D,  dW += D U^T G,  g_m = (U^T G W^T)_mm,
//   dlambda_m += g_m e_m t r_k,  dt += sum_m g_m e_m lambda_m r_k,
//   dr_k += sum_m g_m e_m lambda_m t.
// One CTA per (chunk of branches, sample); dU/dW/dlambda/dr are written per
// chunk and summed by wide_pmatrix_grad_reduce_kernel; dt per branch directly.
template <typename T, int SP>
__global__ void __launch_bounds__(256) wide_pmatrix_backward_kernel(const double *G, const double *lam,
                                                                    const double *U, const double *W,
                                                                    const double *bl, const double *rates, int S,
                                                                    int B, int K, int bchunk, double *dbl,
                                                                    double *part) {
  constexpr int IB = SP / 4;
  constexpr int NB = (IB * IB + 255) / 256;  // 4x4 blocks per thread
  extern __shared__ __align__(128) unsigned char smem[];
  T *ug = reinterpret_cast<T *>(smem);  // [i][perm m] = U[i][m]     (Y = U^T G: rows m)
  T *wt = ug + SP * SP;                  // [j][perm m] = W[m][j]     (H = G W^T: cols m)
  T *gt = wt + SP * SP;                  // [j][perm i] = G[i][j]     (H: rows i)
  T *gg = gt + SP * SP;                  // [i][perm j] = G[i][j]     (Y: cols j)
  double *dg = reinterpret_cast<double *>(gg + SP * SP);  // [IB][SP] partial diagonals
  double *gm = dg + IB * SP;                               // [SP]
  double *acc_l = gm + SP;                                 // [SP] dlambda accumulators
  double *acc_r = acc_l + SP;                              // [K]
  double *red = acc_r + 8;                                 // [SP]
  const int chunk = blockIdx.x, b = blockIdx.y, tid = threadIdx.x;
  for (int e = tid; e < SP * SP; e += 256) {
    const int x = e / SP, y = e - x * SP;
    const bool in = x < S && y < S;
    ug[x * SP + wperm<IB>(y)] = in ? T(U[(size_t(b) * S + x) * S + y]) : T(0);  // x = i, y = m
    wt[y * SP + wperm<IB>(x)] = in ? T(W[(size_t(b) * S + x) * S + y]) : T(0);  // x = m, y = j
  }
  for (int e = tid; e < SP; e += 256) acc_l[e] = 0.0;
  if (tid < 8) acc_r[tid] = 0.0;
  T dU[NB][4][4], dW[NB][4][4];
#pragma unroll
  for (int n = 0; n < NB; ++n)
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) dU[n][i][j] = dW[n][i][j] = T(0);
  const int br0 = chunk * bchunk, br1 = min(B, br0 + bchunk);
  for (int br = br0; br < br1; ++br) {
    const double t = bl[size_t(b) * B + br];
    double dt = 0.0;
    for (int k = 0; k < K; ++k) {
      const double tr = t * rates[size_t(b) * K + k];
      __syncthreads();
      const double *g = G + ((size_t(b) * B + br) * K + k) * S * S;
      for (int e = tid; e < SP * SP; e += 256) {
        const int i = e / SP, j = e - i * SP;
        const T val = (i < S && j < S) ? T(g[i * S + j]) : T(0);
        gt[j * SP + wperm<IB>(i)] = val;
        gg[i * SP + wperm<IB>(j)] = val;
      }
      __syncthreads();
#pragma unroll
      for (int n = 0; n < NB; ++n) {
        const int blk = tid + n * 256;
        if (blk < IB * IB) {
          const int bi = blk / IB, bm = blk - bi * IB;
          // H block: rows i = bi + IB*x, cols m = bm + IB*y
          T h[4][4], y4[4][4];
#pragma unroll
          for (int x = 0; x < 4; ++x)
#pragma unroll
            for (int y = 0; y < 4; ++y) h[x][y] = y4[x][y] = T(0);
          for (int j = 0; j < SP; ++j) {
            T ga[4], wa[4];
            V4<T>::ld(gt + j * SP + bi * 4, ga);
            V4<T>::ld(wt + j * SP + bm * 4, wa);
            outer4(h, ga, wa);
          }
          // Y block: rows m = bi + IB*x, cols j = bm + IB*y  (Y = U^T G)
          for (int i = 0; i < SP; ++i) {
            T ua[4], ga[4];
            V4<T>::ld(ug + i * SP + bi * 4, ua);
            V4<T>::ld(gg + i * SP + bm * 4, ga);
            outer4(y4, ua, ga);
          }
          // dU[i][m] += H[i][m] d_m ; dW[m][j] += d_m Y[m][j] ; diagonal partials sum_i U[i][m] H[i][m]
          double dd[4], dr4[4];
#pragma unroll
          for (int y = 0; y < 4; ++y) {
            const int m = bm + IB * y;
            dd[y] = m < S ? expm1(lam[size_t(b) * S + m] * tr) : 0.0;
          }
#pragma unroll
          for (int x = 0; x < 4; ++x) {
            const int m = bi + IB * x;
            dr4[x] = m < S ? expm1(lam[size_t(b) * S + m] * tr) : 0.0;
          }
#pragma unroll
          for (int x = 0; x < 4; ++x)
#pragma unroll
            for (int y = 0; y < 4; ++y) {
              dU[n][x][y] = fma(h[x][y], T(dd[y]), dU[n][x][y]);
              dW[n][x][y] = fma(T(dr4[x]), y4[x][y], dW[n][x][y]);
            }
          // partial diagonal: for cols m (bm + IB*y): sum over this block's rows i of U[i][m] H[i][m]
#pragma unroll
          for (int y = 0; y < 4; ++y) {
            const int m = bm + IB * y;
            double s = 0.0;
#pragma unroll
            for (int x = 0; x < 4; ++x) {
              const int i = bi + IB * x;
              s += double(ug[i * SP + wperm<IB>(m)]) * double(h[x][y]);
            }
            dg[bi * SP + m] = s;
          }
        }
      }
      __syncthreads();
      for (int m = tid; m < SP; m += 256) {
        double s = 0.0;
        for (int x = 0; x < IB; ++x) s += dg[x * SP + m];
        double q = 0.0;
        if (m < S) {
          const double lm = lam[size_t(b) * S + m];
          const double em = exp(lm * tr);
          q = s * em;  // g_m e_m
          acc_l[m] += q * tr;
          q *= lm;
        }
        red[m] = q;
      }
      __syncthreads();
      if (tid == 0) {
        double s = 0.0;
        for (int m = 0; m < SP; ++m) s += red[m];
        dt += s * rates[size_t(b) * K + k];
        acc_r[k] += s * t;
      }
    }
    if (tid == 0 && dbl) dbl[size_t(b) * B + br] = dt;
  }
  __syncthreads();
  // chunk partial: [dU S*S][dW S*S][dlambda S][dr K]
  const int width = 2 * S * S + S + K;
  double *dst = part + (size_t(b) * gridDim.x + chunk) * width;
#pragma unroll
  for (int n = 0; n < NB; ++n) {
    const int blk = tid + n * 256;
    if (blk < IB * IB) {
      const int bi = blk / IB, bm = blk - bi * IB;
#pragma unroll
      for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y) {
          const int r0 = bi + IB * x, c0 = bm + IB * y;
          if (r0 < S && c0 < S) {
            dst[r0 * S + c0] = double(dU[n][x][y]);          // dU[i][m]
            dst[S * S + r0 * S + c0] = double(dW[n][x][y]);  // dW[m][j]
          }
        }
    }
  }
  for (int m = tid; m < S; m += 256) dst[2 * S * S + m] = acc_l[m];
  if (tid < K) dst[2 * S * S + S + tid] = acc_r[tid];
}

__global__ void wide_pmatrix_grad_reduce_kernel(const double *part, int nchunks, int S, int K, double *dlam,
                                                double *dU, double *dW, double *drates);

}  // namespace tt
