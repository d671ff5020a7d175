// Pattern-tiled pruning kernels.
//
// Patterns are independent up to the final weighted sum
// (torchtree/evolution/tree_likelihood.py:186-221 rescales per pattern), so
// one CTA owns a tile of TILE patterns of one batch sample and walks the
// whole post-order itself.  Each thread owns one pattern and all K rate
// categories.  Child partials that are still needed live in a shared-memory
// stack whose slots the host assigned (Sethi-Ullman order keeps the stack
// depth <= log2(T)+1); the transition matrices of each step are staged into
// shared memory by the TMA engine (cp.async.bulk) a few steps ahead.
//
// Forward  (replaces tree_likelihood.py:40-75 / 186-221): the only HBM
// traffic is writing each non-root internal partial once (when the gradient
// needs it) plus tip codes.
// Backward (replaces autograd through the same lines): walks the schedule in
// reverse (a pre-order), keeps the pre-order ("outside") partials in the
// shared-memory stack, reads each stored post-order partial once, and emits
// per-tile partial sums of dlnL/dP for every branch.
//
// Global partial layout: [batch][internal node - T][K][N][S], S innermost,
// so a warp's S-vector loads/stores of one category are fully coalesced.
#pragma once

#include "tt_common.cuh"

namespace tt {

// One post-order step: 12 ints (3 x int4).
//  [0] node [1] left [2] right [3] fwd slot of left (-1: tip)
//  [4] fwd slot of right [5] fwd output slot (-1: root) [6] bwd input slot
//  (-1: root) [7] bwd output slot of left (-1: tip) [8] bwd output slot of
//  right [9..11] unused
constexpr int kStepInts = 12;

template <typename T>
struct PruneArgs {
  const int4 *steps;
  int n_steps;    // internal nodes (T-1)
  int tip_count;  // T
  int branch_count;
  int N;
  int K;
  int C;  // tip codes in the table
  int slots;
  int rescale;
  int ntiles;
  const uint8_t *codes;   // [T][N]
  const T *table;         // [C][S]
  const T *pmat;          // [batch][n_steps][2][K][S][S]
  const double *props;    // [batch][K]
  const double *freqs;    // [batch][S]
  const double *weights;  // [N]
  T *partials;            // [batch][n_steps-1][K][N][S] or nullptr
  double *site_lnl;       // [batch][N] or nullptr
  double *tile_lnl;       // [batch][ntiles]
  T *gpart;               // [batch][B][ntiles][K*S*S]
  T *rootpart;            // [batch][ntiles][S+K]
  int *status;
  unsigned long long timeout_ns;
};

struct StackLayout {
  size_t pbuf, bars, table, stack, red, red_root, total;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

// Shared-memory carve-up shared by the host (launch size) and the kernels.
template <typename T>
__host__ __device__ inline StackLayout stack_layout(int S, int K, int C, int slots, int tile,
                                                    int nstage, int kmax, bool backward) {
  StackLayout L;
  size_t off = 0;
  L.pbuf = off;
  off = align16(off + size_t(nstage) * 2 * K * S * S * sizeof(T));
  L.bars = off;
  off = align16(off + size_t(nstage) * 8);
  L.table = off;
  off = align16(off + size_t(C) * S * sizeof(T));
  L.stack = off;
  off = align16(off + size_t(slots) * K * tile * S * sizeof(T));
  L.red = off;
  const int vp = ((kmax * S * S + 31) / 32) * 32;
  if (backward) off = align16(off + size_t(2) * (tile / 32) * 2 * vp * sizeof(T));
  L.red_root = off;
  if (backward) off = align16(off + size_t(tile / 32) * (S + kmax) * sizeof(T));
  L.total = off;
  return L;
}

// out[i] = sum_j P[i][j] v[j]   (P row-major S x S in shared memory)
template <typename T, int S>
__device__ __forceinline__ void matvec(T (&out)[S], const T *P, const T (&v)[S]) {
#pragma unroll
  for (int i = 0; i < S; ++i) {
    T row[S];
    load_vec<T, S>(row, P + i * S);
    T acc = T(0);
#pragma unroll
    for (int j = 0; j < S; ++j) acc = fma(row[j], v[j], acc);
    out[i] = acc;
  }
}

// out[j] = sum_i P[i][j] x[i]
template <typename T, int S>
__device__ __forceinline__ void matvec_t(T (&out)[S], const T *P, const T (&x)[S]) {
#pragma unroll
  for (int j = 0; j < S; ++j) out[j] = T(0);
#pragma unroll
  for (int i = 0; i < S; ++i) {
    T row[S];
    load_vec<T, S>(row, P + i * S);
#pragma unroll
    for (int j = 0; j < S; ++j) out[j] = fma(row[j], x[i], out[j]);
  }
}

template <typename T, int S, int KMAX>
__device__ __forceinline__ void rescale_pow2(T (&v)[KMAX][S], int K, int &E) {
  T m = T(0);
#pragma unroll
  for (int k = 0; k < KMAX; ++k)
    if (k < K) {
#pragma unroll
      for (int i = 0; i < S; ++i) m = fmax(m, v[k][i]);
    }
  const int e = scale_exponent(m);
  if (e != 0) {
#pragma unroll
    for (int k = 0; k < KMAX; ++k)
#pragma unroll
      for (int i = 0; i < S; ++i) v[k][i] = times_pow2_neg(v[k][i], e);
    E += e;
  }
}

// Issue the bulk copy of step `s`'s matrix pair into stage `st`.
template <typename T>
__device__ __forceinline__ void issue_pmat(T *pbuf, uint64_t *bars, const T *pm, int s, int st,
                                           size_t pstep) {
  const uint32_t bytes = static_cast<uint32_t>(pstep * sizeof(T));
  mbar_arrive_expect_tx(&bars[st], bytes);
  bulk_copy_g2s(pbuf + st * pstep, pm + size_t(s) * pstep, bytes, &bars[st]);
}

// On a timeout: record it, then give in-flight copies a bounded chance to
// land before the CTA exits.
template <int NSTAGE>
__device__ __forceinline__ void drain_after_timeout(uint64_t *bars, int first, int last,
                                                    int *status) {
  atomicExch(status, kDeviceTimeout);
  for (int j = first; j <= last; ++j)
    mbar_wait_bounded(&bars[j % NSTAGE], (j / NSTAGE) & 1, 100000000ull);
}

// ------------------------------------------------------------------ forward
template <typename T, int S, int KMAX, int TILE, int NSTAGE>
__global__ void __launch_bounds__(TILE) prune_forward_kernel(const PruneArgs<T> a) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ double warp_tot[TILE / 32];
  const int tid = threadIdx.x;
  const int b = blockIdx.y;
  const int tile = blockIdx.x;
  const int n = tile * TILE + tid;
  const bool act = n < a.N;
  const int K = a.K;
  const int KSS = K * S * S;
  const StackLayout L = stack_layout<T>(S, K, a.C, a.slots, TILE, NSTAGE, KMAX, false);
  T *pbuf = reinterpret_cast<T *>(smem + L.pbuf);
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L.bars);
  T *tab = reinterpret_cast<T *>(smem + L.table);
  T *stk = reinterpret_cast<T *>(smem + L.stack);
  const size_t pstep = 2 * size_t(KSS);
  const T *pm = a.pmat + size_t(b) * a.n_steps * pstep;
  const int nst = a.n_steps;

  if (tid == 0) {
#pragma unroll
    for (int st = 0; st < NSTAGE; ++st) mbar_init(&bars[st], 1);
    fence_barrier_init();
  }
  for (int i = tid; i < a.C * S; i += TILE) tab[i] = a.table[i];
  double props[KMAX], freqs[S];
#pragma unroll
  for (int k = 0; k < KMAX; ++k) props[k] = k < K ? a.props[b * K + k] : 0.0;
#pragma unroll
  for (int i = 0; i < S; ++i) freqs[i] = a.freqs[b * S + i];
  __syncthreads();
  if (tid == 0)
    for (int s = 0; s < NSTAGE - 1 && s < nst; ++s) issue_pmat(pbuf, bars, pm, s, s, pstep);
  bool timed_out = !mbar_wait_bounded(&bars[0], 0, a.timeout_ns);
  if (__syncthreads_or(timed_out)) {
    if (tid == 0) drain_after_timeout<NSTAGE>(bars, 0, min(NSTAGE - 2, nst - 1), a.status);
    return;
  }

  int E = 0;
  double ll = 0.0;
  for (int s = 0; s < nst; ++s) {
    if (tid == 0 && s + NSTAGE - 1 < nst) {
      const int sp = s + NSTAGE - 1;
      issue_pmat(pbuf, bars, pm, sp, sp % NSTAGE, pstep);
    }
    const T *Pl = pbuf + (s % NSTAGE) * pstep;
    const T *Pr = Pl + KSS;
    const int4 r0 = __ldg(a.steps + 3 * s);
    const int4 r1 = __ldg(a.steps + 3 * s + 1);
    const int node = r0.x, left = r0.y, right = r0.z;
    T prod[KMAX][S];
    // left child term
    if (left < a.tip_count) {
      const int code = act ? a.codes[size_t(left) * a.N + n] : 0;
      T v[S];
      load_vec<T, S>(v, tab + code * S);
#pragma unroll
      for (int k = 0; k < KMAX; ++k)
        if (k < K) matvec<T, S>(prod[k], Pl + k * S * S, v);
    } else {
      const int slot = r0.w;
#pragma unroll
      for (int k = 0; k < KMAX; ++k)
        if (k < K) {
          T v[S];
          load_vec<T, S>(v, stk + (size_t(slot * K + k) * TILE + tid) * S);
          matvec<T, S>(prod[k], Pl + k * S * S, v);
        }
    }
    // right child term, multiplied in
    if (right < a.tip_count) {
      const int code = act ? a.codes[size_t(right) * a.N + n] : 0;
      T v[S];
      load_vec<T, S>(v, tab + code * S);
#pragma unroll
      for (int k = 0; k < KMAX; ++k)
        if (k < K) {
          T t[S];
          matvec<T, S>(t, Pr + k * S * S, v);
#pragma unroll
          for (int i = 0; i < S; ++i) prod[k][i] *= t[i];
        }
    } else {
      const int slot = r1.x;
#pragma unroll
      for (int k = 0; k < KMAX; ++k)
        if (k < K) {
          T v[S], t[S];
          load_vec<T, S>(v, stk + (size_t(slot * K + k) * TILE + tid) * S);
          matvec<T, S>(t, Pr + k * S * S, v);
#pragma unroll
          for (int i = 0; i < S; ++i) prod[k][i] *= t[i];
        }
    }
    if (a.rescale) rescale_pow2<T, S, KMAX>(prod, K, E);
    const int out_slot = r1.y;
    if (out_slot >= 0) {
      T *gdst = a.partials
                    ? a.partials + (size_t(b) * (nst - 1) + (node - a.tip_count)) * K * size_t(a.N) * S
                    : nullptr;
#pragma unroll
      for (int k = 0; k < KMAX; ++k)
        if (k < K) {
          store_vec<T, S>(stk + (size_t(out_slot * K + k) * TILE + tid) * S, prod[k]);
          if (gdst && act) store_vec_stream<T, S>(gdst + (size_t(k) * a.N + n) * S, prod[k]);
        }
    } else {  // root: fold categories and frequencies in FP64
      double site = 0.0;
#pragma unroll
      for (int k = 0; k < KMAX; ++k)
        if (k < K) {
          double sk = 0.0;
#pragma unroll
          for (int i = 0; i < S; ++i) sk = fma(freqs[i], double(prod[k][i]), sk);
          site = fma(props[k], sk, site);
        }
      ll = log(site) + double(E) * 0.69314718055994530942;
    }
    if (s + 1 < nst) timed_out = !mbar_wait_bounded(&bars[(s + 1) % NSTAGE], ((s + 1) / NSTAGE) & 1,
                                                    a.timeout_ns);
    if (__syncthreads_or(timed_out)) {
      if (tid == 0) drain_after_timeout<NSTAGE>(bars, s + 1, min(s + NSTAGE - 1, nst - 1), a.status);
      return;
    }
  }

  if (a.site_lnl && act) a.site_lnl[size_t(b) * a.N + n] = ll;
  double contrib = act ? a.weights[n] * ll : 0.0;
  contrib = warp_sum(contrib);
  if ((tid & 31) == 0) warp_tot[tid >> 5] = contrib;
  __syncthreads();
  if (tid == 0) {
    double tot = 0.0;
#pragma unroll
    for (int w = 0; w < TILE / 32; ++w) tot += warp_tot[w];
    a.tile_lnl[size_t(b) * a.ntiles + tile] = tot;
  }
}

// ----------------------------------------------------------------- backward
// Child values for the adjoint: the tip's table vector (same for every
// category) or the stored post-order partial of an internal child.
template <typename T, int S, int KMAX>
__device__ __forceinline__ void child_values(T (&v)[KMAX][S], int child, const PruneArgs<T> &a,
                                             const T *tab, int b, int n, bool act) {
  const int K = a.K;
  if (child < a.tip_count) {
    const int code = act ? a.codes[size_t(child) * a.N + n] : 0;
    T t[S];
    load_vec<T, S>(t, tab + code * S);
#pragma unroll
    for (int k = 0; k < KMAX; ++k)
#pragma unroll
      for (int i = 0; i < S; ++i) v[k][i] = t[i];
  } else {
    const T *src =
        a.partials + (size_t(b) * (a.n_steps - 1) + (child - a.tip_count)) * K * size_t(a.N) * S;
    const int nn = act ? n : 0;
#pragma unroll
    for (int k = 0; k < KMAX; ++k)
      if (k < K) load_vec_stream<T, S>(v[k], src + (size_t(k) * a.N + nn) * S);
  }
}

// Reduce the per-pattern outer products coef * x[k][i] * v[k][j] over the
// warp, chunk by chunk of 32 values; lane l stores element 32c+l of the
// padded vector.
template <typename T, int S, int KMAX, int VP>
__device__ __forceinline__ void reduce_outer(T *dst, const T (&x)[KMAX][S], const T (&v)[KMAX][S],
                                             T coef, int K, int lane) {
#pragma unroll
  for (int c = 0; c < VP / 32; ++c) {
    T g[32];
#pragma unroll
    for (int jj = 0; jj < 32; ++jj) {
      const int e = c * 32 + jj;
      const int k = e / (S * S);
      const int i = (e / S) % S;
      const int j = e % S;
      g[jj] = (k < KMAX && k < K) ? coef * x[k < KMAX ? k : 0][i] * v[k < KMAX ? k : 0][j] : T(0);
    }
    warp_reduce_halving<32, T>(g, lane);
    dst[c * 32 + lane] = g[0];
  }
}

template <typename T, int S, int KMAX, int TILE, int NSTAGE>
__global__ void __launch_bounds__(TILE) prune_backward_kernel(const PruneArgs<T> a) {
  extern __shared__ __align__(128) unsigned char smem[];
  constexpr int NW = TILE / 32;
  constexpr int VP = ((KMAX * S * S + 31) / 32) * 32;
  constexpr int RV = 2 * VP;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int b = blockIdx.y;
  const int tile = blockIdx.x;
  const int n = tile * TILE + tid;
  const bool act = n < a.N;
  const int K = a.K;
  const int KSS = K * S * S;
  const int RK = S + K;
  const StackLayout L = stack_layout<T>(S, K, a.C, a.slots, TILE, NSTAGE, KMAX, true);
  T *pbuf = reinterpret_cast<T *>(smem + L.pbuf);
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L.bars);
  T *tab = reinterpret_cast<T *>(smem + L.table);
  T *stk = reinterpret_cast<T *>(smem + L.stack);
  T *red = reinterpret_cast<T *>(smem + L.red);
  T *redr = reinterpret_cast<T *>(smem + L.red_root);
  const size_t pstep = 2 * size_t(KSS);
  const T *pm = a.pmat + size_t(b) * a.n_steps * pstep;
  const int nst = a.n_steps;
  const T w = act ? T(a.weights[n]) : T(0);

  if (tid == 0) {
#pragma unroll
    for (int st = 0; st < NSTAGE; ++st) mbar_init(&bars[st], 1);
    fence_barrier_init();
  }
  for (int i = tid; i < a.C * S; i += TILE) tab[i] = a.table[i];
  double props[KMAX], freqs[S];
#pragma unroll
  for (int k = 0; k < KMAX; ++k) props[k] = k < K ? a.props[b * K + k] : 0.0;
#pragma unroll
  for (int i = 0; i < S; ++i) freqs[i] = a.freqs[b * S + i];
  __syncthreads();
  // iteration j handles step nst-1-j and uses stage j % NSTAGE
  if (tid == 0)
    for (int j = 0; j < NSTAGE - 1 && j < nst; ++j) issue_pmat(pbuf, bars, pm, nst - 1 - j, j, pstep);
  bool timed_out = !mbar_wait_bounded(&bars[0], 0, a.timeout_ns);
  if (__syncthreads_or(timed_out)) {
    if (tid == 0) drain_after_timeout<NSTAGE>(bars, 0, min(NSTAGE - 2, nst - 1), a.status);
    return;
  }

  int prev_left = -1, prev_right = -1;
  bool prev_root = false;
  for (int j = 0; j <= nst; ++j) {
    // finish the block reduction of iteration j-1 (its smem writes are
    // visible after the barrier that closed it)
    if (j > 0) {
      const T *rb = red + ((j - 1) & 1) * NW * RV;
      for (int e = tid; e < 2 * KSS; e += TILE) {
        const int side = e >= KSS;
        const int ei = side ? e - KSS : e;
        T acc = T(0);
#pragma unroll
        for (int ww = 0; ww < NW; ++ww) acc += rb[ww * RV + side * VP + ei];
        const int branch = side ? prev_right : prev_left;
        a.gpart[((size_t(b) * a.branch_count + branch) * a.ntiles + tile) * KSS + ei] = acc;
      }
      if (prev_root)
        for (int e = tid; e < RK; e += TILE) {
          T acc = T(0);
#pragma unroll
          for (int ww = 0; ww < NW; ++ww) acc += redr[ww * (S + KMAX) + e];
          a.rootpart[(size_t(b) * a.ntiles + tile) * RK + e] = acc;
        }
    }
    if (j == nst) break;
    const int s = nst - 1 - j;
    if (tid == 0 && j + NSTAGE - 1 < nst) {
      const int jp = j + NSTAGE - 1;
      issue_pmat(pbuf, bars, pm, nst - 1 - jp, jp % NSTAGE, pstep);
    }
    const T *Pl = pbuf + (j % NSTAGE) * pstep;
    const T *Pr = Pl + KSS;
    const int4 r0 = __ldg(a.steps + 3 * s);
    const int4 r1 = __ldg(a.steps + 3 * s + 1);
    const int4 r2 = __ldg(a.steps + 3 * s + 2);
    const int left = r0.y, right = r0.z;
    const int slot_in = r1.z, slot_l = r1.w, slot_r = r2.x;
    const bool is_root = slot_in < 0;

    T vl[KMAX][S], vr[KMAX][S];
    child_values<T, S, KMAX>(vl, left, a, tab, b, n, act);
    child_values<T, S, KMAX>(vr, right, a, tab, b, n, act);
    T xl[KMAX][S], xr[KMAX][S];  // outside partials at the tops of the two branches
    T rg_pi[S], rg_c[KMAX];      // root only: sums for the frequency / weight gradients
#pragma unroll
    for (int i = 0; i < S; ++i) rg_pi[i] = T(0);
#pragma unroll
    for (int k = 0; k < KMAX; ++k) rg_c[k] = T(0);
    T den = T(0);
#pragma unroll
    for (int k = 0; k < KMAX; ++k) {
      if (k < K) {
        T pre[S];
        if (is_root) {
#pragma unroll
          for (int i = 0; i < S; ++i) pre[i] = T(props[k] * freqs[i]);
        } else {
          load_vec<T, S>(pre, stk + (size_t(slot_in * K + k) * TILE + tid) * S);
        }
        T al[S], ar[S];
        matvec<T, S>(al, Pl + k * S * S, vl[k]);
        matvec<T, S>(ar, Pr + k * S * S, vr[k]);
#pragma unroll
        for (int i = 0; i < S; ++i) {
          xl[k][i] = pre[i] * ar[i];
          xr[k][i] = pre[i] * al[i];
          den = fma(xl[k][i], al[i], den);
        }
        if (is_root) {
#pragma unroll
          for (int i = 0; i < S; ++i) {
            const T r = al[i] * ar[i];
            rg_pi[i] = fma(T(props[k]), r, rg_pi[i]);
            rg_c[k] = fma(T(freqs[i]), r, rg_c[k]);
          }
        }
      } else {
#pragma unroll
        for (int i = 0; i < S; ++i) xl[k][i] = xr[k][i] = T(0);
      }
    }
    // dlnL_n/dP = w_n * x (outer) v / L_n; the per-pattern scale of every
    // factor cancels against den, so no scaler bookkeeping is needed.
    const T coef = (act && den > T(0)) ? w / den : T(0);
    T *rw = red + (j & 1) * NW * RV + warp * RV;
    reduce_outer<T, S, KMAX, VP>(rw, xl, vl, coef, K, lane);
    reduce_outer<T, S, KMAX, VP>(rw + VP, xr, vr, coef, K, lane);
    if (is_root) {
      // dlnL/dpi_i = sum_k c_k R[k][i] / L and dlnL/dc_k = sum_i pi_i R[k][i] / L
      // with R = al * ar the root partial (the root's outside vector is c_k pi_i)
#pragma unroll
      for (int i = 0; i < S; ++i) {
        const T acc = warp_sum(coef * rg_pi[i]);
        if (lane == 0) redr[warp * (S + KMAX) + i] = acc;
      }
#pragma unroll
      for (int k = 0; k < KMAX; ++k)
        if (k < K) {
          const T acc = warp_sum(coef * rg_c[k]);
          if (lane == 0) redr[warp * (S + KMAX) + S + k] = acc;
        }
    }
    // outside partials at the bottoms of internal children -> stack
    if (left >= a.tip_count) {
      T o[KMAX][S];
#pragma unroll
      for (int k = 0; k < KMAX; ++k)
        if (k < K) matvec_t<T, S>(o[k], Pl + k * S * S, xl[k]);
      int E = 0;
      rescale_pow2<T, S, KMAX>(o, K, E);
#pragma unroll
      for (int k = 0; k < KMAX; ++k)
        if (k < K) store_vec<T, S>(stk + (size_t(slot_l * K + k) * TILE + tid) * S, o[k]);
    }
    if (right >= a.tip_count) {
      T o[KMAX][S];
#pragma unroll
      for (int k = 0; k < KMAX; ++k)
        if (k < K) matvec_t<T, S>(o[k], Pr + k * S * S, xr[k]);
      int E = 0;
      rescale_pow2<T, S, KMAX>(o, K, E);
#pragma unroll
      for (int k = 0; k < KMAX; ++k)
        if (k < K) store_vec<T, S>(stk + (size_t(slot_r * K + k) * TILE + tid) * S, o[k]);
    }
    prev_left = left;
    prev_right = right;
    prev_root = is_root;
    if (j + 1 < nst)
      timed_out = !mbar_wait_bounded(&bars[(j + 1) % NSTAGE], ((j + 1) / NSTAGE) & 1, a.timeout_ns);
    if (__syncthreads_or(timed_out)) {
      if (tid == 0) drain_after_timeout<NSTAGE>(bars, j + 1, min(j + NSTAGE - 1, nst - 1), a.status);
      return;
    }
  }
}

// ------------------------------------------------------------- reductions
// dlnL/dP[b][branch] = sum over pattern tiles (fixed order, FP64).
template <typename T>
__global__ void reduce_branch_grads_kernel(const T *gpart, double *G, int branch_count, int ntiles,
                                           int kss) {
  const int branch = blockIdx.x, b = blockIdx.y;
  const T *src = gpart + (size_t(b) * branch_count + branch) * ntiles * size_t(kss);
  for (int e = threadIdx.x; e < kss; e += blockDim.x) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    int t = 0;
    for (; t + 4 <= ntiles; t += 4) {
      a0 += double(src[size_t(t) * kss + e]);
      a1 += double(src[size_t(t + 1) * kss + e]);
      a2 += double(src[size_t(t + 2) * kss + e]);
      a3 += double(src[size_t(t + 3) * kss + e]);
    }
    for (; t < ntiles; ++t) a0 += double(src[size_t(t) * kss + e]);
    G[(size_t(b) * branch_count + branch) * kss + e] = (a0 + a1) + (a2 + a3);
  }
}

template <typename T>
__global__ void reduce_root_grads_kernel(const T *rootpart, double *dfreq, double *dprop, int ntiles,
                                         int S, int K) {
  const int b = blockIdx.x;
  const int RK = S + K;
  for (int e = threadIdx.x; e < RK; e += blockDim.x) {
    double acc = 0.0;
    for (int t = 0; t < ntiles; ++t) acc += double(rootpart[(size_t(b) * ntiles + t) * RK + e]);
    if (e < S) {
      if (dfreq) dfreq[b * S + e] = acc;
    } else if (dprop) {
      dprop[b * K + (e - S)] = acc;
    }
  }
}

// lnL[b] = sum over tiles (fixed-order tree reduction).
__global__ void reduce_lnl_kernel(const double *tile_lnl, double *lnl, int ntiles);

}  // namespace tt
