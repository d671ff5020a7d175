// Pattern-tiled pruning kernels.
//
// Patterns are independent up to the final weighted sum
// (torchtree/evolution/tree_likelihood.py:186-221 rescales per pattern), so
// one CTA owns a tile of TILE patterns of one batch sample and walks the
// whole post-order itself; each thread owns one pattern and all K rate
// categories.  Child partials that are still needed live in a shared-memory
// stack whose slots the host assigned (Sethi-Ullman order keeps the depth
// <= log2(T)+1).
//
// Everything a step reads from global memory is staged into a shared-memory
// ring a few steps ahead by the TMA engine (cp.async.bulk, completion on one
// mbarrier per stage): the step record, the pair of transition matrices, the
// tip-code rows of tip children and, in the adjoint, the stored partial
// tiles of internal children.  The warps then read shared memory only.
//
// Forward (replaces tree_likelihood.py:40-75 / 186-221): HBM traffic is the
// write of each non-root internal partial (only when the gradient needs it).
// Adjoint (replaces autograd through the same lines): walks the schedule in
// reverse (a pre-order), keeps the outside partials in the shared-memory
// stack, reads each stored partial once, and reduces dlnL/dP of each branch
// over the tile through a shared-memory transpose.
//
// Global partial layout: [batch][internal node - T][K][N][S], S innermost:
// one category of one tile is a contiguous TILE*S run (one bulk copy).
// Tip codes: [T][code_stride] bytes, rows padded so each tile's run of
// codes is 16-byte aligned.
#pragma once

#include "tt_common.cuh"

namespace tt {

// One post-order step: 12 ints (3 x int4).
//  [0] node [1] left [2] right [3] fwd slot of left (-1: tip)
//  [4] fwd slot of right [5] fwd output slot (-1: root) [6] bwd input slot
//  (-1: root) [7] bwd output slot of left (-1: tip) [8] bwd output slot of
//  right [9] flags of the in-place FP32 adjoint (kTa*) [10] for a node
//  whose outside partial is stored in place: the reversed-walk index of its
//  parent's step (-1 otherwise) [11] unused
constexpr int kStepInts = 12;
// [9]: this node's outside partial was stored in place over its post-order
// tile (else it arrives in registers from the previous step, or is the root);
// the left / right child's outside partial stays in registers for the next
// step (carry) or is stored in place.
// Records of the producer-warp post-order (tt_plan::d_steps_ws): [0] node
// [1] left [2] right [3] [4] stack slot of the left / right child (-1: tip,
// kWsCarry: the child was the previous step and its partial is in registers)
// [5] output slot (-1: root, kWsCarry: the next step is the parent)
constexpr int kWsCarry = -2;
constexpr int kTaPreStored = 1, kTaCarryLeft = 2, kTaCarryRight = 4, kTaStoreLeft = 8, kTaStoreRight = 16;

template <typename T>
struct PruneArgs {
  const int4 *steps;
  const int4 *steps_rev;  // the same records in reverse order (adjoint issue order)
  int n_steps;    // internal nodes (T-1)
  int tip_count;  // T
  int branch_count;
  int N;
  int K;
  int C;  // tip codes in the table
  int slots;
  int rescale;
  int ntiles;
  int code_stride;        // bytes per tip row of `codes` (multiple of 16, >= ntiles*TILE)
  int nstage;             // depth of the staging ring (kernels with a runtime ring depth)
  const uint8_t *codes;   // [T][code_stride]
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
  // records of the producer-warp post-order (kWs* slots), or nullptr
  const int4 *steps_ws = nullptr;
};

// Arguments of one launch over several plans (one kernel parameter block):
// plan i owns CTAs [first[i], first[i+1]) of the 1-D grid, `per_sample[i]`
// of them per batch sample.
constexpr int kMaxMultiPlans = 16;
template <typename T>
struct MultiPrune {
  int count;
  int first[kMaxMultiPlans + 1];
  int per_sample[kMaxMultiPlans];
  PruneArgs<T> a[kMaxMultiPlans];
  __device__ __forceinline__ void locate(int cta, int &pi, int &tile, int &b) const {
    pi = 0;
    while (pi + 1 < count && cta >= first[pi + 1]) ++pi;
    const int r = cta - first[pi];
    b = r / per_sample[pi];
    tile = r - b * per_sample[pi];
  }
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

// Layout of one ring stage: step record | matrix pair | 2 code rows | 2 child tiles
struct StageLayout {
  size_t rec, pm, codes, kids, bytes;
};

template <typename T>
__host__ __device__ inline StageLayout stage_layout(int S, int K, int tile, bool backward) {
  StageLayout g;
  size_t off = 0;
  g.rec = off;
  off = align16(off + 3 * 16);
  g.pm = off;
  off = align16(off + size_t(2) * K * S * S * sizeof(T));
  g.codes = off;
  off = align16(off + size_t(2) * tile);
  g.kids = off;
  if (backward) off = align16(off + size_t(2) * K * tile * S * sizeof(T));
  g.bytes = off;
  return g;
}

struct StackLayout {
  size_t stages, bars, table, stack, xbuf, red, red_root, total;
};

// Shared-memory carve-up shared by the host (launch size) and the kernels.
template <typename T>
__host__ __device__ inline StackLayout stack_layout(int S, int K, int C, int slots, int tile, int nstage,
                                                    int kmax, bool backward) {
  StackLayout L;
  const StageLayout g = stage_layout<T>(S, K, tile, backward);
  size_t off = 0;
  L.stages = off;
  off = align16(off + size_t(nstage) * g.bytes);
  L.bars = off;
  off = align16(off + size_t(nstage) * 8);
  L.table = off;
  off = align16(off + size_t(C) * S * sizeof(T));
  L.stack = off;
  off = align16(off + size_t(slots) * K * tile * S * sizeof(T));
  L.xbuf = off;
  if (backward) off = align16(off + size_t(2) * tile * (K * S + 16 / sizeof(T)) * sizeof(T));
  L.red = off;
  // per-row partial sums of the transpose reduction, double-buffered
  const int rows = 2 * K * S;
  const int q = tile >= rows ? tile / rows : 1;
  if (backward) off = align16(off + size_t(2) * rows * q * S * sizeof(T));
  L.red_root = off;
  if (backward) off = align16(off + size_t(tile / 32) * (S + kmax) * sizeof(T));
  L.total = off;
  (void)kmax;
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

// Producer side of the ring (one thread): stage everything step `s` needs.
// `rec` is the step's record (already loaded by the caller).
template <typename T, int S, bool BACKWARD>
__device__ __forceinline__ void issue_step(const PruneArgs<T> &a, unsigned char *stage, uint64_t *bar,
                                           const int4 (&rec)[3], int s, int b, int tile, int TILE,
                                           const StageLayout &g) {
  const int K = a.K;
  const size_t kss = size_t(K) * S * S;
  int4 *r = reinterpret_cast<int4 *>(stage + g.rec);
  r[0] = rec[0];
  r[1] = rec[1];
  r[2] = rec[2];
  const int left = rec[0].y, right = rec[0].z;
  const int rem = min(TILE, a.N - tile * TILE);
  const uint32_t pbytes = uint32_t(2 * kss * sizeof(T));
  const uint32_t kid_bytes = uint32_t(rem) * S * sizeof(T);
  uint32_t total = pbytes;
  total += (left < a.tip_count ? TILE : 0) + (right < a.tip_count ? TILE : 0);
  if (BACKWARD) total += (left >= a.tip_count ? K * kid_bytes : 0) + (right >= a.tip_count ? K * kid_bytes : 0);
  mbar_arrive_expect_tx(bar, total);
  bulk_copy_g2s(stage + g.pm, a.pmat + (size_t(b) * a.n_steps + s) * 2 * kss, pbytes, bar);
  const int child[2] = {left, right};
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    if (child[c] < a.tip_count) {
      bulk_copy_g2s(stage + g.codes + c * TILE, a.codes + size_t(child[c]) * a.code_stride + size_t(tile) * TILE,
                    uint32_t(TILE), bar);
    } else if (BACKWARD) {
      const T *src = a.partials +
                     ((size_t(b) * (a.n_steps - 1) + (child[c] - a.tip_count)) * K) * size_t(a.N) * S +
                     size_t(tile) * TILE * S;
      T *dst = reinterpret_cast<T *>(stage + g.kids) + size_t(c) * K * TILE * S;
      for (int k = 0; k < K; ++k) bulk_copy_g2s(dst + size_t(k) * TILE * S, src + size_t(k) * a.N * S, kid_bytes, bar);
    }
  }
}

// On a timeout: record it, then give in-flight copies a bounded chance to
// land before the CTA exits.
template <int NSTAGE>
__device__ __forceinline__ void drain_after_timeout(uint64_t *bars, int first, int last, int *status) {
  atomicExch(status, kDeviceTimeout);
  for (int j = first; j <= last; ++j) mbar_wait_bounded(&bars[j % NSTAGE], (j / NSTAGE) & 1, 100000000ull);
}

__device__ __forceinline__ void load_rec(int4 (&r)[3], const int4 *steps, int s) {
  r[0] = __ldg(steps + 3 * s);
  r[1] = __ldg(steps + 3 * s + 1);
  r[2] = __ldg(steps + 3 * s + 2);
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
  const int nst = a.n_steps;
  const StackLayout L = stack_layout<T>(S, K, a.C, a.slots, TILE, NSTAGE, KMAX, false);
  const StageLayout G = stage_layout<T>(S, K, TILE, false);
  unsigned char *stages = smem + L.stages;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L.bars);
  T *tab = reinterpret_cast<T *>(smem + L.table);
  T *stk = reinterpret_cast<T *>(smem + L.stack);

  int4 nxt[3];  // producer's prefetched record (thread 0)
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
  if (tid == 0) {
    load_rec(nxt, a.steps, 0);
    for (int s = 0; s < NSTAGE - 1 && s < nst; ++s) {
      int4 cur[3] = {nxt[0], nxt[1], nxt[2]};
      if (s + 1 < nst) load_rec(nxt, a.steps, s + 1);
      issue_step<T, S, false>(a, stages + s * G.bytes, &bars[s], cur, s, b, tile, TILE, G);
    }
  }
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
      int4 cur[3] = {nxt[0], nxt[1], nxt[2]};
      if (sp + 1 < nst) load_rec(nxt, a.steps, sp + 1);
      issue_step<T, S, false>(a, stages + (sp % NSTAGE) * G.bytes, &bars[sp % NSTAGE], cur, sp, b, tile, TILE, G);
    }
    const unsigned char *stg = stages + (s % NSTAGE) * G.bytes;
    const int4 *rec = reinterpret_cast<const int4 *>(stg + G.rec);
    const int4 r0 = rec[0], r1 = rec[1];
    const int node = r0.x, left = r0.y, right = r0.z;
    const bool ltip = left < a.tip_count, rtip = right < a.tip_count;
    const T *Pl = reinterpret_cast<const T *>(stg + G.pm);
    const T *Pr = Pl + K * S * S;
    T tl[S], tr[S];
    if (ltip) load_vec<T, S>(tl, tab + int(stg[G.codes + tid]) * S);
    if (rtip) load_vec<T, S>(tr, tab + int(stg[G.codes + TILE + tid]) * S);
    T prod[KMAX][S];
#pragma unroll
    for (int k = 0; k < KMAX; ++k) {
      if (k < K) {
        T vl[S], vr[S], al[S], ar[S];
        if (ltip) {
#pragma unroll
          for (int i = 0; i < S; ++i) vl[i] = tl[i];
        } else {
          load_vec<T, S>(vl, stk + (size_t(r0.w * K + k) * TILE + tid) * S);
        }
        if (rtip) {
#pragma unroll
          for (int i = 0; i < S; ++i) vr[i] = tr[i];
        } else {
          load_vec<T, S>(vr, stk + (size_t(r1.x * K + k) * TILE + tid) * S);
        }
        matvec<T, S>(al, Pl + k * S * S, vl);
        matvec<T, S>(ar, Pr + k * S * S, vr);
#pragma unroll
        for (int i = 0; i < S; ++i) prod[k][i] = al[i] * ar[i];
      } else {
#pragma unroll
        for (int i = 0; i < S; ++i) prod[k][i] = T(0);
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
    if (s + 1 < nst)
      timed_out = !mbar_wait_bounded(&bars[(s + 1) % NSTAGE], ((s + 1) / NSTAGE) & 1, a.timeout_ns);
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
template <typename T, int S, int KMAX, int TILE, int NSTAGE>
__global__ void __launch_bounds__(TILE) prune_backward_kernel(const PruneArgs<T> a) {
  extern __shared__ __align__(128) unsigned char smem[];
  constexpr int NW = TILE / 32;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int b = blockIdx.y;
  const int tile = blockIdx.x;
  const int n = tile * TILE + tid;
  const bool act = n < a.N;
  const int rem = min(TILE, a.N - tile * TILE);
  const int K = a.K;
  const int KS = K * S;
  const int KSS = K * S * S;
  const int RK = S + K;
  const int XS = KS + 16 / int(sizeof(T));  // padded row: conflict-free vector stores
  const int nst = a.n_steps;
  const StackLayout L = stack_layout<T>(S, K, a.C, a.slots, TILE, NSTAGE, KMAX, true);
  const StageLayout G = stage_layout<T>(S, K, TILE, true);
  unsigned char *stages = smem + L.stages;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L.bars);
  T *tab = reinterpret_cast<T *>(smem + L.table);
  T *stk = reinterpret_cast<T *>(smem + L.stack);
  T *xbuf = reinterpret_cast<T *>(smem + L.xbuf);  // [2][TILE][XS]  coef * outside partial
  T *red = reinterpret_cast<T *>(smem + L.red);    // [2][rows][Q][S]
  T *redr = reinterpret_cast<T *>(smem + L.red_root);
  // transpose-reduction work split: rows (child, k, i), Q pattern chunks
  const int rows = 2 * KS;
  const int Q = TILE >= rows ? TILE / rows : 1;
  const int chunk = (TILE + Q - 1) / Q;
  const T w = act ? T(a.weights[n]) : T(0);

  int4 nxt[3];
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
  if (tid == 0) {
    load_rec(nxt, a.steps, nst - 1);
    for (int j = 0; j < NSTAGE - 1 && j < nst; ++j) {
      int4 cur[3] = {nxt[0], nxt[1], nxt[2]};
      if (j + 1 < nst) load_rec(nxt, a.steps, nst - 2 - j);
      issue_step<T, S, true>(a, stages + j * G.bytes, &bars[j], cur, nst - 1 - j, b, tile, TILE, G);
    }
  }
  bool timed_out = !mbar_wait_bounded(&bars[0], 0, a.timeout_ns);
  if (__syncthreads_or(timed_out)) {
    if (tid == 0) drain_after_timeout<NSTAGE>(bars, 0, min(NSTAGE - 2, nst - 1), a.status);
    return;
  }

  int prev_left = -1, prev_right = -1;
  for (int j = 0; j <= nst; ++j) {
    // finish the transpose reduction of iteration j-1 (published by the barrier that closed it)
    if (j > 0) {
      const T *rb = red + size_t((j - 1) & 1) * rows * Q * S;
      for (int e = tid; e < 2 * KSS; e += TILE) {
        const int side = e >= KSS;
        const int ei = side ? e - KSS : e;  // (k, i, jj) of this child
        const int row = side * KS + ei / S;
        const int jj = ei % S;
        T acc = T(0);
        for (int q = 0; q < Q; ++q) acc += rb[(row * Q + q) * S + jj];
        const int branch = side ? prev_right : prev_left;
        a.gpart[((size_t(b) * a.branch_count + branch) * a.ntiles + tile) * KSS + ei] = acc;
      }
    }
    if (j == nst) break;
    if (tid == 0 && j + NSTAGE - 1 < nst) {
      const int jp = j + NSTAGE - 1;
      int4 cur[3] = {nxt[0], nxt[1], nxt[2]};
      if (jp + 1 < nst) load_rec(nxt, a.steps, nst - 2 - jp);
      issue_step<T, S, true>(a, stages + (jp % NSTAGE) * G.bytes, &bars[jp % NSTAGE], cur, nst - 1 - jp, b,
                             tile, TILE, G);
    }
    const unsigned char *stg = stages + (j % NSTAGE) * G.bytes;
    const int4 *rec = reinterpret_cast<const int4 *>(stg + G.rec);
    const int4 r0 = rec[0], r1 = rec[1], r2 = rec[2];
    const int left = r0.y, right = r0.z;
    const int slot_in = r1.z, slot_l = r1.w, slot_r = r2.x;
    const bool is_root = slot_in < 0;
    const bool ltip = left < a.tip_count, rtip = right < a.tip_count;
    const T *Pl = reinterpret_cast<const T *>(stg + G.pm);
    const T *Pr = Pl + KSS;
    const T *kidl = reinterpret_cast<const T *>(stg + G.kids);
    const T *kidr = kidl + size_t(K) * TILE * S;
    T tl[S], tr[S];
    if (ltip) load_vec<T, S>(tl, tab + int(stg[G.codes + tid]) * S);
    if (rtip) load_vec<T, S>(tr, tab + int(stg[G.codes + TILE + tid]) * S);

    // ---- phase A: per pattern, all categories
    T xl[KMAX][S], xr[KMAX][S];  // outside partials at the tops of the two branches
    T ol[KMAX][S], orr[KMAX][S];  // outside partials at the bottoms of the children
    T rg_pi[S], rg_c[KMAX];
#pragma unroll
    for (int i = 0; i < S; ++i) rg_pi[i] = T(0);
    T den = T(0);
#pragma unroll
    for (int k = 0; k < KMAX; ++k) {
      rg_c[k] = T(0);
      if (k < K) {
        T pre[S], vl[S], vr[S], al[S], ar[S];
        if (is_root) {
#pragma unroll
          for (int i = 0; i < S; ++i) pre[i] = T(props[k] * freqs[i]);
        } else {
          load_vec<T, S>(pre, stk + (size_t(slot_in * K + k) * TILE + tid) * S);
        }
        if (ltip) {
#pragma unroll
          for (int i = 0; i < S; ++i) vl[i] = tl[i];
        } else {
          load_vec<T, S>(vl, kidl + (size_t(k) * TILE + tid) * S);
        }
        if (rtip) {
#pragma unroll
          for (int i = 0; i < S; ++i) vr[i] = tr[i];
        } else {
          load_vec<T, S>(vr, kidr + (size_t(k) * TILE + tid) * S);
        }
        T pl[S][S], pr[S][S];  // this category's two matrices, read once
#pragma unroll
        for (int i = 0; i < S; ++i) {
          load_vec<T, S>(pl[i], Pl + (k * S + i) * S);
          load_vec<T, S>(pr[i], Pr + (k * S + i) * S);
        }
#pragma unroll
        for (int i = 0; i < S; ++i) {
          T sa = T(0), sb = T(0);
#pragma unroll
          for (int jj = 0; jj < S; ++jj) {
            sa = fma(pl[i][jj], vl[jj], sa);
            sb = fma(pr[i][jj], vr[jj], sb);
          }
          al[i] = sa;
          ar[i] = sb;
        }
#pragma unroll
        for (int i = 0; i < S; ++i) {
          xl[k][i] = pre[i] * ar[i];
          xr[k][i] = pre[i] * al[i];
          den = fma(xl[k][i], al[i], den);
          if (is_root) {
            const T r = al[i] * ar[i];
            rg_pi[i] = fma(T(props[k]), r, rg_pi[i]);
            rg_c[k] = fma(T(freqs[i]), r, rg_c[k]);
          }
        }
        // outside partials of the children (scale-free: no coefficient)
#pragma unroll
        for (int jj = 0; jj < S; ++jj) {
          T sa = T(0), sb = T(0);
#pragma unroll
          for (int i = 0; i < S; ++i) {
            sa = fma(pl[i][jj], xl[k][i], sa);
            sb = fma(pr[i][jj], xr[k][i], sb);
          }
          ol[k][jj] = sa;
          orr[k][jj] = sb;
        }
      } else {
#pragma unroll
        for (int i = 0; i < S; ++i) xl[k][i] = xr[k][i] = ol[k][i] = orr[k][i] = T(0);
      }
    }
    // dlnL_n/dP = w_n * x (outer) v / L_n; every factor's per-pattern scale
    // cancels against den, so no scaler bookkeeping is needed.
    const T coef = (act && den > T(0)) ? w / den : T(0);
    {
      T *xl_dst = xbuf + size_t(tid) * XS;
      T *xr_dst = xbuf + size_t(TILE + tid) * XS;
#pragma unroll
      for (int k = 0; k < KMAX; ++k)
        if (k < K) {
          T u[S], v[S];
#pragma unroll
          for (int i = 0; i < S; ++i) {
            u[i] = coef * xl[k][i];
            v[i] = coef * xr[k][i];
          }
          store_vec<T, S>(xl_dst + k * S, u);
          store_vec<T, S>(xr_dst + k * S, v);
        }
    }
    if (is_root) {
#pragma unroll
      for (int i = 0; i < S; ++i) {  // lanes past the last pattern hold stale data: mask them
        const T acc = warp_sum(act ? coef * rg_pi[i] : T(0));
        if (lane == 0) redr[warp * (S + KMAX) + i] = acc;
      }
#pragma unroll
      for (int k = 0; k < KMAX; ++k)
        if (k < K) {
          const T acc = warp_sum(act ? coef * rg_c[k] : T(0));
          if (lane == 0) redr[warp * (S + KMAX) + S + k] = acc;
        }
    }
    if (!ltip) {
      int E = 0;
      rescale_pow2<T, S, KMAX>(ol, K, E);
#pragma unroll
      for (int k = 0; k < KMAX; ++k)
        if (k < K) store_vec<T, S>(stk + (size_t(slot_l * K + k) * TILE + tid) * S, ol[k]);
    }
    if (!rtip) {
      int E = 0;
      rescale_pow2<T, S, KMAX>(orr, K, E);
#pragma unroll
      for (int k = 0; k < KMAX; ++k)
        if (k < K) store_vec<T, S>(stk + (size_t(slot_r * K + k) * TILE + tid) * S, orr[k]);
    }
    __syncthreads();  // xbuf complete

    // ---- phase C: G[c][k][i][:] = sum_n xbuf[c][n][k,i] * v_c[k][n][:]
    {
      T *rw = red + size_t(j & 1) * rows * Q * S;
      for (int item = tid; item < rows * Q; item += TILE) {
        const int row = item / Q, q = item % Q;
        const int c = row >= KS;
        const int ki = c ? row - KS : row;
        const int k = ki / S;
        const bool tipc = c ? rtip : ltip;
        const T *xs = xbuf + size_t(c) * TILE * XS + ki;
        const T *vs = (c ? kidr : kidl) + size_t(k) * TILE * S;
        const unsigned char *cs = stg + G.codes + c * TILE;
        T acc[S];
#pragma unroll
        for (int jj = 0; jj < S; ++jj) acc[jj] = T(0);
        const int n0 = q * chunk, n1 = min(n0 + chunk, rem);
        for (int m = n0; m < n1; ++m) {
          const T x = xs[size_t(m) * XS];
          T v[S];
          load_vec<T, S>(v, tipc ? tab + int(cs[m]) * S : vs + size_t(m) * S);
#pragma unroll
          for (int jj = 0; jj < S; ++jj) acc[jj] = fma(x, v[jj], acc[jj]);
        }
        store_vec<T, S>(rw + (size_t(row) * Q + q) * S, acc);
      }
    }
    prev_left = left;
    prev_right = right;
    if (j + 1 < nst)
      timed_out = !mbar_wait_bounded(&bars[(j + 1) % NSTAGE], ((j + 1) / NSTAGE) & 1, a.timeout_ns);
    if (__syncthreads_or(timed_out)) {
      if (tid == 0) drain_after_timeout<NSTAGE>(bars, j + 1, min(j + NSTAGE - 1, nst - 1), a.status);
      return;
    }
    if (is_root)
      for (int e = tid; e < RK; e += TILE) {
        T acc = T(0);
#pragma unroll
        for (int ww = 0; ww < NW; ++ww) acc += redr[ww * (S + KMAX) + e];
        a.rootpart[(size_t(b) * a.ntiles + tile) * RK + e] = acc;
      }
  }
}

// ------------------------------------------------------------- reductions
// dlnL/dP[b][branch] = sum over pattern tiles (fixed order, FP64).
template <typename T>
__global__ void reduce_branch_grads_kernel(const T *gpart, double *G, int branch_count, int ntiles, int kss,
                                           int accumulate) {
  const int branch = blockIdx.x, b = blockIdx.y;
  const T *src = gpart + (size_t(b) * branch_count + branch) * ntiles * size_t(kss);
  for (int e = threadIdx.x; e < kss; e += blockDim.x) {
    // blocks of 8 tiles are summed at T precision (4 independent chains), the
    // block sums in FP64: few FP64 operations, fixed order
    double acc = 0.0;
    int t = 0;
    for (; t + 8 <= ntiles; t += 8) {
      const T *q = src + size_t(t) * kss + e;
      const T s0 = q[0] + q[size_t(4) * kss], s1 = q[size_t(kss)] + q[size_t(5) * kss];
      const T s2 = q[size_t(2) * kss] + q[size_t(6) * kss], s3 = q[size_t(3) * kss] + q[size_t(7) * kss];
      acc += double((s0 + s1) + (s2 + s3));
    }
    for (; t < ntiles; ++t) acc += double(src[size_t(t) * kss + e]);
    double *g = G + (size_t(b) * branch_count + branch) * kss + e;
    *g = accumulate ? *g + acc : acc;
  }
}

template <typename T>
__global__ void reduce_root_grads_kernel(const T *rootpart, double *dfreq, double *dprop, int ntiles, int S,
                                         int K, int accumulate) {
  const int b = blockIdx.x;
  const int RK = S + K;
  for (int e = threadIdx.x; e < RK; e += blockDim.x) {
    double acc = 0.0;
    for (int t = 0; t < ntiles; ++t) acc += double(rootpart[(size_t(b) * ntiles + t) * RK + e]);
    if (e < S) {
      if (dfreq) dfreq[b * S + e] = accumulate ? dfreq[b * S + e] + acc : acc;
    } else if (dprop) {
      double *d = dprop + b * K + (e - S);
      *d = accumulate ? *d + acc : acc;
    }
  }
}

// lnL[b] = sum over tiles (fixed-order tree reduction).
__global__ void reduce_lnl_kernel(const double *tile_lnl, double *lnl, int ntiles, int accumulate);

}  // namespace tt
