// FP32 pruning kernels on packed FP32x2 arithmetic (sm_100+ FFMA2).
//
// Algorithm as in tt_prune.cuh: one CTA walks the whole post-order for a
// tile of P patterns of one batch sample; child partials that are still
// needed live in a shared-memory stack (host-assigned slots, depth
// <= log2(T)+1); the step record, the transition matrices and the tip-code
// rows (and, in the adjoint, the stored child tiles) are staged into a
// shared-memory ring by the TMA engine a few steps ahead.
//
// Mapping: one thread per pattern (R patterns per thread), all categories in
// the thread.  A pattern's vector is stored [state j][category k] with the K
// categories padded to an even KE = 2*KQ, so every matrix-vector product
// works on category pairs with FFMA2: (a_k, a_k') += (P_k[i][j], P_k'[i][j])
// * (v_k[j], v_k'[j]).  All threads read the same matrices (shared-memory
// broadcast), and the per-node maximum / the adjoint's denominator are
// in-thread reductions.
//
// Layouts (FP32 plans):
//   matrices  [batch][step][side][KQ][4][4] float2 pairs (categories 2q, 2q+1;
//             padded categories are zero)
//   partials  [batch][internal node - T][tile][pair q][state j][P] float2:
//             one tile of one node is a contiguous run (one bulk copy), and
//             a (pair, state) row over the tile's patterns is contiguous, so
//             every warp access to a staged tile is conflict-free.  The
//             shared-memory stack keeps [chunk][P] float4 (each thread only
//             touches its own patterns there).
//   table     [code][4] float2: each tip value duplicated for a category pair
#pragma once

#include "tt_common.cuh"
#include "tt_prune.cuh"

namespace tt {

// ---------------------------------------------------------------- layouts
struct TlStage {
  int rec, pm, codes, kids, bytes;
};

// KQ category pairs, P patterns per tile
__host__ __device__ inline TlStage tl_stage(int KQ, int P, bool backward) {
  TlStage g;
  int off = 0;
  g.rec = off;
  off = int(align16(off + 48));
  g.pm = off;
  off = int(align16(off + 2 * KQ * 16 * 8));
  g.codes = off;
  off = int(align16(off + 2 * P));
  g.kids = off;
  if (backward) off = int(align16(off + 2 * P * KQ * 2 * 16));  // 2 children x NC chunks x P x 16 B
  g.bytes = off;
  return g;
}

struct TlLayout {
  int stages, bars, recs, table, onehot, stack, xbuf, red, red_root, total;
};

constexpr int kTlRecChunk = 32;
// CTAs per SM the producer-warp post-order's register budget is sized for:
// six fit the shared memory of up to two category pairs
__host__ __device__ constexpr int tl_ws_min_blocks(int KQ, int NT) { return KQ <= 2 ? (NT <= 64 ? 6 : 4) : 1; }
// width of a stored post-order tile (patterns); the producer-warp post-order
// may walk several tiles of one sample in one CTA
constexpr int kTlPartTile = 64;


// red2: float2 partial-block elements per thread of the adjoint's pattern reduction
__host__ __device__ inline TlLayout tl_layout(int KQ, int C, int slots, int P, int NT, int nstage, bool backward,
                                              int red2 = 16) {
  TlLayout L;
  const TlStage g = tl_stage(KQ, P, backward);
  const int vbytes = 2 * KQ * 4 * 4;  // bytes of one pattern vector (4 states x 2KQ categories)
  int off = 0;
  L.stages = off;
  off = int(align16(off + nstage * g.bytes));
  L.bars = off;
  off = int(align16(off + (nstage + 2) * 8));
  L.recs = off;
  off = int(align16(off + 2 * kTlRecChunk * 48));
  L.table = off;
  off = int(align16(off + C * 32));
  L.onehot = off;
  off = int(align16(off + C));
  L.stack = off;
  off = int(align16(off + slots * P * vbytes));
  L.xbuf = off;
  if (backward) off = int(align16(off + 2 * P * vbytes));
  L.red = off;
  if (backward) off = int(align16(off + red2 * (NT + 1) * 8));  // red2 float2 per thread, [red2][NT+1]
  L.red_root = off;
  if (backward) off = int(align16(off + (NT / 32) * 12 * 4));
  L.total = off;
  return L;
}

// ------------------------------------------------------------ record ring
// Producer-side ring of step records (one thread): records are bulk-copied in
// chunks of CH into two shared-memory slots one chunk ahead; `steps` is in
// issue order.
template <int CH>
struct TlRecRingT {
  int4 *recs;
  uint64_t *bars;
  const int4 *steps;
  int count;
  unsigned long long timeout;
  __device__ __forceinline__ void load_chunk(int c) const {
    if (c * CH >= count) return;
    const int n = min(CH, count - c * CH);
    const uint32_t bytes = uint32_t(n) * 48;
    mbar_arrive_expect_tx(&bars[c & 1], bytes);
    bulk_copy_g2s(recs + (c & 1) * CH * 3, steps + size_t(c) * CH * 3, bytes, &bars[c & 1]);
  }
  __device__ __forceinline__ bool get(int i, int4 (&r)[3]) const {
    const int c = i / CH, o = i - c * CH;
    if (o == 0 && !mbar_wait_bounded(&bars[c & 1], (c >> 1) & 1, timeout)) return false;
    const int4 *src = recs + ((c & 1) * CH + o) * 3;
    r[0] = src[0];
    r[1] = src[1];
    r[2] = src[2];
    if (o == CH - 1) {  // slot free again: order the reads before the refill
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      load_chunk(c + 2);
    }
    return true;
  }
  __device__ __forceinline__ void drain(int next_issue) const {
    const int c = next_issue / CH;
    for (int d = 0; d < 2; ++d)
      if ((c + d) * CH < count) mbar_wait_bounded(&bars[(c + d) & 1], ((c + d) >> 1) & 1, 100000000ull);
  }
};
using TlRecRing = TlRecRingT<kTlRecChunk>;

// Stage step s of tile `tile`: record, matrix pairs, code rows of tip
// children and (adjoint) the stored tiles of internal children.
template <bool BACKWARD>
__device__ __forceinline__ void tl_issue(const PruneArgs<float> &a, int KQ, unsigned char *stage, uint64_t *bar,
                                         const int4 (&rec)[3], int s, int b, int tile, int P, const TlStage &g) {
  int4 *r = reinterpret_cast<int4 *>(stage + g.rec);
  r[0] = rec[0];
  r[1] = rec[1];
  r[2] = rec[2];
  const int left = rec[0].y, right = rec[0].z;
  const uint32_t pbytes = uint32_t(2 * KQ * 16 * 8);
  const uint32_t tile_bytes = uint32_t(P) * KQ * 2 * 16;
  uint32_t total = pbytes + (left < a.tip_count ? P : 0) + (right < a.tip_count ? P : 0);
  if (BACKWARD) total += (left >= a.tip_count ? tile_bytes : 0) + (right >= a.tip_count ? tile_bytes : 0);
  mbar_arrive_expect_tx(bar, total);
  bulk_copy_g2s(stage + g.pm, a.pmat + (size_t(b) * a.n_steps + s) * 2 * KQ * 32, pbytes, bar);
  const int child[2] = {left, right};
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    if (child[c] < a.tip_count) {
      bulk_copy_g2s(stage + g.codes + c * P, a.codes + size_t(child[c]) * a.code_stride + size_t(tile) * P,
                    uint32_t(P), bar);
    } else if (BACKWARD) {
      const float *src = a.partials + ((size_t(b) * (a.n_steps - 1) + (child[c] - a.tip_count)) * a.ntiles + tile) *
                                          size_t(P) * KQ * 8;
      bulk_copy_g2s(stage + g.kids + c * int(tile_bytes), src, tile_bytes, bar);
    }
  }
}

__device__ __forceinline__ void tl_drain(int nstage, uint64_t *bars, int first, int last, int *status) {
  atomicExch(status, kDeviceTimeout);
  for (int j = first; j <= last; ++j) mbar_wait_bounded(&bars[j % nstage], (j / nstage) & 1, 100000000ull);
}

// ------------------------------------------------------------ vector math
// A pattern vector: v[j][q] = (value of category 2q, category 2q+1) at state j.
template <int KQ>
struct Vec {
  float2 v[4][KQ];
};

// chunk c (float4) of a pattern vector holds floats [4c, 4c+4) of [j][k]:
// state j = (4c) / KE, categories 4c % KE .. +3, i.e. two pairs.
template <int KQ>
__device__ __forceinline__ void vec_load(Vec<KQ> &x, const float4 *base, int stride) {
#pragma unroll
  for (int c = 0; c < KQ * 2; ++c) {
    const float4 f = base[c * stride];
    const int e = 4 * c;  // float index of the chunk
    const int j = e / (2 * KQ), q = (e % (2 * KQ)) / 2;
    x.v[j][q] = make_float2(f.x, f.y);
    if (KQ > 1) {
      x.v[(e + 2) / (2 * KQ)][((e + 2) % (2 * KQ)) / 2] = make_float2(f.z, f.w);
    } else {  // KQ == 1: a chunk spans states j and j+1
      x.v[j + 1][0] = make_float2(f.z, f.w);
    }
  }
}

template <int KQ>
__device__ __forceinline__ void vec_store(float4 *base, int stride, const Vec<KQ> &x) {
#pragma unroll
  for (int c = 0; c < KQ * 2; ++c) {
    const int e = 4 * c;
    const int j = e / (2 * KQ), q = (e % (2 * KQ)) / 2;
    const float2 lo = x.v[j][q];
    const float2 hi = KQ > 1 ? x.v[(e + 2) / (2 * KQ)][((e + 2) % (2 * KQ)) / 2] : x.v[j + 1][0];
    base[c * stride] = make_float4(lo.x, lo.y, hi.x, hi.y);
  }
}

template <int KQ>
__device__ __forceinline__ void vec_store_stream(float4 *base, int stride, const Vec<KQ> &x) {
#pragma unroll
  for (int c = 0; c < KQ * 2; ++c) {
    const int e = 4 * c;
    const int j = e / (2 * KQ), q = (e % (2 * KQ)) / 2;
    const float2 lo = x.v[j][q];
    const float2 hi = KQ > 1 ? x.v[(e + 2) / (2 * KQ)][((e + 2) % (2 * KQ)) / 2] : x.v[j + 1][0];
    __stcs(base + size_t(c) * stride, make_float4(lo.x, lo.y, hi.x, hi.y));
  }
}

// Tiles in HBM, the adjoint's staged child tiles and its x buffer use the
// pair-major layout [pair q][state j][pattern p] float2 (a pattern's vector
// is 4 KQ float2 strided by P), so the pattern reduction's reads of one
// (pair, state) row over consecutive patterns are contiguous.
template <int KQ>
__device__ __forceinline__ void vec_load_pm(Vec<KQ> &x, const float2 *base, int p, int P) {
#pragma unroll
  for (int q = 0; q < KQ; ++q)
#pragma unroll
    for (int j = 0; j < 4; ++j) x.v[j][q] = base[(q * 4 + j) * P + p];
}

template <int KQ>
__device__ __forceinline__ void vec_store_pm(float2 *base, int p, int P, const Vec<KQ> &x) {
#pragma unroll
  for (int q = 0; q < KQ; ++q)
#pragma unroll
    for (int j = 0; j < 4; ++j) base[(q * 4 + j) * P + p] = x.v[j][q];
}

template <int KQ>
__device__ __forceinline__ void vec_store_pm_stream(float2 *base, int p, int P, const Vec<KQ> &x) {
#pragma unroll
  for (int q = 0; q < KQ; ++q)
#pragma unroll
    for (int j = 0; j < 4; ++j) __stcs(base + (q * 4 + j) * P + p, x.v[j][q]);
}

// tip vector: the table row duplicated over every category pair
template <int KQ>
__device__ __forceinline__ void vec_tip(Vec<KQ> &x, const float2 *tab2, int code) {
  const float4 a = reinterpret_cast<const float4 *>(tab2)[code * 2];
  const float4 c = reinterpret_cast<const float4 *>(tab2)[code * 2 + 1];
#pragma unroll
  for (int q = 0; q < KQ; ++q) {
    x.v[0][q] = make_float2(a.x, a.y);
    x.v[1][q] = make_float2(a.z, a.w);
    x.v[2][q] = make_float2(c.x, c.y);
    x.v[3][q] = make_float2(c.z, c.w);
  }
}

// pm: the KQ pair-matrices of one side, [q][i][j] float2
// out[i][q] = sum_j P_q[i][j] * in[j][q]
template <int KQ>
__device__ __forceinline__ void mat_vec(Vec<KQ> &out, const float2 *pm, const Vec<KQ> &in) {
#pragma unroll
  for (int q = 0; q < KQ; ++q) {
    float2 p[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float4 r0 = reinterpret_cast<const float4 *>(pm + (q * 4 + i) * 4)[0];
      const float4 r1 = reinterpret_cast<const float4 *>(pm + (q * 4 + i) * 4)[1];
      p[i][0] = make_float2(r0.x, r0.y);
      p[i][1] = make_float2(r0.z, r0.w);
      p[i][2] = make_float2(r1.x, r1.y);
      p[i][3] = make_float2(r1.z, r1.w);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      float2 acc = __fmul2_rn(p[i][0], in.v[0][q]);
      acc = __ffma2_rn(p[i][1], in.v[1][q], acc);
      acc = __ffma2_rn(p[i][2], in.v[2][q], acc);
      out.v[i][q] = __ffma2_rn(p[i][3], in.v[3][q], acc);
    }
  }
}

// State of a one-hot code-table row (exactly one 1 and zeros elsewhere), or
// -1: a tip with such a code contributes the column P[.][s] of each matrix.
template <typename TT>
__device__ __forceinline__ signed char onehot_state(const TT *table, int code) {
  int s = -1, ones = 0;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const TT v = table[code * 4 + j];
    if (v == TT(1)) {
      s = j;
      ++ones;
    } else if (v != TT(0)) {
      return -1;
    }
  }
  return ones == 1 ? static_cast<signed char>(s) : -1;
}

// out[i][q] = P_q[i][s]: the matrix-vector product with the unit vector e_s
template <int KQ>
__device__ __forceinline__ void mat_col(Vec<KQ> &out, const float2 *pm, int s) {
#pragma unroll
  for (int q = 0; q < KQ; ++q)
#pragma unroll
    for (int i = 0; i < 4; ++i) out.v[i][q] = pm[(q * 4 + i) * 4 + s];
}

template <int KQ>
__device__ __forceinline__ float vec_max(const Vec<KQ> &x) {
  // pairwise tree (the maximum is exact in any order): short dependency chains
  float m[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    m[j] = fmaxf(x.v[j][0].x, x.v[j][0].y);
#pragma unroll
    for (int q = 1; q < KQ; ++q) m[j] = fmaxf(m[j], fmaxf(x.v[j][q].x, x.v[j][q].y));
  }
  return fmaxf(fmaxf(fmaxf(m[0], m[1]), fmaxf(m[2], m[3])), 0.0f);
}

// exact power-of-two rescale: multiply by 2^-e with e = floor(log2(max)) for a
// normal maximum (a zero, subnormal or non-finite maximum leaves the vector as
// it is); E accumulates the exponents.
template <int KQ>
__device__ __forceinline__ void vec_rescale(Vec<KQ> &x, int &E) {
  const float m = vec_max(x);
  const int be = (__float_as_int(m) >> 23) & 0xff;
  const int e = (be == 0 || be == 0xff) ? 0 : min(be - 127, 126);
  const float f = __int_as_float((127 - e) << 23);
  const float2 f2 = make_float2(f, f);
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int q = 0; q < KQ; ++q) x.v[j][q] = __fmul2_rn(x.v[j][q], f2);
  E += e;
}

// ------------------------------------------------------------------ forward
template <int KQ, int NT, int R>
__global__ void __launch_bounds__(NT) tl_forward_kernel(const PruneArgs<float> a) {
  constexpr int P = NT * R;
  constexpr int NC = 2 * KQ;  // float4 chunks per pattern vector
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ double warp_tot[NT / 32 > 0 ? NT / 32 : 1];
  const int NSTAGE = a.nstage;
  const int tid = threadIdx.x;
  const int K = a.K;
  const int b = blockIdx.y;
  const int tile = blockIdx.x;
  const int nst = a.n_steps;
  const TlLayout L = tl_layout(KQ, a.C, a.slots, P, NT, NSTAGE, false);
  const TlStage G = tl_stage(KQ, P, false);
  unsigned char *stages = smem + L.stages;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L.bars);
  float2 *tab2 = reinterpret_cast<float2 *>(smem + L.table);
  float4 *stk = reinterpret_cast<float4 *>(smem + L.stack);
  const TlRecRing ring{reinterpret_cast<int4 *>(smem + L.recs), bars + NSTAGE, a.steps, nst, a.timeout_ns};

  if (tid == 0) {
    for (int st = 0; st < NSTAGE + 2; ++st) mbar_init(&bars[st], 1);
    fence_barrier_init();
  }
  for (int i = tid; i < a.C * 4; i += NT) tab2[i] = make_float2(a.table[i], a.table[i]);
  double props[2 * KQ], freqs[4];
#pragma unroll
  for (int k = 0; k < 2 * KQ; ++k) props[k] = k < K ? a.props[b * K + k] : 0.0;
#pragma unroll
  for (int i = 0; i < 4; ++i) freqs[i] = a.freqs[b * 4 + i];
  __syncthreads();
  bool timed_out = false;
  if (tid == 0) {
    ring.load_chunk(0);
    ring.load_chunk(1);
    for (int s = 0; s < NSTAGE - 1 && s < nst && !timed_out; ++s) {
      int4 cur[3];
      if (ring.get(s, cur)) tl_issue<false>(a, KQ, stages + s * G.bytes, &bars[s], cur, s, b, tile, P, G);
      else timed_out = true;
    }
  }
  timed_out = timed_out || !mbar_wait_bounded(&bars[0], 0, a.timeout_ns);
  if (__syncthreads_or(timed_out)) {
    if (tid == 0) {
      tl_drain(NSTAGE, bars, 0, min(NSTAGE - 2, nst - 1), a.status);
      ring.drain(min(NSTAGE - 1, nst));
    }
    return;
  }
  // this tile's run of a node's stored partials: ((node * ntiles + tile) * NC + c) * P + p
  float4 *gtile = a.partials
                      ? reinterpret_cast<float4 *>(a.partials) + (size_t(b) * (nst - 1) * a.ntiles + tile) * NC * P
                      : nullptr;
  const size_t node_stride = size_t(a.ntiles) * NC * P;  // float4 per node

  int E[R];
  double ll[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    E[r] = 0;
    ll[r] = 0.0;
  }
  int cs = 0, cph = 0, is = NSTAGE - 1;
  for (int s = 0; s < nst; ++s) {
    if (tid == 0 && s + NSTAGE - 1 < nst) {
      const int sp = s + NSTAGE - 1;
      int4 cur[3];
      if (ring.get(sp, cur)) tl_issue<false>(a, KQ, stages + is * G.bytes, &bars[is], cur, sp, b, tile, P, G);
      else timed_out = true;
    }
    is = is + 1 == NSTAGE ? 0 : is + 1;
    const unsigned char *stg = stages + cs * G.bytes;
    const int4 r0 = reinterpret_cast<const int4 *>(stg + G.rec)[0];
    const int4 r1 = reinterpret_cast<const int4 *>(stg + G.rec)[1];
    const int node = r0.x;
    const bool ltip = r0.y < a.tip_count, rtip = r0.z < a.tip_count;
    const float2 *pml = reinterpret_cast<const float2 *>(stg + G.pm);
    const float2 *pmr = pml + KQ * 16;
    const int out_slot = r1.y;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int p = r * NT + tid;
      Vec<KQ> v, al, ar;
      if (ltip) vec_tip<KQ>(v, tab2, stg[G.codes + p]);
      else vec_load<KQ>(v, stk + r0.w * NC * P + p, P);
      mat_vec<KQ>(al, pml, v);
      if (rtip) vec_tip<KQ>(v, tab2, stg[G.codes + P + p]);
      else vec_load<KQ>(v, stk + r1.x * NC * P + p, P);
      mat_vec<KQ>(ar, pmr, v);
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int q = 0; q < KQ; ++q) al.v[j][q] = __fmul2_rn(al.v[j][q], ar.v[j][q]);
      if (a.rescale) vec_rescale<KQ>(al, E[r]);
      if (out_slot >= 0) {
        vec_store<KQ>(stk + out_slot * NC * P + p, P, al);
        if (gtile)
          vec_store_pm_stream<KQ>(reinterpret_cast<float2 *>(gtile + size_t(node - a.tip_count) * node_stride), p, P,
                                  al);
      } else {
        double site = 0.0;
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
          for (int q = 0; q < KQ; ++q)
            site = fma(freqs[j], fma(props[2 * q], double(al.v[j][q].x), props[2 * q + 1] * double(al.v[j][q].y)),
                       site);
        ll[r] = log(site) + double(E[r]) * 0.69314718055994530942;
      }
    }
    const int ns = cs + 1 == NSTAGE ? 0 : cs + 1;
    const int nph = ns == 0 ? cph ^ 1 : cph;
    if (s + 1 < nst) timed_out = timed_out || !mbar_wait_bounded(&bars[ns], nph, a.timeout_ns);
    if (__syncthreads_or(timed_out)) {
      if (tid == 0) {
        tl_drain(NSTAGE, bars, s + 1, min(s + NSTAGE - 1, nst - 1), a.status);
        ring.drain(min(s + NSTAGE, nst));
      }
      return;
    }
    cs = ns;
    cph = nph;
  }
  double contrib = 0.0;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int n = tile * P + r * NT + tid;
    if (n < a.N) {
      if (a.site_lnl) a.site_lnl[size_t(b) * a.N + n] = ll[r];
      contrib += a.weights[n] * ll[r];
    }
  }
  contrib = warp_sum(contrib);
  if ((tid & 31) == 0) warp_tot[tid >> 5] = contrib;
  __syncthreads();
  if (tid == 0) {
    double tot = 0.0;
    for (int w = 0; w < (NT + 31) / 32; ++w) tot += warp_tot[w];
    a.tile_lnl[size_t(b) * a.ntiles + tile] = tot;
  }
}

// Post-order with a producer warp: warp NT/32 issues the staging copies
// (waiting for each stage's "empty" barrier), the NT compute threads wait only
// on the stage's "full" barrier and never on each other -- a thread touches
// only its own pattern's stack entries, so the compute warps need no block
// barrier per step and drift up to NSTAGE - 1 steps apart.
template <int KQ, int NT>
__device__ __forceinline__ void tl_forward_ws_body(const PruneArgs<float> &a, const int tile, const int b) {
  constexpr int P = NT;  // patterns of this CTA: NT / kTlPartTile stored tiles of one sample
  constexpr int TPC = NT / kTlPartTile;
  static_assert(NT % kTlPartTile == 0, "whole stored tiles per CTA");
  constexpr int NC = 2 * KQ;
  constexpr int NW = NT / 32;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ double warp_tot[NW];
  __shared__ uint64_t empty[8];
  __shared__ int abort_flag;
  const int NSTAGE = a.nstage;
  const int tid = threadIdx.x, lane = tid & 31;
  const int K = a.K;
  const int nst = a.n_steps;
  const TlLayout L = tl_layout(KQ, a.C, a.slots, P, NT, NSTAGE, false);
  const TlStage G = tl_stage(KQ, P, false);
  unsigned char *stages = smem + L.stages;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L.bars);
  float2 *tab2 = reinterpret_cast<float2 *>(smem + L.table);
  float4 *stk = reinterpret_cast<float4 *>(smem + L.stack);

  if (tid == 0) {
    for (int st = 0; st < NSTAGE + 2; ++st) mbar_init(&bars[st], 1);
    for (int st = 0; st < NSTAGE; ++st) mbar_init(&empty[st], NW);
    abort_flag = 0;
    fence_barrier_init();
  }
  signed char *onehot = reinterpret_cast<signed char *>(smem + L.onehot);
  for (int i = tid; i < a.C * 4; i += NT + 32) tab2[i] = make_float2(a.table[i], a.table[i]);
  for (int c = tid; c < a.C; c += NT + 32) onehot[c] = onehot_state(a.table, c);
  __syncthreads();

  if (tid >= NT) {  // producer warp
    if (lane == 0) {
      const TlRecRing ring{reinterpret_cast<int4 *>(smem + L.recs), bars + NSTAGE, a.steps_ws, nst, a.timeout_ns};
      ring.load_chunk(0);
      ring.load_chunk(1);
      int issued = 0;
      bool ok = true;
      for (int s = 0; s < nst && ok; ++s) {
        const int st = s % NSTAGE, round = s / NSTAGE;
        if (round > 0) ok = mbar_wait_bounded(&empty[st], (round - 1) & 1, a.timeout_ns);
        if (ok && atomicAdd(&abort_flag, 0) != 0) ok = false;
        int4 cur[3];
        if (ok) ok = ring.get(s, cur);
        if (ok) {
          tl_issue<false>(a, KQ, stages + st * G.bytes, &bars[st], cur, s, b, tile, P, G);
          issued = s + 1;
        }
      }
      if (!ok) {
        atomicExch(&abort_flag, 1);
        // wait (bounded) for the copies already issued before leaving
        tl_drain(NSTAGE, bars, max(0, issued - NSTAGE), issued - 1, a.status);
        ring.drain(issued);
      }
    }
  } else {  // compute threads: one pattern each
    const int p = tid;
    const int my_tile = tile * TPC + p / kTlPartTile, pl = p % kTlPartTile;  // stored tile, column in it
    Vec<KQ> carry;  // partial of the previous step's node when this step is its parent
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < KQ; ++q) carry.v[j][q] = make_float2(0.0f, 0.0f);
    float4 *gtile = a.partials && my_tile < a.ntiles
                        ? reinterpret_cast<float4 *>(a.partials) +
                              (size_t(b) * (nst - 1) * a.ntiles + my_tile) * NC * kTlPartTile
                        : nullptr;
    const size_t node_stride = size_t(a.ntiles) * NC * kTlPartTile;  // float4 per node
    int E = 0;
    double ll = 0.0;
    for (int s = 0; s < nst; ++s) {
      const int st = s % NSTAGE;
      if (!mbar_wait_bounded(&bars[st], (s / NSTAGE) & 1, a.timeout_ns)) {
        atomicExch(&abort_flag, 1);
        atomicExch(a.status, kDeviceTimeout);
        break;
      }
      const unsigned char *stg = stages + st * G.bytes;
      const int4 r0 = reinterpret_cast<const int4 *>(stg + G.rec)[0];
      const int4 r1 = reinterpret_cast<const int4 *>(stg + G.rec)[1];
      const int node = r0.x;
      const bool ltip = r0.y < a.tip_count, rtip = r0.z < a.tip_count;
      const float2 *pml = reinterpret_cast<const float2 *>(stg + G.pm);
      const float2 *pmr = pml + KQ * 16;
      const int out_slot = r1.y;
      Vec<KQ> v, al, ar;
      // a tip with a one-hot code contributes a column of P
      const int sl = ltip ? int(onehot[stg[G.codes + p]]) : -1;
      if (sl >= 0) {
        mat_col<KQ>(al, pml, sl);
      } else {
        if (ltip) vec_tip<KQ>(v, tab2, stg[G.codes + p]);
        else if (r0.w == kWsCarry) v = carry;
        else vec_load<KQ>(v, stk + r0.w * NC * P + p, P);
        mat_vec<KQ>(al, pml, v);
      }
      const int sr = rtip ? int(onehot[stg[G.codes + P + p]]) : -1;
      if (sr >= 0) {
        mat_col<KQ>(ar, pmr, sr);
      } else {
        if (rtip) vec_tip<KQ>(v, tab2, stg[G.codes + P + p]);
        else if (r1.x == kWsCarry) v = carry;
        else vec_load<KQ>(v, stk + r1.x * NC * P + p, P);
        mat_vec<KQ>(ar, pmr, v);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[st]);  // stage consumed by this warp
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int q = 0; q < KQ; ++q) al.v[j][q] = __fmul2_rn(al.v[j][q], ar.v[j][q]);
      if (a.rescale) vec_rescale<KQ>(al, E);
      if (out_slot != -1) {  // not the root: to the stack or, for the next step, to registers
        if (out_slot == kWsCarry) carry = al;
        else vec_store<KQ>(stk + out_slot * NC * P + p, P, al);
        if (gtile)
          vec_store_pm_stream<KQ>(reinterpret_cast<float2 *>(gtile + size_t(node - a.tip_count) * node_stride), pl,
                                  kTlPartTile, al);
      } else {
        double site = 0.0;  // category weights and root frequencies are read here only
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const double fj = a.freqs[b * 4 + j];
#pragma unroll
          for (int q = 0; q < KQ; ++q) {
            const double p0 = a.props[b * K + 2 * q], p1 = 2 * q + 1 < K ? a.props[b * K + 2 * q + 1] : 0.0;
            site = fma(fj, fma(p0, double(al.v[j][q].x), p1 * double(al.v[j][q].y)), site);
          }
        }
        ll = log(site) + double(E) * 0.69314718055994530942;
      }
    }
    double contrib = 0.0;
    const int n = tile * P + p;
    if (n < a.N) {
      if (a.site_lnl) a.site_lnl[size_t(b) * a.N + n] = ll;
      contrib = a.weights[n] * ll;
    }
    contrib = warp_sum(contrib);
    if (lane == 0) warp_tot[tid >> 5] = contrib;
  }
  __syncthreads();
  if (tid < TPC) {  // one sum per stored tile, its warps in order
    constexpr int WPT = kTlPartTile / 32;
    double tot = 0.0;
    for (int w = 0; w < WPT; ++w) tot += warp_tot[tid * WPT + w];
    if (tile * TPC + tid < a.ntiles) a.tile_lnl[size_t(b) * a.ntiles + tile * TPC + tid] = tot;
  }
}

template <int KQ, int NT>
__global__ void __launch_bounds__(NT + 32, tl_ws_min_blocks(KQ, NT))
    tl_forward_ws_kernel(const __grid_constant__ PruneArgs<float> a) {
  tl_forward_ws_body<KQ, NT>(a, blockIdx.x, blockIdx.y);
}

// The same post-order over the tiles of several plans in one launch (plans
// of one category-pair count): CTA x of the 1-D grid walks tile `tile` of
// sample `b` of plan `pi` (MultiPrune::locate).
template <int KQ, int NT>
__global__ void __launch_bounds__(NT + 32, tl_ws_min_blocks(KQ, NT))
    tl_forward_ws_multi_kernel(const __grid_constant__ MultiPrune<float> m) {
  int pi, tile, b;
  m.locate(blockIdx.x, pi, tile, b);
  tl_forward_ws_body<KQ, NT>(m.a[pi], tile, b);
}

// ----------------------------------------------------------------- backward
// One pattern per thread (R = 1): the adjoint keeps too many vectors live.
template <int KQ, int NT>
__global__ void __launch_bounds__(NT) tl_backward_kernel(const PruneArgs<float> a) {
  constexpr int P = NT;
  constexpr int NC = 2 * KQ;
  constexpr int NW = NT / 32;
  extern __shared__ __align__(128) unsigned char smem[];
  const int NSTAGE = a.nstage;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int K = a.K;
  const int b = blockIdx.y;
  const int tile = blockIdx.x;
  const int n = tile * P + tid;
  const bool act = n < a.N;
  const int rem = min(P, a.N - tile * P);
  const int KSS = K * 16;
  const int nst = a.n_steps;
  const TlLayout L = tl_layout(KQ, a.C, a.slots, P, NT, NSTAGE, true);
  const TlStage G = tl_stage(KQ, P, true);
  unsigned char *stages = smem + L.stages;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L.bars);
  float2 *tab2 = reinterpret_cast<float2 *>(smem + L.table);
  float4 *stk = reinterpret_cast<float4 *>(smem + L.stack);
  float4 *xbuf = reinterpret_cast<float4 *>(smem + L.xbuf);  // [2] pair-major tiles: coef * outside partial
  float2 *red = reinterpret_cast<float2 *>(smem + L.red);    // [16][NT+1] float2: element ij of each thread's block
  float *redr = reinterpret_cast<float *>(smem + L.red_root);
  const TlRecRing ring{reinterpret_cast<int4 *>(smem + L.recs), bars + NSTAGE, a.steps_rev, nst, a.timeout_ns};
  // reduction split: unit = (child, category pair), U threads per unit
  constexpr int UNITS = 2 * KQ;
  constexpr int U = NT / UNITS;
  const float w = act ? float(a.weights[n]) : 0.0f;

  if (tid == 0) {
    for (int st = 0; st < NSTAGE + 2; ++st) mbar_init(&bars[st], 1);
    fence_barrier_init();
  }
  for (int i = tid; i < a.C * 4; i += NT) tab2[i] = make_float2(a.table[i], a.table[i]);
  double props[2 * KQ], freqs[4];
#pragma unroll
  for (int k = 0; k < 2 * KQ; ++k) props[k] = k < K ? a.props[b * K + k] : 0.0;
#pragma unroll
  for (int i = 0; i < 4; ++i) freqs[i] = a.freqs[b * 4 + i];
  __syncthreads();
  bool timed_out = false;
  if (tid == 0) {
    ring.load_chunk(0);
    ring.load_chunk(1);
    for (int j = 0; j < NSTAGE - 1 && j < nst && !timed_out; ++j) {
      int4 cur[3];
      if (ring.get(j, cur)) tl_issue<true>(a, KQ, stages + j * G.bytes, &bars[j], cur, nst - 1 - j, b, tile, P, G);
      else timed_out = true;
    }
  }
  timed_out = timed_out || !mbar_wait_bounded(&bars[0], 0, a.timeout_ns);
  if (__syncthreads_or(timed_out)) {
    if (tid == 0) {
      tl_drain(NSTAGE, bars, 0, min(NSTAGE - 2, nst - 1), a.status);
      ring.drain(min(NSTAGE - 1, nst));
    }
    return;
  }

  int prev_left = -1, prev_right = -1;
  int cs = 0, cph = 0, is = NSTAGE - 1;
  for (int j = 0; j <= nst; ++j) {
    if (j > 0) {  // finish iteration j-1's per-branch sums (fixed order over the U partial blocks)
      for (int e = tid; e < 2 * KSS; e += NT) {
        const int side = e >= KSS;
        const int ei = side ? e - KSS : e;  // (k, i, jj) in the output order
        const int k = ei >> 4, ij = ei & 15;
        const int unit = side * KQ + (k >> 1);
        const float2 *rb = red + ij * (NT + 1) + unit * U;
        float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};  // four chains, fixed order
#pragma unroll
        for (int u = 0; u < U; ++u) acc[u & 3] += (k & 1) ? rb[u].y : rb[u].x;
        const int branch = side ? prev_right : prev_left;
        a.gpart[((size_t(b) * a.branch_count + branch) * a.ntiles + tile) * KSS + ei] =
            (acc[0] + acc[1]) + (acc[2] + acc[3]);
      }
    }
    if (j == nst) break;
    if (tid == 0 && j + NSTAGE - 1 < nst) {
      const int jp = j + NSTAGE - 1;
      int4 cur[3];
      if (ring.get(jp, cur)) tl_issue<true>(a, KQ, stages + is * G.bytes, &bars[is], cur, nst - 1 - jp, b, tile, P, G);
      else timed_out = true;
    }
    is = is + 1 == NSTAGE ? 0 : is + 1;
    const unsigned char *stg = stages + cs * G.bytes;
    const int4 r0 = reinterpret_cast<const int4 *>(stg + G.rec)[0];
    const int4 r1 = reinterpret_cast<const int4 *>(stg + G.rec)[1];
    const int4 r2 = reinterpret_cast<const int4 *>(stg + G.rec)[2];
    const int left = r0.y, right = r0.z;
    const int slot_in = r1.z, slot_l = r1.w, slot_r = r2.x;
    const bool is_root = slot_in < 0;
    const bool ltip = left < a.tip_count, rtip = right < a.tip_count;
    const float2 *pml = reinterpret_cast<const float2 *>(stg + G.pm);
    const float2 *pmr = pml + KQ * 16;
    const float2 *kidl = reinterpret_cast<const float2 *>(stg + G.kids);  // pair-major tiles
    const float2 *kidr = kidl + NC * P * 2;

    Vec<KQ> pre, vl, vr, al, ar;
    if (is_root) {
#pragma unroll
      for (int jj = 0; jj < 4; ++jj)
#pragma unroll
        for (int q = 0; q < KQ; ++q)
          pre.v[jj][q] = make_float2(float(props[2 * q] * freqs[jj]), float(props[2 * q + 1] * freqs[jj]));
    } else {
      vec_load<KQ>(pre, stk + slot_in * NC * P + tid, P);
    }
    if (ltip) vec_tip<KQ>(vl, tab2, stg[G.codes + tid]);
    else vec_load_pm<KQ>(vl, kidl, tid, P);
    if (rtip) vec_tip<KQ>(vr, tab2, stg[G.codes + P + tid]);
    else vec_load_pm<KQ>(vr, kidr, tid, P);
    mat_vec<KQ>(ar, pmr, vr);
    // the left matrices stay in registers for the outside product below
    float2 ml[KQ][4][4];
#pragma unroll
    for (int q = 0; q < KQ; ++q)
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float4 r0v = reinterpret_cast<const float4 *>(pml + (q * 4 + i) * 4)[0];
        const float4 r1v = reinterpret_cast<const float4 *>(pml + (q * 4 + i) * 4)[1];
        ml[q][i][0] = make_float2(r0v.x, r0v.y);
        ml[q][i][1] = make_float2(r0v.z, r0v.w);
        ml[q][i][2] = make_float2(r1v.x, r1v.y);
        ml[q][i][3] = make_float2(r1v.z, r1v.w);
      }
#pragma unroll
    for (int q = 0; q < KQ; ++q)
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        float2 acc = __fmul2_rn(ml[q][i][0], vl.v[0][q]);
        acc = __ffma2_rn(ml[q][i][1], vl.v[1][q], acc);
        acc = __ffma2_rn(ml[q][i][2], vl.v[2][q], acc);
        al.v[i][q] = __ffma2_rn(ml[q][i][3], vl.v[3][q], acc);
      }
    // outside partials at the tops of the two branches: xl = pre*ar, xr = pre*al
    Vec<KQ> xl, xr;
    float2 d2[2] = {make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f)};  // two chains
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int q = 0; q < KQ; ++q) {
        xl.v[i][q] = __fmul2_rn(pre.v[i][q], ar.v[i][q]);
        xr.v[i][q] = __fmul2_rn(pre.v[i][q], al.v[i][q]);
        d2[i & 1] = __ffma2_rn(xl.v[i][q], al.v[i][q], d2[i & 1]);
      }
    const float den = (d2[0].x + d2[1].x) + (d2[0].y + d2[1].y);
    // dlnL_n/dP = w_n * x (outer) v / L_n; per-pattern scales cancel against den
    const float coef = (act && den > 0.0f) ? w / den : 0.0f;
    if (is_root) {
      // dlnL/dpi_i = sum_k c_k R[k][i] / L and dlnL/dc_k = sum_i pi_i R[k][i] / L, R = al * ar
      float rpi[4] = {0.0f, 0.0f, 0.0f, 0.0f}, rc[2 * KQ];
#pragma unroll
      for (int k = 0; k < 2 * KQ; ++k) rc[k] = 0.0f;
      if (act) {
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int q = 0; q < KQ; ++q) {
            const float2 rr = __fmul2_rn(al.v[i][q], ar.v[i][q]);
            rpi[i] = fmaf(coef * float(props[2 * q]), rr.x, fmaf(coef * float(props[2 * q + 1]), rr.y, rpi[i]));
            rc[2 * q] = fmaf(coef * float(freqs[i]), rr.x, rc[2 * q]);
            rc[2 * q + 1] = fmaf(coef * float(freqs[i]), rr.y, rc[2 * q + 1]);
          }
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float s = warp_sum(rpi[i]);
        if (lane == 0) redr[warp * 12 + i] = s;
      }
#pragma unroll
      for (int k = 0; k < 2 * KQ; ++k) {
        const float s = warp_sum(rc[k]);
        if (lane == 0 && k < K) redr[warp * 12 + 4 + k] = s;
      }
    }
    // coef * x for the reduction; outside partials at the children's bottoms
    {
      const float2 c2 = make_float2(coef, coef);
      Vec<KQ> u;
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int q = 0; q < KQ; ++q) u.v[i][q] = __fmul2_rn(xl.v[i][q], c2);
      vec_store_pm<KQ>(reinterpret_cast<float2 *>(xbuf), tid, P, u);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int q = 0; q < KQ; ++q) u.v[i][q] = __fmul2_rn(xr.v[i][q], c2);
      vec_store_pm<KQ>(reinterpret_cast<float2 *>(xbuf + NC * P), tid, P, u);
    }
    // o[jj][q] = sum_i P_q[i][jj] * x[i][q] (scale-free: no coefficient)
    if (!ltip) {
      Vec<KQ> o;
#pragma unroll
      for (int q = 0; q < KQ; ++q) {
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) o.v[jj][q] = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          o.v[0][q] = __ffma2_rn(ml[q][i][0], xl.v[i][q], o.v[0][q]);
          o.v[1][q] = __ffma2_rn(ml[q][i][1], xl.v[i][q], o.v[1][q]);
          o.v[2][q] = __ffma2_rn(ml[q][i][2], xl.v[i][q], o.v[2][q]);
          o.v[3][q] = __ffma2_rn(ml[q][i][3], xl.v[i][q], o.v[3][q]);
        }
      }
      int E = 0;
      vec_rescale<KQ>(o, E);
      vec_store<KQ>(stk + slot_l * NC * P + tid, P, o);
    }
    if (!rtip) {
      Vec<KQ> o;
#pragma unroll
      for (int q = 0; q < KQ; ++q) {
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) o.v[jj][q] = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float4 r0v = reinterpret_cast<const float4 *>(pmr + (q * 4 + i) * 4)[0];
          const float4 r1v = reinterpret_cast<const float4 *>(pmr + (q * 4 + i) * 4)[1];
          o.v[0][q] = __ffma2_rn(make_float2(r0v.x, r0v.y), xr.v[i][q], o.v[0][q]);
          o.v[1][q] = __ffma2_rn(make_float2(r0v.z, r0v.w), xr.v[i][q], o.v[1][q]);
          o.v[2][q] = __ffma2_rn(make_float2(r1v.x, r1v.y), xr.v[i][q], o.v[2][q]);
          o.v[3][q] = __ffma2_rn(make_float2(r1v.z, r1v.w), xr.v[i][q], o.v[3][q]);
        }
      }
      int E = 0;
      vec_rescale<KQ>(o, E);
      vec_store<KQ>(stk + slot_r * NC * P + tid, P, o);
    }
    __syncthreads();  // xbuf complete

    // reduction over the tile's patterns, register-blocked:
    //   G[c][k][i][jj] = sum_p (coef x_c)[p][i][k] * v_c[p][jj][k]
    // a thread owns the 4x4 block of one (child, category pair) over patterns
    // s, s+U, ...; the U partial blocks are summed by the next finalize.
    {
      const int unit = tid / U, sidx = tid - unit * U;
      if (unit < UNITS) {
        const int c = unit / KQ, t = unit - c * KQ;
        const bool tipc = c ? rtip : ltip;
        const float2 *xs = reinterpret_cast<const float2 *>(xbuf + c * NC * P) + t * 4 * P;  // pair t rows
        const float2 *vs = (c ? kidr : kidl) + t * 4 * P;
        const unsigned char *csd = stg + G.codes + c * P;
        float2 acc[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) acc[i][jj] = make_float2(0.0f, 0.0f);
#pragma unroll 4
        for (int m = sidx; m < rem; m += U) {
          float2 x[4], v[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) x[i] = xs[i * P + m];
          if (tipc) {
            const float4 *tr = reinterpret_cast<const float4 *>(tab2 + int(csd[m]) * 4);
            const float4 t0 = tr[0], t1 = tr[1];
            v[0] = make_float2(t0.x, t0.y);
            v[1] = make_float2(t0.z, t0.w);
            v[2] = make_float2(t1.x, t1.y);
            v[3] = make_float2(t1.z, t1.w);
          } else {
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) v[jj] = vs[jj * P + m];
          }
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) acc[i][jj] = __ffma2_rn(x[i], v[jj], acc[i][jj]);
        }
        // element-major with a padded row: consecutive threads write consecutive words
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) red[(i * 4 + jj) * (NT + 1) + tid] = acc[i][jj];
      }
    }
    prev_left = left;
    prev_right = right;
    const int ns = cs + 1 == NSTAGE ? 0 : cs + 1;
    const int nph = ns == 0 ? cph ^ 1 : cph;
    if (j + 1 < nst) timed_out = timed_out || !mbar_wait_bounded(&bars[ns], nph, a.timeout_ns);
    if (__syncthreads_or(timed_out)) {
      if (tid == 0) {
        tl_drain(NSTAGE, bars, j + 1, min(j + NSTAGE - 1, nst - 1), a.status);
        ring.drain(min(j + NSTAGE, nst));
      }
      return;
    }
    cs = ns;
    cph = nph;
    if (is_root)
      for (int e = tid; e < 4 + K; e += NT) {
        float acc = 0.0f;
        for (int ww = 0; ww < NW; ++ww) acc += redr[ww * 12 + e];
        a.rootpart[(size_t(b) * a.ntiles + tile) * (4 + K) + e] = acc;
      }
  }
}

}  // namespace tt
