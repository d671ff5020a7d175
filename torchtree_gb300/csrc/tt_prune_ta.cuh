// FP32 pre-order adjoint with in-place outside partials (S = 4).
//
// Same mapping as tl_backward_kernel: one CTA walks the reversed post-order
// over a tile of P patterns of one sample, one thread per pattern, all
// categories in the thread on category pairs with FFMA2, the step record,
// the matrices, the tip-code rows and the stored child tiles staged by the
// TMA engine.  It keeps no shared-memory stack of outside partials:
//  * the reversed walk visits one child of a node right after the node, and
//    that child's outside partial stays in registers (the carry);
//  * the other internal child's outside partial overwrites the child's own
//    post-order tile in HBM, which this step has just read for the last time
//    (a node's post-order tile is read only by its parent's step); at the
//    child's step each thread loads its own column back (it wrote that
//    column itself, so program order is all the ordering needed);
//  * the branch-gradient blocks of the pattern reduction are summed across
//    lanes by warp shuffles and written at once.
// The freed shared memory buys CTAs per SM: the walk is latency-bound.
// The post-order tiles are consumed: a second adjoint needs a new post-order.
#pragma once

#include "tt_prune_tl.cuh"

namespace tt {

constexpr int kTaRecChunk = 16;

// step record | matrix pairs | 2 code rows | 2 child tiles
struct TaStage {
  int rec, pm, codes, kids, bytes;
};

__host__ __device__ inline TaStage ta_stage(int KQ, int P) {
  TaStage g;
  const int tile_bytes = P * KQ * 32;
  int off = 0;
  g.rec = off;
  off = int(align16(off + 48));
  g.pm = off;
  off = int(align16(off + 2 * KQ * 16 * 8));
  g.codes = off;
  off = int(align16(off + 2 * P));
  g.kids = off;
  off = int(align16(off + 2 * tile_bytes));
  g.bytes = off;
  return g;
}

struct TaLayout {
  int stages, bars, recs, table, onehot, xbuf, red_root, total;
};

__host__ __device__ inline TaLayout ta_layout(int KQ, int C, int P, int NT, int nstage) {
  TaLayout L;
  const TaStage g = ta_stage(KQ, P);
  const int vbytes = 2 * KQ * 4 * 4;
  int off = 0;
  L.stages = off;
  off = int(align16(off + nstage * g.bytes));
  L.bars = off;
  off = int(align16(off + (nstage + 2) * 8));
  L.recs = off;
  off = int(align16(off + 2 * kTaRecChunk * 48));
  L.table = off;
  off = int(align16(off + C * 32));
  L.onehot = off;
  off = int(align16(off + C));
  L.xbuf = off;
  off = int(align16(off + 2 * P * vbytes));
  L.red_root = off;
  off = int(align16(off + (NT / 32) * 12 * 4));
  L.total = off;
  return L;
}

// lanes that share one (child, category pair) block of the pattern reduction:
// the largest power of two <= n, at most a warp
__host__ __device__ constexpr int ta_red_lanes(int n) {
  return n >= 32 ? 32 : n >= 16 ? 16 : n >= 8 ? 8 : n >= 4 ? 4 : n >= 2 ? 2 : 1;
}

// CTAs per SM the register budget is sized for: eight 64-thread CTAs fit the
// shared memory of up to two category pairs
__host__ __device__ constexpr int ta_min_blocks(int KQ) { return KQ <= 2 ? 8 : 1; }

// the post-order tile of internal node `node` (pair-major, P patterns)
__device__ __forceinline__ float *ta_tile(const PruneArgs<float> &a, int KQ, int b, int node, int tile, int P) {
  return a.partials + ((size_t(b) * (a.n_steps - 1) + (node - a.tip_count)) * a.ntiles + tile) * size_t(P) * KQ * 8;
}

// Stage reversed step s (forward index fs): record, matrix pairs, code rows
// of tip children and tiles of internal children.
__device__ __forceinline__ void ta_issue(const PruneArgs<float> &a, int KQ, unsigned char *stage, uint64_t *bar,
                                         const int4 (&rec)[3], int fs, int b, int tile, int P, const TaStage &g) {
  int4 *r = reinterpret_cast<int4 *>(stage + g.rec);
  r[0] = rec[0];
  r[1] = rec[1];
  r[2] = rec[2];
  const int left = rec[0].y, right = rec[0].z;
  const uint32_t pbytes = uint32_t(2 * KQ * 16 * 8);
  const uint32_t tile_bytes = uint32_t(P) * KQ * 32;
  uint32_t total = pbytes;
  total += left < a.tip_count ? uint32_t(P) : tile_bytes;
  total += right < a.tip_count ? uint32_t(P) : tile_bytes;
  mbar_arrive_expect_tx(bar, total);
  bulk_copy_g2s(stage + g.pm, a.pmat + (size_t(b) * a.n_steps + fs) * 2 * KQ * 32, pbytes, bar);
  const int child[2] = {left, right};
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    if (child[c] < a.tip_count)
      bulk_copy_g2s(stage + g.codes + c * P, a.codes + size_t(child[c]) * a.code_stride + size_t(tile) * P,
                    uint32_t(P), bar);
    else
      bulk_copy_g2s(stage + g.kids + c * int(tile_bytes), ta_tile(a, KQ, b, child[c], tile, P), tile_bytes, bar);
  }
  // this step reads back the outside tile its parent's step stored: bring it
  // into L2 now, a step ahead of the threads' loads
  if (rec[2].y & kTaPreStored) bulk_prefetch_l2(ta_tile(a, KQ, b, rec[0].x, tile, P), tile_bytes);
}

// o[jj][q] = sum_i P_q[i][jj] x[i][q] with the pair matrices of one side in
// shared memory
template <int KQ>
__device__ __forceinline__ void mat_t_vec(Vec<KQ> &o, const float2 *pm, const Vec<KQ> &x) {
#pragma unroll
  for (int q = 0; q < KQ; ++q) {
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) o.v[jj][q] = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float4 r0v = reinterpret_cast<const float4 *>(pm + (q * 4 + i) * 4)[0];
      const float4 r1v = reinterpret_cast<const float4 *>(pm + (q * 4 + i) * 4)[1];
      o.v[0][q] = __ffma2_rn(make_float2(r0v.x, r0v.y), x.v[i][q], o.v[0][q]);
      o.v[1][q] = __ffma2_rn(make_float2(r0v.z, r0v.w), x.v[i][q], o.v[1][q]);
      o.v[2][q] = __ffma2_rn(make_float2(r1v.x, r1v.y), x.v[i][q], o.v[2][q]);
      o.v[3][q] = __ffma2_rn(make_float2(r1v.z, r1v.w), x.v[i][q], o.v[3][q]);
    }
  }
}

template <int KQ, int NT>
__device__ __forceinline__ void ta_backward_body(const PruneArgs<float> &a, const int tile, const int b) {
  constexpr int P = NT;
  constexpr int NW = NT / 32;
  constexpr int UNITS = 2 * KQ;                   // (child, category pair) blocks
  constexpr int UR = ta_red_lanes(NT / UNITS);    // lanes per block
  static_assert(UNITS * UR <= NT, "reduction lanes exceed the CTA");
  extern __shared__ __align__(128) unsigned char smem[];
  const int NSTAGE = a.nstage;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int K = a.K;
  const int n = tile * P + tid;
  const bool act = n < a.N;
  const int rem = min(P, a.N - tile * P);
  const int KSS = K * 16;
  const int nst = a.n_steps;
  const TaLayout L = ta_layout(KQ, a.C, P, NT, NSTAGE);
  const TaStage G = ta_stage(KQ, P);
  unsigned char *stages = smem + L.stages;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L.bars);
  float2 *tab2 = reinterpret_cast<float2 *>(smem + L.table);
  float2 *xbuf = reinterpret_cast<float2 *>(smem + L.xbuf);  // [2] pair-major tiles: coef * outside partial
  float *redr = reinterpret_cast<float *>(smem + L.red_root);
  const TlRecRingT<kTaRecChunk> ring{reinterpret_cast<int4 *>(smem + L.recs), bars + NSTAGE, a.steps_rev, nst,
                                     a.timeout_ns};
  const float w = act ? float(a.weights[n]) : 0.0f;

  if (tid == 0) {
    for (int st = 0; st < NSTAGE + 2; ++st) mbar_init(&bars[st], 1);
    fence_barrier_init();
  }
  signed char *onehot = reinterpret_cast<signed char *>(smem + L.onehot);
  for (int i = tid; i < a.C * 4; i += NT) tab2[i] = make_float2(a.table[i], a.table[i]);
  for (int c = tid; c < a.C; c += NT) onehot[c] = onehot_state(a.table, c);
  __syncthreads();

  // producer state (thread 0): the next reversed step to stage
  int next_issue = 0;
  bool timed_out = false;
  auto issue = [&](int limit) {  // stage steps up to `limit`
    while (next_issue < nst && next_issue <= limit) {
      int4 rec[3];
      if (!ring.get(next_issue, rec)) {
        timed_out = true;
        return;
      }
      const int st = next_issue % NSTAGE;
      ta_issue(a, KQ, stages + st * G.bytes, &bars[st], rec, nst - 1 - next_issue, b, tile, P, G);
      ++next_issue;
    }
  };
  auto give_up = [&](int consumed) {  // wait (bounded) for the copies in flight, then leave
    if (tid == 0) {
      tl_drain(NSTAGE, bars, consumed, next_issue - 1, a.status);
      ring.drain(next_issue);
    }
  };
  if (tid == 0) {
    ring.load_chunk(0);
    ring.load_chunk(1);
    issue(NSTAGE - 2);
  }
  timed_out = timed_out || !mbar_wait_bounded(&bars[0], 0, a.timeout_ns);
  if (__syncthreads_or(timed_out)) {
    give_up(0);
    return;
  }

  Vec<KQ> carry;  // outside partial of the node walked next
#pragma unroll
  for (int jj = 0; jj < 4; ++jj)
#pragma unroll
    for (int q = 0; q < KQ; ++q) carry.v[jj][q] = make_float2(0.0f, 0.0f);
  for (int j = 0; j < nst; ++j) {
    if (tid == 0) issue(j + NSTAGE - 1);
    const unsigned char *stg = stages + (j % NSTAGE) * G.bytes;
    const int4 r0 = reinterpret_cast<const int4 *>(stg + G.rec)[0];
    const int4 r2 = reinterpret_cast<const int4 *>(stg + G.rec)[2];
    const int left = r0.y, right = r0.z, flags = r2.y;
    const bool is_root = j == 0;
    const bool ltip = left < a.tip_count, rtip = right < a.tip_count;
    const float2 *pml = reinterpret_cast<const float2 *>(stg + G.pm);
    const float2 *pmr = pml + KQ * 16;
    const float2 *kidl = reinterpret_cast<const float2 *>(stg + G.kids);  // pair-major tiles
    const float2 *kidr = kidl + KQ * 4 * P;

    // category weights and root frequencies, read at the root step only
    float props[2 * KQ], freqs[4];
    Vec<KQ> pre, vl, vr, al, ar;
    if (is_root) {
#pragma unroll
      for (int k = 0; k < 2 * KQ; ++k) props[k] = k < K ? float(a.props[b * K + k]) : 0.0f;
#pragma unroll
      for (int i = 0; i < 4; ++i) freqs[i] = float(a.freqs[b * 4 + i]);
#pragma unroll
      for (int jj = 0; jj < 4; ++jj)
#pragma unroll
        for (int q = 0; q < KQ; ++q)
          pre.v[jj][q] = make_float2(float(a.props[b * K + 2 * q] * a.freqs[b * 4 + jj]),
                                     2 * q + 1 < K ? float(a.props[b * K + 2 * q + 1] * a.freqs[b * 4 + jj]) : 0.0f);
    } else if (flags & kTaPreStored) {  // this thread's column, stored by this thread at the parent's step
      vec_load_pm<KQ>(pre, reinterpret_cast<const float2 *>(ta_tile(a, KQ, b, r0.x, tile, P)), tid, P);
    } else {
      pre = carry;
    }
    // a tip with a one-hot code contributes a column of P; any other vector
    // goes through the matrix-vector product
    {
      const int sr = rtip ? int(onehot[stg[G.codes + P + tid]]) : -1;
      if (sr >= 0) {
        mat_col<KQ>(ar, pmr, sr);
      } else {
        if (rtip) vec_tip<KQ>(vr, tab2, stg[G.codes + P + tid]);
        else vec_load_pm<KQ>(vr, kidr, tid, P);
        mat_vec<KQ>(ar, pmr, vr);
      }
      const int sl = ltip ? int(onehot[stg[G.codes + tid]]) : -1;
      if (sl >= 0) {
        mat_col<KQ>(al, pml, sl);
      } else {
        if (ltip) vec_tip<KQ>(vl, tab2, stg[G.codes + tid]);
        else vec_load_pm<KQ>(vl, kidl, tid, P);
        mat_vec<KQ>(al, pml, vl);
      }
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
    // dlnL_n/dP = w_n * x (outer) v / L_n; per-pattern scales cancel against den.
    // den is a sum of 16 products of rescaled vectors (well inside the range
    // where the approximate division is within 2 ulp)
    const float coef = (act && den > 0.0f) ? __fdividef(w, den) : 0.0f;
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
            rpi[i] = fmaf(coef * props[2 * q], rr.x, fmaf(coef * props[2 * q + 1], rr.y, rpi[i]));
            rc[2 * q] = fmaf(coef * freqs[i], rr.x, rc[2 * q]);
            rc[2 * q + 1] = fmaf(coef * freqs[i], rr.y, rc[2 * q + 1]);
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
    // coef * x for the reduction
    {
      const float2 c2 = make_float2(coef, coef);
      Vec<KQ> u;
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int q = 0; q < KQ; ++q) u.v[i][q] = __fmul2_rn(xl.v[i][q], c2);
      vec_store_pm<KQ>(xbuf, tid, P, u);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int q = 0; q < KQ; ++q) u.v[i][q] = __fmul2_rn(xr.v[i][q], c2);
      vec_store_pm<KQ>(xbuf + KQ * 4 * P, tid, P, u);
    }
    // outside partials at the children's bottoms (scale-free: no coefficient),
    // kept for the next step or stored over the child's post-order tile
    if (!ltip) {
      Vec<KQ> o;
      mat_t_vec<KQ>(o, pml, xl);
      int E = 0;
      vec_rescale<KQ>(o, E);
      if (flags & kTaCarryLeft) carry = o;
      else vec_store_pm<KQ>(reinterpret_cast<float2 *>(ta_tile(a, KQ, b, left, tile, P)), tid, P, o);
    }
    if (!rtip) {
      Vec<KQ> o;
      mat_t_vec<KQ>(o, pmr, xr);
      int E = 0;
      vec_rescale<KQ>(o, E);
      if (flags & kTaCarryRight) carry = o;
      else vec_store_pm<KQ>(reinterpret_cast<float2 *>(ta_tile(a, KQ, b, right, tile, P)), tid, P, o);
    }
    __syncthreads();  // xbuf complete

    // reduction over the tile's patterns, register-blocked:
    //   G[c][k][i][jj] = sum_p (coef x_c)[p][i][k] * v_c[p][jj][k]
    // UR lanes own the 4x4 blocks of one (child, category pair) over patterns
    // s, s+UR, ...; recursive halving across the UR lanes (packed pair adds)
    // leaves each lane 32 / UR floats of the block, written straight to HBM.
    // The halving splits the block index (i1 i0 jj1 jj0 k) from the top bit
    // down, lane bit UR/2 first.  A lane whose bits are (a1 a0 b1 b0 ..) loads
    // row i ^ a of x and, for an internal child, row jj ^ b of v, so register
    // slot (i', jj') holds element (i' ^ a, jj' ^ b): every lane then keeps
    // the lower half of its slots at every level and sends the upper half,
    // which holds the partner's kept elements, with no lane-dependent selects.
    // A tip child's v comes from the code table, whose row halves a lane
    // loads in the order b1 gives (jj1 permuted); its jj0 level and the
    // category level select as plain recursive halving.
    {
      constexpr int LV = UR >= 32 ? 5 : UR >= 16 ? 4 : UR >= 8 ? 3 : UR >= 4 ? 2 : UR >= 2 ? 1 : 0;
      constexpr int PL = (P + UR - 1) / UR;  // patterns per lane
      const int unit = tid / UR, sidx = tid - unit * UR;
      const bool uact = unit < UNITS;
      const int c = unit / KQ, t = unit - (unit / KQ) * KQ;
      const bool tipc = uact && (c ? rtip : ltip);
      // permutation bits: the top LV bits of the 5-bit block index
      const int bits = LV > 0 ? (sidx << (5 - LV)) : 0;
      const int pa = bits >> 3, pb = (bits >> 1) & (tipc ? 2 : 3);
      float2 acc[4][4];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) acc[i][jj] = make_float2(0.0f, 0.0f);
      if (uact) {
        const float2 *xs = xbuf + c * KQ * 4 * P + t * 4 * P + sidx;  // pair t rows
        const float2 *vs = (c ? kidr : kidl) + t * 4 * P + sidx;
        const unsigned char *csd = stg + G.codes + c * P + sidx;
        const float2 *xr[4], *vr[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          xr[i] = xs + (i ^ pa) * P;
          vr[i] = vs + (i ^ pb) * P;
        }
#pragma unroll
        for (int kk = 0; kk < PL; ++kk) {
          if (sidx + kk * UR < rem) {
            float2 x[4], v[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) x[i] = xr[i][kk * UR];
            if (tipc) {
              const float4 *tr = reinterpret_cast<const float4 *>(tab2 + int(csd[kk * UR]) * 4);
              const float4 t0 = tr[pb >> 1], t1 = tr[(pb >> 1) ^ 1];
              v[0] = make_float2(t0.x, t0.y);
              v[1] = make_float2(t0.z, t0.w);
              v[2] = make_float2(t1.x, t1.y);
              v[3] = make_float2(t1.z, t1.w);
            } else {
#pragma unroll
              for (int jj = 0; jj < 4; ++jj) v[jj] = vr[jj][kk * UR];
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
              for (int jj = 0; jj < 4; ++jj) acc[i][jj] = __ffma2_rn(x[i], v[jj], acc[i][jj]);
          }
        }
      }
      // slot s = i' * 4 + jj' holds categories (2t, 2t + 1) of element (i', jj')
      float2 g[16];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) g[i * 4 + jj] = acc[i][jj];
      // a warp with no tip-child lane skips the jj levels' selects
      const bool sel_jj = __any_sync(0xffffffffu, tipc);
#pragma unroll
      for (int o = UR / 2, h = 8; o >= 1 && h >= 1; o >>= 1, h >>= 1) {
        if (h >= 2 || !sel_jj) {  // i and jj1 levels, and jj0 with every lane permuted
#pragma unroll
          for (int e = 0; e < h; ++e) g[e] = __fadd2_rn(g[e], shfl_xor_f2(g[e + h], o));
        } else {  // jj0 level of tip lanes (internal lanes never swap)
          const bool swap = tipc && (lane & o) != 0;
#pragma unroll
          for (int e = 0; e < h; ++e) {
            const float2 send = swap ? g[e] : g[e + h];
            const float2 keep = swap ? g[e + h] : g[e];
            g[e] = __fadd2_rn(keep, shfl_xor_f2(send, o));
          }
        }
      }
      if (LV == 5) {  // 32 lanes per block: a last level over the pair's two categories
        const bool up = (lane & 1) != 0;
        const float send = up ? g[0].x : g[0].y, keep = up ? g[0].y : g[0].x;
        g[0].x = keep + __shfl_xor_sync(0xffffffffu, send, 1);
      }
      if (uact) {
        const int branch = c ? right : left;
        float *dst = a.gpart + ((size_t(b) * a.branch_count + branch) * a.ntiles + tile) * KSS + 32 * t;
        if (LV == 5) {
          const int k = sidx & 1;
          if (2 * t + k < K) dst[k * 16 + (sidx >> 1)] = g[0].x;
        } else {
          // kept slot s holds element (sidx << (4 - LV)) | s = i * 4 + jj
          constexpr int NG = LV >= 4 ? 1 : 16 >> LV;
#pragma unroll
          for (int s = 0; s < NG; ++s) {
            const int el = (sidx << (LV >= 4 ? 0 : 4 - LV)) | s;
            dst[el] = g[s].x;
            if (2 * t + 1 < K) dst[16 + el] = g[s].y;
          }
        }
      }
    }
    if (j + 1 < nst) timed_out = timed_out || !mbar_wait_bounded(&bars[(j + 1) % NSTAGE], ((j + 1) / NSTAGE) & 1,
                                                                  a.timeout_ns);
    if (__syncthreads_or(timed_out)) {
      give_up(j + 1);
      return;
    }
    if (is_root)
      for (int e = tid; e < 4 + K; e += NT) {
        float acc = 0.0f;
        for (int ww = 0; ww < NW; ++ww) acc += redr[ww * 12 + e];
        a.rootpart[(size_t(b) * a.ntiles + tile) * (4 + K) + e] = acc;
      }
  }
}

template <int KQ, int NT>
__global__ void __launch_bounds__(NT, ta_min_blocks(KQ)) ta_backward_kernel(const __grid_constant__ PruneArgs<float> a) {
  ta_backward_body<KQ, NT>(a, blockIdx.x, blockIdx.y);
}

// the same adjoint over the tiles of several plans in one launch
template <int KQ, int NT>
__global__ void __launch_bounds__(NT, ta_min_blocks(KQ))
    ta_backward_multi_kernel(const __grid_constant__ MultiPrune<float> m) {
  int pi, tile, b;
  m.locate(blockIdx.x, pi, tile, b);
  ta_backward_body<KQ, NT>(m.a[pi], tile, b);
}

}  // namespace tt
