// FP32 pre-order adjoint with in-place outside partials, one thread per
// (pattern, category pair) (S = 4, K categories in KQ = 1, 2 or 4 pairs).
//
// The algorithm, the step records, the staging and the HBM layouts are those
// of ta_backward_kernel (tt_prune_ta.cuh): one CTA walks the reversed
// post-order over one stored tile of 64 patterns of one sample, keeps the
// outside partial of the child walked next in registers, stores the other
// internal child's over that child's consumed post-order tile, and reduces
// dlnL/dP per branch over the tile's patterns through a shared-memory buffer.
// Here the KQ category pairs of a pattern are spread over KQ adjacent lanes,
// so a thread holds 4-element vectors of one pair instead of 4 x KQ: a
// quarter to a half of the registers, KQ times the resident warps, and a
// per-step dependency chain KQ times shorter.  The pattern's denominator and
// the power of two that rescales an outside vector are the only values the
// lanes of a pattern exchange (shuffles within the warp).  The pattern
// reduction splits each 4 x 4 block of a (child, pair) into two halves of
// rows, so that 16 lanes share a unit whatever KQ is.
#pragma once

#include "tt_prune_ta.cuh"
#include "tt_prune_tq.cuh"

namespace tt {

constexpr int kTpTile = 64;  // patterns per CTA: one stored tile

// CTAs per SM the register budget is sized for (64 KQ threads each)
__host__ __device__ constexpr int tp_min_blocks(int KQ) { return KQ == 1 ? 16 : KQ == 2 ? 7 : 4; }

// a pattern's 4 states of one category pair: PairVec (tt_prune_tq.cuh), with
// its pair_sum / pair_max over the KQ lanes of a pattern
using Vp = PairVec;

// out[i] = sum_j P_q[i][j] in[j] (pair q's matrices of one side)
__device__ __forceinline__ void pmat_vec(Vp &out, const float2 *pm, int q, const Vp &in) {
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float4 r0 = reinterpret_cast<const float4 *>(pm + (q * 4 + i) * 4)[0];
    const float4 r1 = reinterpret_cast<const float4 *>(pm + (q * 4 + i) * 4)[1];
    float2 acc = __fmul2_rn(make_float2(r0.x, r0.y), in.v[0]);
    acc = __ffma2_rn(make_float2(r0.z, r0.w), in.v[1], acc);
    acc = __ffma2_rn(make_float2(r1.x, r1.y), in.v[2], acc);
    out.v[i] = __ffma2_rn(make_float2(r1.z, r1.w), in.v[3], acc);
  }
}

// out[j] = sum_i P_q[i][j] in[i]
__device__ __forceinline__ void pmat_t_vec(Vp &out, const float2 *pm, int q, const Vp &in) {
#pragma unroll
  for (int j = 0; j < 4; ++j) out.v[j] = make_float2(0.0f, 0.0f);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float4 r0 = reinterpret_cast<const float4 *>(pm + (q * 4 + i) * 4)[0];
    const float4 r1 = reinterpret_cast<const float4 *>(pm + (q * 4 + i) * 4)[1];
    out.v[0] = __ffma2_rn(make_float2(r0.x, r0.y), in.v[i], out.v[0]);
    out.v[1] = __ffma2_rn(make_float2(r0.z, r0.w), in.v[i], out.v[1]);
    out.v[2] = __ffma2_rn(make_float2(r1.x, r1.y), in.v[i], out.v[2]);
    out.v[3] = __ffma2_rn(make_float2(r1.z, r1.w), in.v[i], out.v[3]);
  }
}

// out[i] = P_q[i][s]
__device__ __forceinline__ void pmat_col(Vp &out, const float2 *pm, int q, int s) {
#pragma unroll
  for (int i = 0; i < 4; ++i) out.v[i] = pm[(q * 4 + i) * 4 + s];
}

template <int KQ>
__device__ __forceinline__ void tp_backward_body(const PruneArgs<float> &a, const int tile, const int b) {
  static_assert(KQ == 1 || KQ == 2 || KQ == 4, "pairs per pattern must be a power of two");
  constexpr int P = kTpTile;
  constexpr int NT = P * KQ;
  constexpr int NW = NT / 32;
  constexpr int UNITS = 4 * KQ;  // (child, pair, half of the rows) blocks of the pattern reduction
  constexpr int UR = NT / UNITS; // 16 lanes per block
  static_assert(UR == 16, "sixteen lanes per reduction block");
  extern __shared__ __align__(128) unsigned char smem[];
  const int NSTAGE = a.nstage;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int q = tid & (KQ - 1), p = tid / KQ;  // category pair, pattern of this thread
  const int K = a.K;
  const int n = tile * P + p;
  const bool act = n < a.N;
  const int rem = min(P, a.N - tile * P);
  const int KSS = K * 16;
  const int nst = a.n_steps;
  const TaLayout L = ta_layout(KQ, a.C, P, NT, NSTAGE);
  const TaStage G = ta_stage(KQ, P);
  unsigned char *stages = smem + L.stages;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L.bars);
  float2 *tab2 = reinterpret_cast<float2 *>(smem + L.table);
  signed char *onehot = reinterpret_cast<signed char *>(smem + L.onehot);
  float2 *xbuf = reinterpret_cast<float2 *>(smem + L.xbuf);  // [2] pair-major tiles: coef * outside partial
  float *redr = reinterpret_cast<float *>(smem + L.red_root);
  const TlRecRingT<kTaRecChunk> ring{reinterpret_cast<int4 *>(smem + L.recs), bars + NSTAGE, a.steps_rev, nst,
                                     a.timeout_ns};
  const float w = act ? float(a.weights[n]) : 0.0f;

  if (tid == 0) {
    for (int st = 0; st < NSTAGE + 2; ++st) mbar_init(&bars[st], 1);
    fence_barrier_init();
  }
  for (int i = tid; i < a.C * 4; i += NT) tab2[i] = make_float2(a.table[i], a.table[i]);
  for (int c = tid; c < a.C; c += NT) onehot[c] = onehot_state(a.table, c);
  __syncthreads();

  // producer state (thread 0): the next reversed step to stage
  int next_issue = 0;
  bool timed_out = false;
  auto issue = [&](int limit) {
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
  auto give_up = [&](int consumed) {
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

  Vp carry;  // outside partial (this pair) of the node walked next
#pragma unroll
  for (int j = 0; j < 4; ++j) carry.v[j] = make_float2(0.0f, 0.0f);
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

    Vp pre, al, ar;
    if (is_root) {
#pragma unroll
      for (int i = 0; i < 4; ++i)
        pre.v[i] = make_float2(float(a.props[b * K + 2 * q] * a.freqs[b * 4 + i]),
                               2 * q + 1 < K ? float(a.props[b * K + 2 * q + 1] * a.freqs[b * 4 + i]) : 0.0f);
    } else if (flags & kTaPreStored) {  // this thread's column, stored by this thread at the parent's step
      const float2 *src = reinterpret_cast<const float2 *>(ta_tile(a, KQ, b, r0.x, tile, P));
#pragma unroll
      for (int i = 0; i < 4; ++i) pre.v[i] = src[(q * 4 + i) * P + p];
    } else {
      pre = carry;
    }
    {  // a tip with a one-hot code contributes a column of P
      const int sr = rtip ? int(onehot[stg[G.codes + P + p]]) : -1;
      if (sr >= 0) {
        pmat_col(ar, pmr, q, sr);
      } else {
        Vp v;
        if (rtip) {
          const int code = stg[G.codes + P + p];
#pragma unroll
          for (int i = 0; i < 4; ++i) v.v[i] = tab2[code * 4 + i];
        } else {
#pragma unroll
          for (int i = 0; i < 4; ++i) v.v[i] = kidr[(q * 4 + i) * P + p];
        }
        pmat_vec(ar, pmr, q, v);
      }
      const int sl = ltip ? int(onehot[stg[G.codes + p]]) : -1;
      if (sl >= 0) {
        pmat_col(al, pml, q, sl);
      } else {
        Vp v;
        if (ltip) {
          const int code = stg[G.codes + p];
#pragma unroll
          for (int i = 0; i < 4; ++i) v.v[i] = tab2[code * 4 + i];
        } else {
#pragma unroll
          for (int i = 0; i < 4; ++i) v.v[i] = kidl[(q * 4 + i) * P + p];
        }
        pmat_vec(al, pml, q, v);
      }
    }
    // outside partials at the tops of the two branches: xl = pre*ar, xr = pre*al
    Vp xl, xr;
    float2 d2 = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      xl.v[i] = __fmul2_rn(pre.v[i], ar.v[i]);
      xr.v[i] = __fmul2_rn(pre.v[i], al.v[i]);
      d2 = __ffma2_rn(xl.v[i], al.v[i], d2);
    }
    const float den = pair_sum<KQ>(d2.x + d2.y);
    // dlnL_n/dP = w_n * x (outer) v / L_n; per-pattern scales cancel against den
    const float coef = (act && den > 0.0f) ? w / den : 0.0f;
    if (is_root) {
      // dlnL/dpi_i = sum_k c_k R[k][i] / L and dlnL/dc_k = sum_i pi_i R[k][i] / L, R = al * ar
      float rpi[4] = {0.0f, 0.0f, 0.0f, 0.0f}, rc[2] = {0.0f, 0.0f};
      if (act) {
        const float c0 = float(a.props[b * K + 2 * q]), c1 = 2 * q + 1 < K ? float(a.props[b * K + 2 * q + 1]) : 0.0f;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float2 rr = __fmul2_rn(al.v[i], ar.v[i]);
          const float fi = float(a.freqs[b * 4 + i]);
          rpi[i] = coef * (c0 * rr.x + c1 * rr.y);
          rc[0] = fmaf(coef * fi, rr.x, rc[0]);
          rc[1] = fmaf(coef * fi, rr.y, rc[1]);
        }
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float s = warp_sum(rpi[i]);
        if (lane == 0) redr[warp * 12 + i] = s;
      }
      // category sums: the lanes of pair t hold categories 2t, 2t+1
#pragma unroll
      for (int t = 0; t < KQ; ++t)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const float s = warp_sum(q == t ? rc[h] : 0.0f);
          if (lane == 0 && 2 * t + h < K) redr[warp * 12 + 4 + 2 * t + h] = s;
        }
    }
    // coef * x for the reduction
    {
      const float2 c2 = make_float2(coef, coef);
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        xbuf[(q * 4 + i) * P + p] = __fmul2_rn(xl.v[i], c2);
        xbuf[KQ * 4 * P + (q * 4 + i) * P + p] = __fmul2_rn(xr.v[i], c2);
      }
    }
    // outside partials at the children's bottoms (scale-free), kept for the
    // next step or stored over the child's post-order tile
    if (!ltip) {
      Vp o;
      pmat_t_vec(o, pml, q, xl);
      int E = 0;
      pv_rescale<KQ>(o, E);
      if (flags & kTaCarryLeft) {
        carry = o;
      } else {
        float2 *dst = reinterpret_cast<float2 *>(ta_tile(a, KQ, b, left, tile, P));
#pragma unroll
        for (int i = 0; i < 4; ++i) dst[(q * 4 + i) * P + p] = o.v[i];
      }
    }
    if (!rtip) {
      Vp o;
      pmat_t_vec(o, pmr, q, xr);
      int E = 0;
      pv_rescale<KQ>(o, E);
      if (flags & kTaCarryRight) {
        carry = o;
      } else {
        float2 *dst = reinterpret_cast<float2 *>(ta_tile(a, KQ, b, right, tile, P));
#pragma unroll
        for (int i = 0; i < 4; ++i) dst[(q * 4 + i) * P + p] = o.v[i];
      }
    }
    __syncthreads();  // xbuf complete

    // reduction over the tile's patterns, register-blocked:
    //   G[c][k][i][jj] = sum_m (coef x_c)[m][i][k] * v_c[m][jj][k]
    // 16 lanes own rows {2h, 2h+1} of the 4 x 4 blocks of one (child c, pair t)
    // over patterns m = s, s+16, ...; recursive halving across the 16 lanes
    // leaves each lane one float of the unit's 16, written straight to HBM.
    {
      const int unit = tid / UR, sidx = tid - unit * UR;
      const int c = unit / (2 * KQ), t = (unit >> 1) & (KQ - 1), h = unit & 1;
      float2 acc[2][4];
#pragma unroll
      for (int rr = 0; rr < 2; ++rr)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) acc[rr][jj] = make_float2(0.0f, 0.0f);
      const bool tipc = c ? rtip : ltip;
      const float2 *xs = xbuf + c * KQ * 4 * P + (t * 4 + 2 * h) * P;  // rows 2h, 2h+1 of pair t
      const float2 *vs = (c ? kidr : kidl) + t * 4 * P;
      const unsigned char *csd = stg + G.codes + c * P;
#pragma unroll 4
      for (int m = sidx; m < rem; m += UR) {
        const float2 x0 = xs[m], x1 = xs[P + m];
        float2 v[4];
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
        for (int jj = 0; jj < 4; ++jj) {
          acc[0][jj] = __ffma2_rn(x0, v[jj], acc[0][jj]);
          acc[1][jj] = __ffma2_rn(x1, v[jj], acc[1][jj]);
        }
      }
      // float e of the unit: row 2h + (e >> 3), column (e >> 1) & 3, category 2t + (e & 1)
      float f[16];
#pragma unroll
      for (int rr = 0; rr < 2; ++rr)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          f[rr * 8 + jj * 2] = acc[rr][jj].x;
          f[rr * 8 + jj * 2 + 1] = acc[rr][jj].y;
        }
#pragma unroll
      for (int o = UR / 2, hh = 8; o >= 1; o >>= 1, hh >>= 1) {
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int e = 0; e < hh; ++e) {
          const float send = up ? f[e] : f[e + hh];
          const float keep = up ? f[e + hh] : f[e];
          f[e] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
      }
      const int rr = sidx >> 3, jj = (sidx >> 1) & 3, cat = sidx & 1;
      if (2 * t + cat < K) {
        const int branch = c ? right : left;
        float *dst = a.gpart + ((size_t(b) * a.branch_count + branch) * a.ntiles + tile) * KSS;
        dst[32 * t + 16 * cat + 4 * (2 * h + rr) + jj] = f[0];
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

template <int KQ, int MB = tp_min_blocks(KQ)>
__global__ void __launch_bounds__(kTpTile * KQ, MB) tp_backward_kernel(const __grid_constant__ PruneArgs<float> a) {
  tp_backward_body<KQ>(a, blockIdx.x, blockIdx.y);
}

// the same adjoint over the tiles of several plans in one launch
template <int KQ, int MB = tp_min_blocks(KQ)>
__global__ void __launch_bounds__(kTpTile * KQ, MB)
    tp_backward_multi_kernel(const __grid_constant__ MultiPrune<float> m) {
  int pi, tile, b;
  m.locate(blockIdx.x, pi, tile, b);
  tp_backward_body<KQ>(m.a[pi], tile, b);
}

}  // namespace tt
