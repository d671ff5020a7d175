// FP32 pruning kernels with one thread per (pattern, category pair).
//
// Same algorithm, staging ring, shared-memory stack and HBM layouts as the
// kernels of tt_prune_tl.cuh, which give a pattern's whole vector to one
// thread; here the KQ category pairs of a pattern are spread over KQ
// neighbouring lanes (KQ in {1, 2, 4}), so a 64-pattern tile runs with
// 64 KQ threads: twice the warps per SM at the same shared memory for the
// usual four categories.  A thread keeps its pair's two 4x4 matrices of the
// step in registers (loaded once, used by the forward products, the outside
// products and the adjoint).  Per-pattern reductions across pairs (the
// rescaling maximum, the adjoint's denominator, the root sums) are lane
// shuffles within the pattern's KQ lanes.  Products and rescaling follow the
// one-thread kernels operation for operation, so both produce identical
// partials.
#pragma once

#include "tt_prune_tl.cuh"

namespace tt {

constexpr int kTqTile = 64;    // patterns per CTA
constexpr int kTqRed2 = 8;     // float2 partial-block elements per adjoint thread

// float2 index of (state j, pair q) of pattern p in a pair-major tile
// [pair][state][P] float2 (the layout of stored partials, staged child tiles,
// the x buffer and, in these kernels, the stack)
template <int KQ>
__device__ __forceinline__ int tq_index(int j, int q, int p) {
  return (q * 4 + j) * kTqTile + p;
}

struct PairVec {
  float2 v[4];  // (category 2q, 2q+1) at state j
};

struct PairMat {
  float2 m[4][4];  // [i][j]
};

template <int KQ>
__device__ __forceinline__ void pv_load(PairVec &x, const float2 *base, int q, int p) {
#pragma unroll
  for (int j = 0; j < 4; ++j) x.v[j] = base[tq_index<KQ>(j, q, p)];
}

template <int KQ>
__device__ __forceinline__ void pv_store(float2 *base, int q, int p, const PairVec &x) {
#pragma unroll
  for (int j = 0; j < 4; ++j) base[tq_index<KQ>(j, q, p)] = x.v[j];
}

template <int KQ>
__device__ __forceinline__ void pv_store_stream(float2 *base, int q, int p, const PairVec &x) {
#pragma unroll
  for (int j = 0; j < 4; ++j) __stcs(base + tq_index<KQ>(j, q, p), x.v[j]);
}

__device__ __forceinline__ void pv_tip(PairVec &x, const float2 *tab2, int code) {
  const float4 a = reinterpret_cast<const float4 *>(tab2)[code * 2];
  const float4 c = reinterpret_cast<const float4 *>(tab2)[code * 2 + 1];
  x.v[0] = make_float2(a.x, a.y);
  x.v[1] = make_float2(a.z, a.w);
  x.v[2] = make_float2(c.x, c.y);
  x.v[3] = make_float2(c.z, c.w);
}

__device__ __forceinline__ void pm_load(PairMat &M, const float2 *pm) {
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float4 r0 = reinterpret_cast<const float4 *>(pm + i * 4)[0];
    const float4 r1 = reinterpret_cast<const float4 *>(pm + i * 4)[1];
    M.m[i][0] = make_float2(r0.x, r0.y);
    M.m[i][1] = make_float2(r0.z, r0.w);
    M.m[i][2] = make_float2(r1.x, r1.y);
    M.m[i][3] = make_float2(r1.z, r1.w);
  }
}

// out[i] = sum_j M[i][j] in[j]   (same operation order as mat_vec)
__device__ __forceinline__ void pm_mul(PairVec &out, const PairMat &M, const PairVec &in) {
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    float2 acc = __fmul2_rn(M.m[i][0], in.v[0]);
    acc = __ffma2_rn(M.m[i][1], in.v[1], acc);
    acc = __ffma2_rn(M.m[i][2], in.v[2], acc);
    out.v[i] = __ffma2_rn(M.m[i][3], in.v[3], acc);
  }
}

// out[j] = sum_i M[i][j] in[i]   (same operation order as the one-thread adjoint)
__device__ __forceinline__ void pm_mul_t(PairVec &out, const PairMat &M, const PairVec &in) {
#pragma unroll
  for (int j = 0; j < 4; ++j) out.v[j] = make_float2(0.0f, 0.0f);
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) out.v[j] = __ffma2_rn(M.m[i][j], in.v[i], out.v[j]);
}

template <int KQ, typename T>
__device__ __forceinline__ T pair_sum(T x) {
  if (KQ >= 2) x += __shfl_xor_sync(0xffffffffu, x, 1);
  if (KQ >= 4) x += __shfl_xor_sync(0xffffffffu, x, 2);
  return x;
}

template <int KQ>
__device__ __forceinline__ float pair_max(float x) {
  if (KQ >= 2) x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, 1));
  if (KQ >= 4) x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, 2));
  return x;
}

// exact power-of-two rescale by the pattern maximum over all pairs (as vec_rescale)
template <int KQ>
__device__ __forceinline__ void pv_rescale(PairVec &x, int &E) {
  float m = fmaxf(fmaxf(fmaxf(x.v[0].x, x.v[0].y), fmaxf(x.v[1].x, x.v[1].y)),
                  fmaxf(fmaxf(x.v[2].x, x.v[2].y), fmaxf(x.v[3].x, x.v[3].y)));
  m = pair_max<KQ>(fmaxf(m, 0.0f));
  const int be = (__float_as_int(m) >> 23) & 0xff;
  const int e = (be == 0 || be == 0xff) ? 0 : min(be - 127, 126);
  const float f = __int_as_float((127 - e) << 23);
  const float2 f2 = make_float2(f, f);
#pragma unroll
  for (int j = 0; j < 4; ++j) x.v[j] = __fmul2_rn(x.v[j], f2);
  E += e;
}

// ------------------------------------------------------------------ forward
template <int KQ>
__global__ void __launch_bounds__(kTqTile * KQ) tq_forward_kernel(const PruneArgs<float> a) {
  constexpr int P = kTqTile, NT = P * KQ, NC = 2 * KQ;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ double warp_tot[NT / 32];
  const int NSTAGE = a.nstage;
  const int tid = threadIdx.x, p = tid / KQ, q = tid - (tid / KQ) * KQ;
  const int K = a.K;
  const int b = blockIdx.y;
  const int tile = blockIdx.x;
  const int nst = a.n_steps;
  const TlLayout L = tl_layout(KQ, a.C, a.slots, P, NT, NSTAGE, false);
  const TlStage G = tl_stage(KQ, P, false);
  unsigned char *stages = smem + L.stages;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L.bars);
  float2 *tab2 = reinterpret_cast<float2 *>(smem + L.table);
  float2 *stk = reinterpret_cast<float2 *>(smem + L.stack);
  const TlRecRing ring{reinterpret_cast<int4 *>(smem + L.recs), bars + NSTAGE, a.steps, nst, a.timeout_ns};

  if (tid == 0) {
    for (int st = 0; st < NSTAGE + 2; ++st) mbar_init(&bars[st], 1);
    fence_barrier_init();
  }
  for (int i = tid; i < a.C * 4; i += NT) tab2[i] = make_float2(a.table[i], a.table[i]);
  const double pr0 = 2 * q < K ? a.props[b * K + 2 * q] : 0.0;
  const double pr1 = 2 * q + 1 < K ? a.props[b * K + 2 * q + 1] : 0.0;
  double freqs[4];
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
  float2 *gtile = a.partials ? reinterpret_cast<float2 *>(a.partials) +
                                   (size_t(b) * (nst - 1) * a.ntiles + tile) * NC * P * 2
                             : nullptr;
  const size_t node_stride = size_t(a.ntiles) * NC * P * 2;  // float2 per node

  int E = 0;
  double ll = 0.0;
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
    const int out_slot = r1.y;
    PairMat M;
    PairVec v, al, ar;
    pm_load(M, pml + q * 16);
    if (ltip) pv_tip(v, tab2, stg[G.codes + p]);
    else pv_load<KQ>(v, stk + r0.w * NC * P * 2, q, p);
    pm_mul(al, M, v);
    pm_load(M, pml + (KQ + q) * 16);
    if (rtip) pv_tip(v, tab2, stg[G.codes + P + p]);
    else pv_load<KQ>(v, stk + r1.x * NC * P * 2, q, p);
    pm_mul(ar, M, v);
#pragma unroll
    for (int j = 0; j < 4; ++j) al.v[j] = __fmul2_rn(al.v[j], ar.v[j]);
    if (a.rescale) pv_rescale<KQ>(al, E);
    if (out_slot >= 0) {
      pv_store<KQ>(stk + out_slot * NC * P * 2, q, p, al);
      if (gtile) pv_store_stream<KQ>(gtile + size_t(node - a.tip_count) * node_stride, q, p, al);
    } else {
      double site = 0.0;
#pragma unroll
      for (int j = 0; j < 4; ++j)
        site = fma(freqs[j], fma(pr0, double(al.v[j].x), pr1 * double(al.v[j].y)), site);
      site = pair_sum<KQ>(site);
      ll = log(site) + double(E) * 0.69314718055994530942;
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
  const int n = tile * P + p;
  if (q == 0 && n < a.N) {
    if (a.site_lnl) a.site_lnl[size_t(b) * a.N + n] = ll;
    contrib = a.weights[n] * ll;
  }
  contrib = warp_sum(contrib);
  if ((tid & 31) == 0) warp_tot[tid >> 5] = contrib;
  __syncthreads();
  if (tid == 0) {
    double tot = 0.0;
    for (int w = 0; w < NT / 32; ++w) tot += warp_tot[w];
    a.tile_lnl[size_t(b) * a.ntiles + tile] = tot;
  }
}

// ----------------------------------------------------------------- backward
// Pattern reduction: unit = (child, pair t, row half), 16 threads per unit,
// each over 4 patterns, a 2 x 4 float2 block per thread.
template <int KQ>
__global__ void __launch_bounds__(kTqTile * KQ) tq_backward_kernel(const PruneArgs<float> a) {
  constexpr int P = kTqTile, NT = P * KQ, NC = 2 * KQ, NW = NT / 32;
  constexpr int UNITS = 4 * KQ, U = NT / UNITS;  // U = 16
  extern __shared__ __align__(128) unsigned char smem[];
  const int NSTAGE = a.nstage;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int p = tid / KQ, q = tid - (tid / KQ) * KQ;
  const int K = a.K;
  const int b = blockIdx.y;
  const int tile = blockIdx.x;
  const int n = tile * P + p;
  const bool act = n < a.N;
  const int rem = min(P, a.N - tile * P);
  const int KSS = K * 16;
  const int nst = a.n_steps;
  const TlLayout L = tl_layout(KQ, a.C, a.slots, P, NT, NSTAGE, true, kTqRed2);
  const TlStage G = tl_stage(KQ, P, true);
  unsigned char *stages = smem + L.stages;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L.bars);
  float2 *tab2 = reinterpret_cast<float2 *>(smem + L.table);
  float2 *stk = reinterpret_cast<float2 *>(smem + L.stack);
  float2 *xbuf = reinterpret_cast<float2 *>(smem + L.xbuf);  // [2][NC][P] float4 as float2: coef * outside
  float2 *red = reinterpret_cast<float2 *>(smem + L.red);    // [8][NT+1] float2
  float *redr = reinterpret_cast<float *>(smem + L.red_root);
  const TlRecRing ring{reinterpret_cast<int4 *>(smem + L.recs), bars + NSTAGE, a.steps_rev, nst, a.timeout_ns};
  const float w = act ? float(a.weights[n]) : 0.0f;

  if (tid == 0) {
    for (int st = 0; st < NSTAGE + 2; ++st) mbar_init(&bars[st], 1);
    fence_barrier_init();
  }
  for (int i = tid; i < a.C * 4; i += NT) tab2[i] = make_float2(a.table[i], a.table[i]);
  const double pr0 = 2 * q < K ? a.props[b * K + 2 * q] : 0.0;
  const double pr1 = 2 * q + 1 < K ? a.props[b * K + 2 * q + 1] : 0.0;
  double freqs[4];
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

  // reduction ownership
  const int unit = tid / U, sidx = tid - (tid / U) * U;
  const int uc = unit / (2 * KQ), ut = (unit - uc * 2 * KQ) >> 1, uh = unit & 1;

  int prev_left = -1, prev_right = -1;
  int cs = 0, cph = 0, is = NSTAGE - 1;
  for (int j = 0; j <= nst; ++j) {
    if (j > 0) {  // finish iteration j-1's per-branch sums (fixed order over the U partial blocks)
      for (int e = tid; e < 2 * KSS; e += NT) {
        const int side = e >= KSS;
        const int ei = side ? e - KSS : e;  // (k, i, jj) in the output order
        const int k = ei >> 4, i = (ei >> 2) & 3, jj = ei & 3;
        const int un = side * 2 * KQ + (k >> 1) * 2 + (i >> 1);
        const float2 *rb = red + ((i & 1) * 4 + jj) * (NT + 1) + un * U;
        float acc = 0.0f;
#pragma unroll 4
        for (int u = 0; u < U; ++u) acc += (k & 1) ? rb[u].y : rb[u].x;
        const int branch = side ? prev_right : prev_left;
        a.gpart[((size_t(b) * a.branch_count + branch) * a.ntiles + tile) * KSS + ei] = acc;
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
    const float2 *kidl = reinterpret_cast<const float2 *>(stg + G.kids);
    const float2 *kidr = kidl + NC * P * 2;

    PairMat Ml, Mr;
    pm_load(Ml, pml + q * 16);
    pm_load(Mr, pml + (KQ + q) * 16);
    PairVec pre, vl, vr, al, ar;
    if (is_root) {
#pragma unroll
      for (int jj = 0; jj < 4; ++jj) pre.v[jj] = make_float2(float(pr0 * freqs[jj]), float(pr1 * freqs[jj]));
    } else {
      pv_load<KQ>(pre, stk + slot_in * NC * P * 2, q, p);
    }
    if (ltip) pv_tip(vl, tab2, stg[G.codes + p]);
    else pv_load<KQ>(vl, kidl, q, p);
    if (rtip) pv_tip(vr, tab2, stg[G.codes + P + p]);
    else pv_load<KQ>(vr, kidr, q, p);
    pm_mul(al, Ml, vl);
    pm_mul(ar, Mr, vr);
    PairVec xl, xr;
    float2 d2 = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      xl.v[i] = __fmul2_rn(pre.v[i], ar.v[i]);
      xr.v[i] = __fmul2_rn(pre.v[i], al.v[i]);
      d2 = __ffma2_rn(xl.v[i], al.v[i], d2);
    }
    const float den = pair_sum<KQ>(d2.x + d2.y);
    const float coef = (act && den > 0.0f) ? w / den : 0.0f;
    if (is_root) {
      // dlnL/dpi_i = sum_k c_k R[k][i] / L and dlnL/dc_k = sum_i pi_i R[k][i] / L, R = al * ar
      float rpi[4] = {0.0f, 0.0f, 0.0f, 0.0f}, rc0 = 0.0f, rc1 = 0.0f;
      if (act) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float2 rr = __fmul2_rn(al.v[i], ar.v[i]);
          rpi[i] = fmaf(coef * float(pr0), rr.x, coef * float(pr1) * rr.y);
          rc0 = fmaf(coef * float(freqs[i]), rr.x, rc0);
          rc1 = fmaf(coef * float(freqs[i]), rr.y, rc1);
        }
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float s = warp_sum(rpi[i]);
        if (lane == 0) redr[warp * 12 + i] = s;
      }
#pragma unroll
      for (int k = 0; k < 2 * KQ; ++k) {
        const float s = warp_sum(k == 2 * q ? rc0 : (k == 2 * q + 1 ? rc1 : 0.0f));
        if (lane == 0 && k < K) redr[warp * 12 + 4 + k] = s;
      }
    }
    {  // coef * x for the pattern reduction
      const float2 c2 = make_float2(coef, coef);
      PairVec u;
#pragma unroll
      for (int i = 0; i < 4; ++i) u.v[i] = __fmul2_rn(xl.v[i], c2);
      pv_store<KQ>(xbuf, q, p, u);
#pragma unroll
      for (int i = 0; i < 4; ++i) u.v[i] = __fmul2_rn(xr.v[i], c2);
      pv_store<KQ>(xbuf + NC * P * 2, q, p, u);
    }
    // outside partials at the children's bottoms (scale-free)
    if (!ltip) {
      PairVec o;
      pm_mul_t(o, Ml, xl);
      int E = 0;
      pv_rescale<KQ>(o, E);
      pv_store<KQ>(stk + slot_l * NC * P * 2, q, p, o);
    }
    if (!rtip) {
      PairVec o;
      pm_mul_t(o, Mr, xr);
      int E = 0;
      pv_rescale<KQ>(o, E);
      pv_store<KQ>(stk + slot_r * NC * P * 2, q, p, o);
    }
    __syncthreads();  // xbuf complete

    {  // G[c][k][i][jj] = sum_p (coef x_c)[p][i][k] * v_c[p][jj][k], rows 2uh, 2uh+1 of pair ut
      const bool tipc = uc ? rtip : ltip;
      const float2 *xs = xbuf + uc * NC * P * 2;
      const float2 *vs = uc ? kidr : kidl;
      const unsigned char *csd = stg + G.codes + uc * P;
      float2 acc[2][4];
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) acc[i][jj] = make_float2(0.0f, 0.0f);
#pragma unroll 4
      for (int m = sidx; m < rem; m += U) {
        float2 x[2], v[4];
        x[0] = xs[tq_index<KQ>(2 * uh, ut, m)];
        x[1] = xs[tq_index<KQ>(2 * uh + 1, ut, m)];
        if (tipc) {
          const float4 *tr = reinterpret_cast<const float4 *>(tab2 + int(csd[m]) * 4);
          const float4 t0 = tr[0], t1 = tr[1];
          v[0] = make_float2(t0.x, t0.y);
          v[1] = make_float2(t0.z, t0.w);
          v[2] = make_float2(t1.x, t1.y);
          v[3] = make_float2(t1.z, t1.w);
        } else {
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) v[jj] = vs[tq_index<KQ>(jj, ut, m)];
        }
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) acc[i][jj] = __ffma2_rn(x[i], v[jj], acc[i][jj]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) red[(i * 4 + jj) * (NT + 1) + tid] = acc[i][jj];
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
