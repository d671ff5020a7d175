// Codon (SP = 64) adjoint on the 5th-generation tensor cores.
//
// One CTA = (chunk of pattern tiles, node v, sample b x category k), 576
// threads; a tile is 128 patterns.  For each side c of v (child c, the other
// child c') and tile:
//   u_c[i][p] = pre_v[i][p] * (P_c' x_c')[i][p]   (outside partial of v times
//                                                  the other side's product,
//                                                  stored by the post-order)
//   GEMM3  G_c[i][j] += sum_p u_c[i][p] (coef_p x_c[j][p]), both sides in one
//          block-diagonal product: M = 128 rows (side, i), N = 128 rows
//          (side, j), K = patterns; the diagonal 64 x 64 blocks are G_l and
//          G_r, accumulated in tensor memory over all tiles of the chunk (the
//          off-diagonal blocks are not read);
//   GEMM2  o_c[p][j]  = sum_i u_c[i][p] P_c[i][j]             M = 128
//          (patterns), N = 64 (j), K = 64 (i), for internal children only:
//          the child's outside partial, rescaled by the power of two of its
//          per-pattern maximum and stored over the child's post-order partial
//          (which GEMM3 of the same side has already staged).
// Both are tcgen05.mma kind::tf32 with the split-TF32 scheme (operands as
// big + small, three products per K-step) of wide_forward_tc_kernel, and the
// same K-major no-swizzle operand layout (8-row x 16-byte core matrices, SBO
// = 128 B between 8-row groups, LBO between 4-element K groups).
//
// The work of a tile is a sequence of units: four GEMM3 units of 32
// patterns (K = 32, both sides), then for each internal child two GEMM2
// units of 32 states (K = 32) and that side's epilogue.  The CTA (one per SM)
// is warp specialised: a copy warp issues each unit's raw rows (tiles of the
// pattern-contiguous partial and product rows; GEMM3 rows with the 128-byte
// swizzle, so that a warp reading one 16-byte column of 32 rows meets no
// more bank conflicts than its 512 bytes need) as 2-D bulk tensor copies into
// a ring of three raw slots;
// sixteen converter warps turn a unit's raw rows into its MMA operands
// (products, TF32 split) and run the epilogues; an MMA warp issues the
// tensor-core work of each converted unit.  A operands (u for GEMM3, u^T for
// GEMM2: M = 128 rows = TMEM lanes, K = columns) go to tensor memory by
// tcgen05.st, in a ring of two 64-column slots; GEMM3's B operand goes to
// shared memory (K-major stores) in a ring of two operand slots.  The
// converters' issue rate and the per-unit synchronisation bound this kernel,
// so units are wide (32 patterns or states) and A in tensor memory keeps the
// A writes and reads off shared memory.  Full / empty mbarriers per slot
// order the roles; the converters meet at a named barrier only at epilogues
// and tile ends.  GEMM2's B operand, P_c transposed into the operand layout
// and split, is written once per (sample, branch, category) by
// wide_pimages_kernel; a GEMM2 unit's 32-state slice of it travels in the
// unit's raw slot (two 8 KB bulk copies) and the MMAs read it there.
//
// Tensor memory (cta_group::1, M = 128): row m is lane m, column n is column
// n, for the accumulators (G in columns [0, 128), o in [128, 192)) and for
// the A operands (slot sl in [256 + 64 sl, 256 + 64 sl + 64): TF32 big in
// the first 32 columns, small in the next 32).  A warp reads and writes the
// 32 lanes of its quarter (warp id mod 4).
#pragma once

#include <cuda.h>

#include "tt_wide_tc.cuh"

namespace tt {

namespace tcb {

constexpr int kPT = 128;                  // patterns per tile (GEMM2 M)
constexpr int kConv = 512;                // converter threads (16 warps)
constexpr int kThreads = kConv + 64;      // + the copy warp and the MMA warp
constexpr int kKC3 = 32;                  // patterns (K) per GEMM3 unit
constexpr int kKC2 = 32;                  // states (K) per GEMM2 unit
constexpr int kU3 = kPT / kKC3;           // GEMM3 units per tile (both sides)
constexpr int kU2 = 64 / kKC2;            // GEMM2 units per internal side and tile
constexpr int kOpSlot = 32768;            // one GEMM3 unit's B operand (big, small)
constexpr int kNS = 2;                    // operand slots (shared memory B, TMEM A)
constexpr int kRawSlot = 49152;           // one unit's raw rows (GEMM3: 32 patterns of 320 rows, 40 KB; GEMM2: 32 rows x 2 and the image slice)
constexpr int kNR = 3;                    // raw slots
constexpr int kMeta = kPT * 16 + 2 * kPT; // a tile's coefficients, exponents and tip codes
constexpr int kOffRaw = kNS * kOpSlot;
constexpr int kOffMeta = kOffRaw + kNR * kRawSlot;
constexpr int kOffMraw = kOffMeta + 2 * kMeta;  // the next tile's weights and site log2 L (FP64) as copied
constexpr int kOffRed = kOffMraw + 2 * kPT * 8; // float [4][128]
constexpr int kOffRoot = kOffRed + 4 * kPT * 4; // float [512] root partial sums
constexpr int kTabRows = 64;               // code-table rows held in shared memory (tip children)
constexpr int kOffTab = kOffRoot + kConv * 4;   // uint2 [kTabRows]: the rows of a 0 / 1 table as bit masks
constexpr int kOffBar = kOffTab + kTabRows * 8;
// mbarriers: raw full / empty [kNR], operand full / empty [kNS], accumulator full / empty, done
constexpr int kBars = 2 * kNR + 2 * kNS + 3;
constexpr int kSmem = kOffBar + 8 * kBars + 16;
constexpr uint32_t kTmemCols = 512;       // G (block-diagonal) [0, 128), o [128, 192), A slots [256, 384)
constexpr uint32_t kTmA = 256;            // first A-slot column
constexpr uint32_t kASlot = 64;           // columns per A slot: big [0, 32), small [32, 64)
constexpr int kImgFloats = 2 * 64 * 64;   // one P^T image: big then small

}  // namespace tcb

// Split K-major images of the transition matrices, one per (sample, branch,
// category), TF32 big then small (LBO = 1024 B between 4-element K groups):
// img_f holds P (row i, K element j: the post-order's B), img_b holds P^T
// (row j, K element i: the adjoint's GEMM2 B); either may be NULL.  One CTA
// per matrix: the matrix is read once, coalesced, into shared memory (rows
// padded to 65 floats), then both images are written with coalesced stores.
__global__ void __launch_bounds__(256) wide_pimages_kernel(const float *pmat, float *img_f, float *img_b) {
  __shared__ float sp[64 * 65];
  const long long m = blockIdx.x;
  const float4 *src = reinterpret_cast<const float4 *>(pmat + m * 4096);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int f = threadIdx.x + 256 * q, i = f >> 4, j = (f & 15) * 4;
    const float4 v = __ldg(src + f);
    sp[i * 65 + j] = v.x;
    sp[i * 65 + j + 1] = v.y;
    sp[i * 65 + j + 2] = v.z;
    sp[i * 65 + j + 3] = v.w;
  }
  __syncthreads();
#pragma unroll 4
  for (int o = threadIdx.x; o < 4096; o += 256) {
    // o (a float index) -> byte offset 4o = (kk >> 2) * 1024 + (row >> 3) * 128 + (row & 7) * 16 + (kk & 3) * 4
    const int byte = 4 * o;
    const int kk = (byte >> 10) * 4 + ((byte & 15) >> 2);
    const int row = ((byte & 1023) >> 7) * 8 + ((byte & 127) >> 4);
    float big, small;
    if (img_f) {
      tc::split_tf32(sp[row * 65 + kk], big, small);
      img_f[m * tcb::kImgFloats + o] = big;
      img_f[m * tcb::kImgFloats + 4096 + o] = small;
    }
    if (img_b) {
      tc::split_tf32(sp[kk * 65 + row], big, small);
      img_b[m * tcb::kImgFloats + o] = big;
      img_b[m * tcb::kImgFloats + 4096 + o] = small;
    }
  }
}

__device__ __forceinline__ float4 ldg4(const float *p) { return __ldg(reinterpret_cast<const float4 *>(p)); }

__device__ __forceinline__ void tmem_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// eight consecutive 32-bit TMEM columns of this thread's lane
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const float (&v)[8]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr),
               "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
               "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
               "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
               : "memory");
}

// a and b split into TF32 big and small: columns c .. c + 7 (big) and c + 32 .. c + 39 (small)
__device__ __forceinline__ void split8_tmem(uint32_t taddr, float4 a, float4 b) {
  float hb[8], hs[8];
  const float v[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
  for (int e = 0; e < 8; ++e) tc::split_tf32(v[e], hb[e], hs[e]);
  tmem_st8(taddr, hb);
  tmem_st8(taddr + 32u, hs);
}

// D (TMEM) (+)= A (TMEM, M = 128 lanes x K = 8 columns) x B (shared-memory descriptor)
__device__ __forceinline__ void mma_tf32_ta(uint32_t dtmem, uint32_t atmem, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(dtmem),
      "r"(atmem), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void split4_store(unsigned char *big, unsigned char *small, float4 v) {
  float4 hb, hs;
  tc::split_tf32(v.x, hb.x, hs.x);
  tc::split_tf32(v.y, hb.y, hs.y);
  tc::split_tf32(v.z, hb.z, hs.z);
  tc::split_tf32(v.w, hb.w, hs.w);
  *reinterpret_cast<float4 *>(big) = hb;
  *reinterpret_cast<float4 *>(small) = hs;
}

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// 2-D bulk tensor copy of the box at (x, y) of `map` into shared memory,
// completion counted on `bar`.  x (the pattern coordinate) is a multiple of
// 32 floats (128 bytes); dst is 1024-byte aligned (the 128-byte swizzle's
// period).
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// A tile's per-pattern data in shared memory.
struct TcbMeta {
  float *cf;              // [128] w_p 2^(Ep + El + Er - log2 L_p)
  int *el, *er, *ep;      // [128] exponents of x_l, x_r and of v's outside partial
  unsigned char *codes;   // [2][128] tip codes of the left / right child
};

__device__ __forceinline__ TcbMeta tcb_meta(unsigned char *base) {
  TcbMeta m;
  m.cf = reinterpret_cast<float *>(base);
  m.el = reinterpret_cast<int *>(base + 512);
  m.er = m.el + 128;
  m.ep = m.er + 128;
  m.codes = base + 2048;
  return m;
}

// Tensor maps of the adjoint's raw rows: the partials [b][I][K][64][Npad]
// and the children's products [b][I][K][2][64][Npad] as 2-D arrays of rows,
// with 32-pattern boxes of 64 partial rows / 128 product rows (GEMM3 units,
// 128-byte swizzle: the 16-byte chunk c of box row r lands at chunk
// c ^ (r & 7), address bits 4-6 XOR bits 7-9) and 128-pattern x 32-row boxes
// (GEMM2 units, no swizzle).
struct TcbMaps {
  CUtensorMap part32, prod32, part128, prod128;
};

// Barrier among the converter warps (named barrier 1) that also ORs a
// failure flag across them.
template <int NT = tcb::kConv>
__device__ __forceinline__ bool conv_sync_any(bool flag) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "bar.red.or.pred q, 1, %2, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"(flag ? 1u : 0u), "n"(NT)
      : "memory");
  return r != 0;
}

// Adjoint level kernel for FP32 codon plans: a.tiles_per_chunk / a.ntiles /
// a.nchunks count 128-pattern tiles.
__global__ void __launch_bounds__(tcb::kThreads, 1)
    wide_backward_tc_kernel(const WideArgs<float> a, const __grid_constant__ TcbMaps maps, const float *pimg,
                            int code_count, int *status, unsigned long long timeout_ns) {
  using namespace tcb;
  constexpr int SP = 64, PT = kPT;
  extern __shared__ __align__(1024) unsigned char smem[];
  float *red = reinterpret_cast<float *>(smem + kOffRed);
  float *rsum = reinterpret_cast<float *>(smem + kOffRoot);
  uint64_t *raw_full = reinterpret_cast<uint64_t *>(smem + kOffBar);  // [kNR] count 1 + bytes
  uint64_t *raw_empty = raw_full + kNR;                                // [kNR] 16 converter warps + MMA warp
  uint64_t *op_full = raw_empty + kNR;                                 // [kNS] 16 converter warps
  uint64_t *op_empty = op_full + kNS;                                  // [kNS] MMA commit
  uint64_t *acc_full = op_empty + kNS;                                 // MMA commit: a side's GEMM2 done
  uint64_t *acc_empty = acc_full + 1;                                  // 16 converter warps: o read
  uint64_t *done = acc_empty + 1;                                      // MMA commit: every MMA done
  uint32_t *tslot = reinterpret_cast<uint32_t *>(done + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // the swizzled raw rows assume a 1024-byte-aligned shared-memory window
  if (smem_u32(smem) & 1023u) {
    if (tid == 0) atomicExch(status, TT_ERR_CUDA);
    return;
  }
  const int v = a.nodes[blockIdx.y];
  const int b = blockIdx.z / a.K, k = blockIdx.z - (blockIdx.z / a.K) * a.K;
  const int chunk = blockIdx.x;
  const int l = a.left[v - a.tips], r = a.right[v - a.tips];
  const bool is_root = v == 2 * a.tips - 2;
  const double wk = a.props[size_t(b) * a.K + k];
  const size_t npad = size_t(a.Npad);
  const int vblk = ((b * a.I + (v - a.tips)) * a.K + k);  // v's (b, node, k) block of 64 rows
  const bool int0 = l >= a.tips, int1 = r >= a.tips;
  const int lblk = int0 ? (b * a.I + (l - a.tips)) * a.K + k : 0;
  const int rblk = int1 ? (b * a.I + (r - a.tips)) * a.K + k : 0;
  const int t0 = chunk * a.tiles_per_chunk, t1 = min(a.ntiles, t0 + a.tiles_per_chunk);
  const int UT = kU3 + (int0 ? kU2 : 0) + (int1 ? kU2 : 0);  // units per tile
  const int total = (t1 - t0) * UT;

  // a unit: tile index tt and position rr in the tile -> GEMM3 (idx) or GEMM2 of a side (idx)
  struct Unit {
    bool g2;
    int side, idx;
  };
  auto unit_of = [&](int rr) {
    Unit un;
    un.g2 = rr >= kU3;
    if (!un.g2) {
      un.side = 0;
      un.idx = rr;
    } else {
      const int q = rr - kU3;
      un.side = (int0 && q < kU2) ? 0 : 1;
      un.idx = q - (un.side && int0 ? kU2 : 0);
    }
    return un;
  };

  if (warp == 0) tc::tmem_alloc(tslot, kTmemCols);
  if (tid == kConv) {
    for (int i = 0; i < 2 * kNR; ++i) mbar_init(&raw_full[i], i < kNR ? 1 : 17);
    for (int i = 0; i < kNS; ++i) {
      mbar_init(&op_full[i], 16);
      mbar_init(&op_empty[i], 1);
    }
    mbar_init(acc_full, 1);
    mbar_init(acc_empty, 16);
    mbar_init(done, 1);
    fence_barrier_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const float *img0 = pimg + ((size_t(b) * a.B + l) * a.K + k) * kImgFloats;
  const float *img1 = pimg + ((size_t(b) * a.B + r) * a.K + k) * kImgFloats;

  if (warp == kConv / 32) {
    // ------------------------------------------------------------ copy warp (lane 0)
    if (lane == 0) {
      if (int0) bulk_prefetch_l2(img0, uint32_t(kImgFloats * sizeof(float)));
      if (int1) bulk_prefetch_l2(img1, uint32_t(kImgFloats * sizeof(float)));
      uint32_t ph_re = (1u << kNR) - 1u, pend_rf = 0;  // every raw slot starts free
      bool ok = true;
      int tt = 0, rr = 0;
      for (int u = 0; u < total; ++u) {
        const int rs = u % kNR;
        // the slot is free once its last unit is converted and, for a GEMM2 unit, multiplied
        ok = mbar_wait_bounded(&raw_empty[rs], ph_re >> rs & 1u, timeout_ns);
        if (!ok) break;
        ph_re ^= 1u << rs;
        // the converters wait for every earlier use of this slot before the MMA warp releases it
        pend_rf &= ~(1u << rs);
        unsigned char *raw = smem + kOffRaw + rs * kRawSlot;
        const Unit un = unit_of(rr);
        const int n0 = (t0 + tt) * PT;
        if (!un.g2) {
          const int x = n0 + un.idx * kKC3;
          mbar_arrive_expect_tx(&raw_full[rs],
                                uint32_t(16384 + 8192 * ((is_root ? 0 : 1) + (int0 ? 1 : 0) + (int1 ? 1 : 0))));
          tma_load_2d(raw, &maps.prod32, x, vblk * 2 * SP, &raw_full[rs]);
          if (!is_root) tma_load_2d(raw + 16384, &maps.part32, x, vblk * SP, &raw_full[rs]);
          if (int0) tma_load_2d(raw + 24576, &maps.part32, x, lblk * SP, &raw_full[rs]);
          if (int1) tma_load_2d(raw + 32768, &maps.part32, x, rblk * SP, &raw_full[rs]);
        } else {
          const int y = un.idx * kKC2, oblk = vblk * 2 + (1 - un.side);
          mbar_arrive_expect_tx(&raw_full[rs], uint32_t(16384 * (2 + (is_root ? 0 : 1))));
          tma_load_2d(raw, &maps.prod128, n0, oblk * SP + y, &raw_full[rs]);
          if (!is_root) tma_load_2d(raw + 16384, &maps.part128, n0, vblk * SP + y, &raw_full[rs]);
          // the unit's 32-state slice of the P^T image (K groups 8 idx .. 8 idx + 7), big and small
          const float *src = (un.side ? img1 : img0) + un.idx * 2048;
          bulk_copy_g2s(raw + 32768, src, 8192u, &raw_full[rs]);
          bulk_copy_g2s(raw + 40960, src + 4096, 8192u, &raw_full[rs]);
        }
        pend_rf |= 1u << rs;
        if (++rr == UT) {
          rr = 0;
          ++tt;
        }
      }
      if (!ok) {
        atomicExch(status, kDeviceTimeout);
        for (int rs = 0; rs < kNR; ++rs)  // copies in flight land before the CTA exits
          if (pend_rf >> rs & 1u) mbar_wait_bounded(&raw_full[rs], (ph_re >> rs & 1u) ^ 1u, 100000000ull);
      }
    }
    __syncwarp();
  } else if (warp == kConv / 32 + 1) {
    // ------------------------------------------------------------ MMA warp (the whole warp runs the
    // loop, lane 0 issues)
    const bool leader = lane == 0;
    // operand descriptors: slot / raw-slot bases, advanced by (byte offset >> 4) per K step
    const uint64_t dOp = tc::smem_desc(smem_u32(smem), 2048, 128);         // GEMM3 B (operand slots)
    const uint64_t dB = tc::smem_desc(smem_u32(smem + kOffRaw), 1024, 128);  // GEMM2 B (image in the raw slot)
    uint32_t ph_of = 0, ph_ae = 1u;
    bool ok = true, started = false;
    int rr = 0;
    for (int u = 0; u < total && ok; ++u) {
      const int rs = u % kNR, sl = u % kNS;
      const Unit un = unit_of(rr);
      ok = __all_sync(0xffffffffu, mbar_wait_bounded(&op_full[sl], ph_of >> sl & 1u, timeout_ns));
      if (!ok) break;
      ph_of ^= 1u << sl;
      if (un.g2 && un.idx == 0) {  // the previous epilogue has read o
        ok = __all_sync(0xffffffffu, mbar_wait_bounded(acc_empty, ph_ae, timeout_ns));
        if (!ok) break;
        ph_ae ^= 1u;
      }
      tc::fence_after_sync();
      const uint64_t so = uint64_t(sl * kOpSlot) >> 4, ro = uint64_t(rs * kRawSlot) >> 4;
      const uint32_t ta = tmem + kTmA + kASlot * uint32_t(sl);  // the unit's A: big at ta, small at ta + 32
      if (leader) {
        if (!un.g2) {
          constexpr uint32_t idesc = tc::idesc_tf32(128, 128);
#pragma unroll
          for (int kk = 0; kk < kKC3 / 8; ++kk) {
            const uint64_t o = so + uint64_t(kk * 4096 >> 4);
            const uint32_t at = ta + 8u * kk;
            mma_tf32_ta(tmem, at, dOp + o, idesc, (started || kk > 0) ? 1u : 0u);
            mma_tf32_ta(tmem, at, dOp + o + (16384 >> 4), idesc, 1u);
            mma_tf32_ta(tmem, at + 32u, dOp + o, idesc, 1u);
          }
          tc::mma_commit(&op_empty[sl]);
          mbar_arrive(&raw_empty[rs]);  // the MMAs do not read the raw slot
        } else {
          constexpr uint32_t idesc = tc::idesc_tf32(128, 64);
#pragma unroll
          for (int kk = 0; kk < kKC2 / 8; ++kk) {
            const uint64_t ob = ro + uint64_t(32768 + kk * 2048 >> 4);
            const uint32_t at = ta + 8u * kk;
            mma_tf32_ta(tmem + 128u, at, dB + ob, idesc, (un.idx > 0 || kk > 0) ? 1u : 0u);
            mma_tf32_ta(tmem + 128u, at, dB + ob + (8192 >> 4), idesc, 1u);
            mma_tf32_ta(tmem + 128u, at + 32u, dB + ob, idesc, 1u);
          }
          tc::mma_commit(&op_empty[sl]);
          tc::mma_commit(&raw_empty[rs]);  // the raw slot held B
          if (un.idx == kU2 - 1) tc::mma_commit(acc_full);  // the side's o is complete
        }
      }
      __syncwarp();
      if (!un.g2) started = true;
      if (++rr == UT) rr = 0;
    }
    if (leader) {
      tc::mma_commit(done);  // every MMA issued so far
      if (!ok) atomicExch(status, kDeviceTimeout);
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------------ converter warps
    double *mw = reinterpret_cast<double *>(smem + kOffMraw), *ml2 = mw + PT;
    auto fetch_meta = [&](int t, TcbMeta m) {  // cp.async into buffer m (pattern tid; codes four per copy)
      const int n = t * PT + (tid & (PT - 1));
      if (tid < PT) {
        if (!is_root) cp_async4(&m.ep[tid], a.expo + size_t(vblk) * npad + n);
        if (int0) cp_async4(&m.el[tid], a.expo + size_t(lblk) * npad + n);
        if (int1) cp_async4(&m.er[tid], a.expo + size_t(rblk) * npad + n);
        if (n < a.N) {  // padding patterns have neither (log2 L is written for n < N only)
          cp_async8(&mw[tid], a.weights + n);
          cp_async8(&ml2[tid], a.log2L + size_t(b) * npad + n);
        }
      } else if (tid < PT + 64) {
        const int sd = (tid - PT) >> 5, t4 = (tid - PT) & 31;
        if (!(sd ? int1 : int0))
          cp_async4(m.codes + sd * PT + 4 * t4, a.codes + size_t(sd ? r : l) * a.code_stride + t * PT + 4 * t4);
      }
      cp_async_commit();
    };
    auto finish_meta = [&](int t, TcbMeta m) {  // own copies landed: zeros for tips / root, coefficient
      if (tid < PT) {
        const int n = t * PT + tid;
        const int Ep = is_root ? 0 : m.ep[tid], El = int0 ? m.el[tid] : 0, Er = int1 ? m.er[tid] : 0;
        m.ep[tid] = Ep;
        m.el[tid] = El;
        m.er[tid] = Er;
        // w 2^(E - log2 L): the exponent difference in FP64, its fraction's power in FP32 (an FP64
        // exp2 costs thousands of cycles of this GPU's FP64 pipe per warp)
        const double dd = double(Ep + El + Er) - ml2[tid], fl = floor(dd);
        m.cf[tid] = n < a.N ? ldexpf(float(mw[tid]) * exp2f(float(dd - fl)), int(fl)) : 0.0f;
      }
    };
    // a tip child's rows of the code table: as bit masks in shared memory when every entry is 0 or 1
    // (the encodings' indicator rows) and the table is small, else read from global memory
    uint2 *tabm = reinterpret_cast<uint2 *>(smem + kOffTab);
    bool tab_bits = (!int0 || !int1) && code_count <= kTabRows;
    if (tab_bits) {
      bool binary = true;
      for (int e = tid; e < code_count * 2; e += kConv) {  // row e >> 1, states 32 (e & 1) .. + 31
        const float *row = a.table + (e >> 1) * SP + 32 * (e & 1);
        uint32_t m = 0;
#pragma unroll 8
        for (int j = 0; j < 32; ++j) {
          const float t = __ldg(row + j);
          binary = binary && (t == 0.0f || t == 1.0f);
          m |= (t == 1.0f ? 1u : 0u) << j;
        }
        if (e & 1) tabm[e >> 1].y = m;
        else tabm[e >> 1].x = m;
      }
      tab_bits = !conv_sync_any(!binary);
    }
    // x of tip code c at state i
    auto tipx = [&](int c, int i) -> float {
      if (tab_bits) {
        const uint2 m = tabm[c];
        return ((i < 32 ? m.x >> i : m.y >> (i - 32)) & 1u) ? 1.0f : 0.0f;
      }
      return __ldg(a.table + c * SP + i);
    };
    // GEMM3 item of this thread: row R3 = (side s3, state i3) = its TMEM lane (32 (warp & 3) + lane),
    // patterns 8 q3 .. 8 q3 + 7 of the unit (q3 = warp >> 2, the row's 16-byte chunks 2 q3 and
    // 2 q3 + 1).  It writes u[R3][..] (A) to tensor memory and (c x)[R3][..] (B) to eight rows of
    // one core matrix per quarter warp; the raw rows' 128-byte swizzle moves chunk c of row r to
    // c ^ (r & 7).
    const int R3 = 32 * (warp & 3) + lane, q3 = warp >> 2;
    const int s3 = R3 >> 6, i3 = R3 & 63;
    const int sw3a = 16 * ((2 * q3) ^ (i3 & 7)), sw3b = 16 * ((2 * q3 + 1) ^ (i3 & 7));  // rows i3, 64 + i3
    const bool x3in = s3 ? int1 : int0;
    const float pre3 = is_root && i3 < a.S ? float(wk * a.freqs[size_t(b) * a.S + i3]) : 0.0f;
    // this warp's lane quarter of tensor memory
    const uint32_t tq = tmem + (uint32_t(32 * (warp & 3)) << 16);
    uint32_t ph_rf = 0, ph_oe = (1u << kNS) - 1u, ph_af = 0;  // every operand slot starts free
    bool ok = true;        // uniform across the converters after every conv_sync_any
    float root_acc = 0.0f; // root: this thread's share of sum_p c_p al[i][p] ar[i][p], i = tid & 63
    if (t0 < t1) {
      fetch_meta(t0, tcb_meta(smem + kOffMeta));
      cp_async_wait<0>();
      finish_meta(t0, tcb_meta(smem + kOffMeta));
    }
    ok = !conv_sync_any(!ok);
    int tt = 0, rr = 0;
    for (int u = 0; u < total; ++u) {
      const Unit un = unit_of(rr);
      const int tile = t0 + tt, n0 = tile * PT;
      const TcbMeta meta = tcb_meta(smem + kOffMeta + (tt & 1) * kMeta);
      if (ok && rr == 0) {
        if (tile + 1 < t1) fetch_meta(tile + 1, tcb_meta(smem + kOffMeta + ((tt + 1) & 1) * kMeta));
        if (is_root) {  // R[i][p] = c_p al[i][p] ar[i][p]: row i = tid & 63, patterns 4 (tid >> 6 + 8 m) ..
          const float *pb = a.prod + size_t(vblk) * 2 * SP * npad;
          const int i = tid & 63;
#pragma unroll
          for (int m = 0; m < 4; ++m) {
            const int quad = (tid >> 6) + 8 * m;
            const float4 al = ldg4(pb + size_t(i) * npad + n0 + 4 * quad);
            const float4 ar = ldg4(pb + size_t(SP + i) * npad + n0 + 4 * quad);
            const float4 c4 = *reinterpret_cast<const float4 *>(meta.cf + 4 * quad);
            root_acc += c4.x * al.x * ar.x + c4.y * al.y * ar.y + c4.z * al.z * ar.z + c4.w * al.w * ar.w;
          }
        }
      }
      const int rs = u % kNR, sl = u % kNS;
      if (ok) ok = mbar_wait_bounded(&raw_full[rs], ph_rf >> rs & 1u, timeout_ns);   // the unit's rows landed
      if (ok) ok = mbar_wait_bounded(&op_empty[sl], ph_oe >> sl & 1u, timeout_ns);  // the slot is free
      ok = __all_sync(0xffffffffu, ok);  // the tcgen05.st below are warp-collective
      ph_rf ^= 1u << rs;
      ph_oe ^= 1u << sl;
      if (ok) {
        tc::fence_after_sync();  // the MMAs that read this slot's A have completed
        unsigned char *op = smem + sl * kOpSlot;
        const unsigned char *raw = smem + kOffRaw + rs * kRawSlot;
        const uint32_t ta = tq + kTmA + kASlot * uint32_t(sl);
        if (!un.g2) {
          const int pt = un.idx * kKC3 + 8 * q3;  // pattern offset in the tile
          // u_s = pre * (the other side's product): product rows (1 - s) * 64 + i
          const unsigned char *orow = raw + ((1 - s3) * 64 + i3) * 128, *prow = raw + 16384 + i3 * 128;
          const float4 oa = *reinterpret_cast<const float4 *>(orow + sw3a);
          const float4 ob = *reinterpret_cast<const float4 *>(orow + sw3b);
          const float4 pa = is_root ? make_float4(pre3, pre3, pre3, pre3) : *reinterpret_cast<const float4 *>(prow + sw3a);
          const float4 pb = is_root ? make_float4(pre3, pre3, pre3, pre3) : *reinterpret_cast<const float4 *>(prow + sw3b);
          float4 xa, xb;
          if (x3in) {
            const unsigned char *xrow = raw + 24576 + s3 * 8192 + i3 * 128;
            xa = *reinterpret_cast<const float4 *>(xrow + sw3a);
            xb = *reinterpret_cast<const float4 *>(xrow + sw3b);
          } else {
            const unsigned char *cc = meta.codes + s3 * PT + pt;
            xa = make_float4(tipx(cc[0], i3), tipx(cc[1], i3), tipx(cc[2], i3), tipx(cc[3], i3));
            xb = make_float4(tipx(cc[4], i3), tipx(cc[5], i3), tipx(cc[6], i3), tipx(cc[7], i3));
          }
          const float4 ca = *reinterpret_cast<const float4 *>(meta.cf + pt);
          const float4 cb = *reinterpret_cast<const float4 *>(meta.cf + pt + 4);
          split8_tmem(ta + 8u * q3, make_float4(pa.x * oa.x, pa.y * oa.y, pa.z * oa.z, pa.w * oa.w),
                      make_float4(pb.x * ob.x, pb.y * ob.y, pb.z * ob.z, pb.w * ob.w));
          const uint32_t offa = tc::kmajor_off(R3, 8 * q3, 2048), offb = tc::kmajor_off(R3, 8 * q3 + 4, 2048);
          split4_store(op + offa, op + 16384 + offa, make_float4(xa.x * ca.x, xa.y * ca.y, xa.z * ca.z, xa.w * ca.w));
          split4_store(op + offb, op + 16384 + offb, make_float4(xb.x * cb.x, xb.y * cb.y, xb.z * cb.z, xb.w * cb.w));
        } else {
          // item (pattern p = this thread's TMEM lane, states 32 idx + 8 sq ..): A = u^T, row p, K = 8 states
          const int pp = tid & (PT - 1), sq = tid >> 7;
          float uu[8];
#pragma unroll
          for (int e = 0; e < 8; ++e) {
            const int row = 8 * sq + e, i = un.idx * kKC2 + row;
            const float ot = *reinterpret_cast<const float *>(raw + row * 512 + pp * 4);
            const float pv = is_root ? (i < a.S ? float(wk * a.freqs[size_t(b) * a.S + i]) : 0.0f)
                                     : *reinterpret_cast<const float *>(raw + 16384 + row * 512 + pp * 4);
            uu[e] = pv * ot;
          }
          split8_tmem(ta + 8u * sq, make_float4(uu[0], uu[1], uu[2], uu[3]), make_float4(uu[4], uu[5], uu[6], uu[7]));
        }
        tmem_st_wait();
        if (!un.g2) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // B: generic writes -> tensor cores
        tc::fence_before_sync();
        __syncwarp();
        if (lane == 0) {
          mbar_arrive(&op_full[sl]);
          mbar_arrive(&raw_empty[rs]);
        }
      }
      if (un.g2 && un.idx == kU2 - 1) {  // the side's outside partials: o = P_c^T u, rescaled, over x_c
        const int side = un.side;
        if (ok) ok = mbar_wait_bounded(acc_full, ph_af, timeout_ns);
        ph_af ^= 1u;
        tc::fence_after_sync();
        const int cblk = side ? rblk : lblk;
        const int qd = warp & 3, cg = warp >> 2, pp = 32 * qd + lane;  // columns [16 cg, 16 cg + 16)
        uint32_t rg[16];
        float mx = 0.0f;
        if (ok) {
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
              : "=r"(rg[0]), "=r"(rg[1]), "=r"(rg[2]), "=r"(rg[3]), "=r"(rg[4]), "=r"(rg[5]), "=r"(rg[6]),
                "=r"(rg[7]), "=r"(rg[8]), "=r"(rg[9]), "=r"(rg[10]), "=r"(rg[11]), "=r"(rg[12]), "=r"(rg[13]),
                "=r"(rg[14]), "=r"(rg[15])
              : "r"(tmem + (uint32_t(32 * qd) << 16) + 128u + uint32_t(16 * cg)));
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int jj = 0; jj < 16; ++jj) mx = fmaxf(mx, __uint_as_float(rg[jj]));
          red[cg * PT + pp] = mx;
        }
        tc::fence_before_sync();
        __syncwarp();
        if (lane == 0) mbar_arrive(acc_empty);  // o is in registers: the next side's GEMM2 may overwrite it
        ok = !conv_sync_any(!ok);
        if (ok) {
          const int e =
              scale_exponent(fmaxf(fmaxf(red[pp], red[PT + pp]), fmaxf(red[2 * PT + pp], red[3 * PT + pp])));
          float *dst = a.part + size_t(cblk) * SP * npad + n0 + pp;
#pragma unroll
          for (int jj = 0; jj < 16; ++jj) dst[size_t(16 * cg + jj) * npad] = times_pow2_neg(__uint_as_float(rg[jj]), e);
          if (cg == 0) a.expo[size_t(cblk) * npad + n0 + pp] = meta.ep[pp] + (side ? meta.el[pp] : meta.er[pp]) + e;
        }
        ok = !conv_sync_any(!ok);  // red is reused
        if (!ok) break;
      }
      if (rr == UT - 1 && tile + 1 < t1) {  // the next tile's per-pattern data
        cp_async_wait<0>();
        if (ok) finish_meta(tile + 1, tcb_meta(smem + kOffMeta + ((tt + 1) & 1) * kMeta));
        ok = !conv_sync_any(!ok);
        if (!ok) break;
      }
      if (++rr == UT) {
        rr = 0;
        ++tt;
      }
    }
    cp_async_wait<0>();  // no copy into this CTA's shared memory is left in flight
    ok = !conv_sync_any(!ok);
    const bool fin = mbar_wait_bounded(done, 0, timeout_ns);  // every MMA is complete
    tc::fence_after_sync();
    ok = !conv_sync_any(!(ok && fin));
    if (ok) {
      // the chunk's gradient blocks: G_side row i = lane quarter 32 (w & 3) + lane - 64 side,
      // side = (w & 3) >> 1, columns 64 side + [16 cg, 16 cg + 16)
      const int qd = warp & 3, cg = warp >> 2, side = qd >> 1, i = (32 * qd + lane) & 63;
      uint32_t rg[16];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(rg[0]), "=r"(rg[1]), "=r"(rg[2]), "=r"(rg[3]), "=r"(rg[4]), "=r"(rg[5]), "=r"(rg[6]),
            "=r"(rg[7]), "=r"(rg[8]), "=r"(rg[9]), "=r"(rg[10]), "=r"(rg[11]), "=r"(rg[12]), "=r"(rg[13]),
            "=r"(rg[14]), "=r"(rg[15])
          : "r"(tmem + (uint32_t(32 * qd) << 16) + uint32_t(64 * side + 16 * cg)));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      float *dst = a.gpart + (((size_t(b) * a.B + (side ? r : l)) * a.nchunks + chunk) * a.K + k) * SP * SP +
                   i * SP + 16 * cg;
#pragma unroll
      for (int jj = 0; jj < 16; jj += 4)
        *reinterpret_cast<float4 *>(dst + jj) = make_float4(__uint_as_float(rg[jj]), __uint_as_float(rg[jj + 1]),
                                                             __uint_as_float(rg[jj + 2]), __uint_as_float(rg[jj + 3]));
      if (is_root) {  // dlnL/dpi rows (times w_k) and dlnL/dw_k of the chunk, fixed order
        rsum[tid] = root_acc;
        conv_sync_any(false);
        float *dr = a.rootpart + ((size_t(b) * a.nchunks + chunk) * a.K + k) * (SP + 1);
        if (tid < SP) {  // the eight threads of row i: i + 64 j
          float s = 0.0f;
#pragma unroll
          for (int jr = 0; jr < 8; ++jr) s += rsum[tid + 64 * jr];
          red[tid] = s;
          dr[tid] = float(wk) * s;
        }
        conv_sync_any(false);
        if (tid == 0) {
          float s = 0.0f;
          for (int ii = 0; ii < a.S; ++ii) s += float(a.freqs[size_t(b) * a.S + ii]) * red[ii];
          dr[SP] = s;
        }
      }
    } else if (tid == 0) {
      atomicExch(status, kDeviceTimeout);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

}  // namespace tt
