// Codon (SP = 64) post-order contraction on the 5th-generation tensor cores.
//
// One CTA = (node, category, tile of 128 patterns), 128 threads.  Per side c
// the product  D_c[p][i] = sum_j x_c[j][p] P_c[i][j]  is an M = 128
// (patterns) x N = 64 (states) x K = 64 (states) matrix product issued as
// tcgen05.mma kind::tf32 by one thread, accumulated in tensor memory (TMEM
// columns [64c, 64c + 64), lane = pattern).  FP32 accuracy comes from the
// split-TF32 scheme: every operand is written as big + small with
// big = tf32(v), small = tf32(v - big), and D = Ab Bb + Ab Bs + As Bb.
//
// Operands are staged in shared memory in the canonical K-major layout
// without swizzle: 8-row x 16-byte core matrices, rows 16 B apart, the next
// 8 rows SBO = 128 B further, the next 4 K-elements LBO further.
//   A (x^T, 128 x 64): LBO = 2048 B,  one MMA K-step (8 elements) = 4096 B
//   B (P,    64 x 64): LBO = 1024 B,  one MMA K-step               = 2048 B
// The two sides are staged one after the other in the same 96 KB (the
// second once the first side's MMAs have completed), so that two CTAs fit
// per SM and one CTA's staging overlaps the other's MMAs and epilogue.
// After the MMAs complete (tcgen05.commit -> mbarrier, bounded wait) each
// thread loads its pattern's 64 + 64 accumulators with tcgen05.ld, forms
// the product, rescales by the power of two of its maximum and stores the
// partial exactly as wide_forward_kernel does.
#pragma once

#include "tt_wide.cuh"

namespace tt {

namespace tc {

constexpr int kPT = 128;                 // patterns per CTA (MMA M)
constexpr int kThreads = 128;
constexpr int kAbytes = 128 * 64 * 4;    // one A operand (big or small)
constexpr int kBbytes = 64 * 64 * 4;     // one B operand
// shared memory (one side at a time): [B: P big, P small][A: x big, x small][barrier, tmem slot]
constexpr int kOffB = 0;
constexpr int kOffA = 2 * kBbytes;
constexpr int kOffBar = kOffA + 2 * kAbytes;
constexpr int kSmem = kOffBar + 64;
constexpr uint32_t kTmemCols = 128;

__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  // D = F32 (bits 4-5 = 1), A = B = TF32 (bits 7-9, 10-12 = 2), both K-major,
  // N >> 3 at bits 17-22, M >> 4 at bits 24-28
  return (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  // start address, leading / stride byte offsets (all >> 4), version 1, no swizzle
  return uint64_t((saddr >> 4) & 0x3FFF) | (uint64_t((lbo >> 4) & 0x3FFF) << 16) |
         (uint64_t((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// byte offset of element (row, k) in a K-major no-swizzle operand with LBO `lbo`
__device__ __forceinline__ uint32_t kmajor_off(int row, int k, uint32_t lbo) {
  return uint32_t(k >> 2) * lbo + uint32_t(row >> 3) * 128u + uint32_t(row & 7) * 16u + uint32_t(k & 3) * 4u;
}

__device__ __forceinline__ float tf32_round(float v) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
  return __uint_as_float(r);
}

__device__ __forceinline__ void split_tf32(float v, float &big, float &small) {
  big = tf32_round(v);
  small = tf32_round(v - big);
}

__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(cols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 32 consecutive accumulator columns of this warp's 32 lanes
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc

// Post-order level kernel for FP32 codon plans on the tensor cores.
// pimg: split P images (row i, K element j, big then small; wide_pimages_kernel),
// one 32 KB bulk copy per side; NULL stages P by the
// threads.  The second side's child values are loaded into registers while
// the first side's MMAs run.  A CTA walks a.tiles_per_chunk tiles of one
// (node, sample, category), reusing its TMEM and barriers.
__global__ void __launch_bounds__(tc::kThreads, 2) wide_forward_tc_kernel(const WideArgs<float> a, const float *pimg,
                                                                         int *status, unsigned long long timeout_ns) {
  constexpr int SP = 64;
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char *sB = smem + tc::kOffB;
  unsigned char *sA = smem + tc::kOffA;
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem + tc::kOffBar);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + tc::kOffBar + 8);
  uint64_t *bar_b = reinterpret_cast<uint64_t *>(smem + tc::kOffBar + 16);  // the image copy
  const int tid = threadIdx.x, warp = tid >> 5;
  const int v = a.nodes[blockIdx.y];
  const int b = blockIdx.z / a.K, k = blockIdx.z - (blockIdx.z / a.K) * a.K;
  // this CTA's 128-pattern tiles [t0, t1): TMEM, barriers and set-up paid once for them
  const int t0 = blockIdx.x * a.tiles_per_chunk, t1 = min(a.ntiles, t0 + a.tiles_per_chunk);
  int n0 = t0 * tc::kPT;
  const int l = a.left[v - a.tips], r = a.right[v - a.tips];
  const bool is_root = v == 2 * a.tips - 2;

  if (warp == 0) tc::tmem_alloc(tslot, tc::kTmemCols);
  if (tid == 0) {
    mbar_init(bar, 1);
    mbar_init(bar_b, 1);
    fence_barrier_init();
  }
  __syncthreads();  // barriers initialised before the first copy
  // per side c: stage, then one thread issues the side's MMAs into TMEM
  // columns [64c, 64c + 64); the next side's staging waits for their completion
  bool ok = true;
  int phase = 0, phase_b = 0;
  bool b_pending = false;  // thread 0: an image copy whose completion it has not seen
  uint32_t tmem = 0;  // read from the slot after the first barrier
  // the A operand values of a side: x_c^T, M = pattern (this thread's), K = j, all 64 loads in
  // flight at once; the second side's are issued while the first side's MMAs run
  float xv[SP];
  auto load_x = [&](int child) {
    if (child < a.tips) {
      const int code = a.codes[size_t(child) * a.code_stride + n0 + tid];
      const float4 *row = reinterpret_cast<const float4 *>(a.table + size_t(code) * SP);
#pragma unroll
      for (int j = 0; j < SP; j += 4) {
        const float4 t4 = __ldg(row + j / 4);
        xv[j] = t4.x, xv[j + 1] = t4.y, xv[j + 2] = t4.z, xv[j + 3] = t4.w;
      }
    } else {
      const float *src = a.part + ((size_t(b) * a.I + (child - a.tips)) * a.K + k) * SP * size_t(a.Npad) + n0 + tid;
#pragma unroll
      for (int j = 0; j < SP; ++j) xv[j] = __ldg(src + size_t(j) * a.Npad);
    }
  };
  for (int tile = t0; tile < t1 && ok; ++tile) {
    n0 = tile * tc::kPT;
    load_x(l);
    for (int c = 0; c < 2 && ok; ++c) {
      const int child = c ? r : l;
      // B operand: P_c[i][j], N = i, K = j: the split image in one bulk copy, or
      // eight 16-byte loads per thread in flight before the split
      if (pimg) {
        if (tid == 0) {
          b_pending = true;
          mbar_arrive_expect_tx(bar_b, uint32_t(2 * tc::kBbytes));
          bulk_copy_g2s(sB, pimg + ((size_t(b) * a.B + child) * a.K + k) * 2 * SP * SP, uint32_t(2 * tc::kBbytes),
                        bar_b);
        }
      } else {
        float4 pv[8];
#pragma unroll
        for (int m = 0; m < 8; ++m) {
          const int f = (tid + m * tc::kThreads) * 4, i = f / SP;
          pv[m] = __ldg(reinterpret_cast<const float4 *>(
              a.pmat + ((size_t(b) * a.B + child) * a.K + k) * SP * SP + (f - i * SP) + i * SP));
        }
#pragma unroll
        for (int m = 0; m < 8; ++m) {
          const int f = (tid + m * tc::kThreads) * 4, i = f / SP, j = f - i * SP;
          float4 hb, hs;
          tc::split_tf32(pv[m].x, hb.x, hs.x);
          tc::split_tf32(pv[m].y, hb.y, hs.y);
          tc::split_tf32(pv[m].z, hb.z, hs.z);
          tc::split_tf32(pv[m].w, hb.w, hs.w);
          const uint32_t off = tc::kmajor_off(i, j, 1024);
          *reinterpret_cast<float4 *>(sB + off) = hb;
          *reinterpret_cast<float4 *>(sB + tc::kBbytes + off) = hs;
        }
      }
      // A operand: the side's loaded values split, four j per 16-byte store
      {
#pragma unroll
        for (int j = 0; j < SP; j += 4) {
          float4 hb, hs;
          tc::split_tf32(xv[j], hb.x, hs.x);
          tc::split_tf32(xv[j + 1], hb.y, hs.y);
          tc::split_tf32(xv[j + 2], hb.z, hs.z);
          tc::split_tf32(xv[j + 3], hb.w, hs.w);
          const uint32_t off = tc::kmajor_off(tid, j, 2048);
          *reinterpret_cast<float4 *>(sA + off) = hb;
          *reinterpret_cast<float4 *>(sA + tc::kAbytes + off) = hs;
        }
      }
      // generic-proxy writes -> visible to the tensor cores (async proxy)
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      tc::fence_before_sync();
      __syncthreads();
      tc::fence_after_sync();
      tmem = *tslot;
      if (tid == 0 && b_pending) {  // the image has landed
        if (mbar_wait_bounded(bar_b, phase_b, timeout_ns)) {
          b_pending = false;
          phase_b ^= 1;
        }
      }
      if (tid == 0 && !b_pending) {
        constexpr uint32_t idesc = tc::idesc_tf32(128, 64);
        const uint32_t d = tmem + uint32_t(64 * c);
        const uint32_t ab = smem_u32(sA), as = ab + tc::kAbytes;
        const uint32_t bb = smem_u32(sB), bs = bb + tc::kBbytes;
#pragma unroll
        for (int kk = 0; kk < SP / 8; ++kk) {
          const uint64_t dab = tc::smem_desc(ab + kk * 4096, 2048, 128), das = tc::smem_desc(as + kk * 4096, 2048, 128);
          const uint64_t dbb = tc::smem_desc(bb + kk * 2048, 1024, 128), dbs = tc::smem_desc(bs + kk * 2048, 1024, 128);
          tc::mma_tf32(d, dab, dbb, idesc, kk > 0 ? 1u : 0u);
          tc::mma_tf32(d, dab, dbs, idesc, 1u);
          tc::mma_tf32(d, das, dbb, idesc, 1u);
        }
        tc::mma_commit(bar);
      } else if (tid == 0) {
        mbar_arrive(bar);  // no MMAs (the image never landed): complete the phase; the side fails below
      }
      if (c == 0) load_x(r);  // while the MMAs run: the other side's values into registers
      // every thread sees the side's MMAs complete before the shared memory is restaged or TMEM read
      ok = mbar_wait_bounded(bar, phase, timeout_ns) && !(tid == 0 && b_pending);
      tc::fence_after_sync();
      ok = !__syncthreads_or(!ok);
      if (ok) phase ^= 1;
    }
    if (ok) {
      // this thread's pattern = TMEM lane 32 * warp + lane
      const uint32_t lane_addr = tmem + (uint32_t(32 * warp) << 16);
      const int n = n0 + tid;
      float *pd = a.prod ? a.prod + ((size_t(b) * a.I + (v - a.tips)) * a.K + k) * 2 * SP * size_t(a.Npad) + n
                         : nullptr;
      float L[64];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        float dl[32], dr[32];
        tc::tmem_ld32(lane_addr + uint32_t(32 * h), dl);
        tc::tmem_ld32(lane_addr + uint32_t(64 + 32 * h), dr);
        if (pd) {  // the children's products for the adjoint
#pragma unroll
          for (int i = 0; i < 32; ++i) {
            pd[size_t(32 * h + i) * a.Npad] = dl[i];
            pd[size_t(SP + 32 * h + i) * a.Npad] = dr[i];
          }
        }
#pragma unroll
        for (int i = 0; i < 32; ++i) L[32 * h + i] = dl[i] * dr[i];
      }
      const int El = wide_child_expo(a, l, b, k, n), Er = wide_child_expo(a, r, b, k, n);
      if (is_root) {
        double s = 0.0;
#pragma unroll
        for (int i = 0; i < 64; ++i)
          if (i < a.S) s = fma(a.freqs[size_t(b) * a.S + i], double(L[i]), s);
        const size_t o = (size_t(b) * a.K + k) * a.Npad + n;
        a.root_site[o] = s;
        a.root_expo[o] = El + Er;
      } else {
        int e = 0;
        if (a.rescale) {
          float m = 0.0f;
#pragma unroll
          for (int i = 0; i < 64; ++i) m = fmaxf(m, L[i]);
          e = scale_exponent(m);
#pragma unroll
          for (int i = 0; i < 64; ++i) L[i] = times_pow2_neg(L[i], e);
        }
        float *dst = a.part + ((size_t(b) * a.I + (v - a.tips)) * a.K + k) * SP * size_t(a.Npad) + n;
#pragma unroll
        for (int i = 0; i < 64; ++i) dst[size_t(i) * a.Npad] = L[i];
        a.expo[((size_t(b) * a.I + (v - a.tips)) * a.K + k) * a.Npad + n] = El + Er + e;
      }
    }
  }  // tiles
  if (!ok) {
    if (tid == 0) {
      atomicExch(status, kDeviceTimeout);
      if (b_pending) mbar_wait_bounded(bar_b, phase_b, 100000000ull);  // the image copy lands before exit
    }
    mbar_wait_bounded(bar, phase, 100000000ull);  // give the tensor cores a last chance before freeing TMEM
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, tc::kTmemCols);
}

}  // namespace tt
