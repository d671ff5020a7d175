// Shared device helpers: mbarrier + bulk-copy (TMA) PTX wrappers, bounded
// waits, vector moves, power-of-two rescaling and warp reductions.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace tt {

// Device status codes written by kernels (mirror tt_status).
constexpr int kDeviceTimeout = 5;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

// Make barrier initialisation visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Non-blocking probe of a barrier phase.
__device__ __forceinline__ bool mbar_test_wait(uint64_t *bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ uint64_t global_timer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wait for a barrier phase with a wall-clock limit; false when it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity,
                                                  uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_timer_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (global_timer_ns() - t0 > limit_ns) return false;
  }
  return true;
}

// Wait by polling (no suspension) with a wall-clock limit; false when it gave up.
__device__ __forceinline__ bool mbar_spin_bounded(uint64_t *bar, uint32_t parity, uint64_t limit_ns) {
  if (mbar_test_wait(bar, parity)) return true;
  const uint64_t t0 = global_timer_ns();
  while (!mbar_test_wait(bar, parity)) {
    if (global_timer_ns() - t0 > limit_ns) return false;
  }
  return true;
}

// 1-D bulk copy global -> shared (TMA engine), completion counted on `bar`.
// Both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes,
                                              uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Bulk prefetch of global memory into L2 (TMA engine, no completion to wait
// for).  Address 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_prefetch_l2(const void *src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// ---------------------------------------------------------------- vectors
template <typename T>
struct Vec16;  // 16-byte packet of T
template <>
struct Vec16<float> {
  using type = float4;
  static constexpr int n = 4;
};
template <>
struct Vec16<double> {
  using type = double2;
  static constexpr int n = 2;
};

template <typename T, int S>
__device__ __forceinline__ void load_vec(T (&v)[S], const T *p) {
  static_assert((S * sizeof(T)) % 16 == 0, "S-vector must be a whole number of 16-byte packets");
  using P = typename Vec16<T>::type;
  constexpr int W = Vec16<T>::n;
  const P *q = reinterpret_cast<const P *>(p);
#pragma unroll
  for (int c = 0; c < S / W; ++c) {
    P x = q[c];
    const T *xs = reinterpret_cast<const T *>(&x);
#pragma unroll
    for (int w = 0; w < W; ++w) v[c * W + w] = xs[w];
  }
}

template <typename T, int S>
__device__ __forceinline__ void store_vec(T *p, const T (&v)[S]) {
  using P = typename Vec16<T>::type;
  constexpr int W = Vec16<T>::n;
  P *q = reinterpret_cast<P *>(p);
#pragma unroll
  for (int c = 0; c < S / W; ++c) {
    P x;
    T *xs = reinterpret_cast<T *>(&x);
#pragma unroll
    for (int w = 0; w < W; ++w) xs[w] = v[c * W + w];
    q[c] = x;
  }
}

// Streaming (evict-first) global store / load of an S-vector.
template <typename T, int S>
__device__ __forceinline__ void store_vec_stream(T *p, const T (&v)[S]) {
  using P = typename Vec16<T>::type;
  constexpr int W = Vec16<T>::n;
  P *q = reinterpret_cast<P *>(p);
#pragma unroll
  for (int c = 0; c < S / W; ++c) {
    P x;
    T *xs = reinterpret_cast<T *>(&x);
#pragma unroll
    for (int w = 0; w < W; ++w) xs[w] = v[c * W + w];
    __stcs(q + c, x);
  }
}

template <typename T, int S>
__device__ __forceinline__ void load_vec_stream(T (&v)[S], const T *p) {
  using P = typename Vec16<T>::type;
  constexpr int W = Vec16<T>::n;
  const P *q = reinterpret_cast<const P *>(p);
#pragma unroll
  for (int c = 0; c < S / W; ++c) {
    P x = __ldcs(q + c);
    const T *xs = reinterpret_cast<const T *>(&x);
#pragma unroll
    for (int w = 0; w < W; ++w) v[c * W + w] = xs[w];
  }
}

// ------------------------------------------------------- power-of-two scale
// Exponent e with m * 2^-e in [1, 2) for finite m > 0; 0 for m == 0 or
// non-finite m.  Scaling by 2^-e is exact for every value that stays normal.
__device__ __forceinline__ int scale_exponent(float m) {
  const uint32_t bits = __float_as_uint(m);
  const int be = (bits >> 23) & 0xff;
  if (be == 0xff || m <= 0.0f) return 0;
  if (be == 0) {  // subnormal: count leading zeros of the fraction
    const uint32_t frac = bits & 0x7fffff;  // value = frac * 2^-149
    return -118 - __clz(frac);
  }
  return be - 127;
}

__device__ __forceinline__ int scale_exponent(double m) {
  const unsigned long long bits = __double_as_longlong(m);
  const int be = static_cast<int>((bits >> 52) & 0x7ff);
  if (be == 0x7ff || m <= 0.0) return 0;
  if (be == 0) {
    const unsigned long long frac = bits & 0xfffffffffffffull;  // value = frac * 2^-1074
    return -1011 - __clzll(frac);
  }
  return be - 1023;
}

// 2^-e as T, for e in the range a single factor can represent.
__device__ __forceinline__ float pow2_neg(int e, float) {
  return __uint_as_float(static_cast<uint32_t>(127 - e) << 23);
}
__device__ __forceinline__ double pow2_neg(int e, double) {
  return __longlong_as_double(static_cast<long long>(1023 - e) << 52);
}

// Multiply by 2^-e exactly (two factors when 2^-e itself is not normal).
template <typename T>
__device__ __forceinline__ T times_pow2_neg(T x, int e) {
  constexpr int lim = sizeof(T) == 4 ? 126 : 1022;
  if (e >= -lim && e <= lim) return x * pow2_neg(e, T());
  const int h = e / 2;
  return (x * pow2_neg(h, T())) * pow2_neg(e - h, T());
}

// ------------------------------------------------------------ reductions
__device__ __forceinline__ float2 shfl_xor_f2(float2 v, int o) {
  return make_float2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o));
}

template <typename T>
__device__ __forceinline__ T warp_sum(T x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

}  // namespace tt
