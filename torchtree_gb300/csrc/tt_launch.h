// Host-side launchers implemented in the per-precision translation units.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "tt_prune.cuh"
#include "tt_prune_tl.cuh"

namespace tt {

// Set the calling thread's tt_last_error() message; returns `code`.
int record_error(int code, const char *msg);

// Raise a kernel's dynamic shared-memory limit to `bytes` on the current
// device; with max_carveout also prefer the largest shared-memory carveout.
// The attribute is set once per (kernel, device) and size: later launches of
// the same kernel make no attribute call, so a launch inside stream capture
// or while the kernel runs on another stream touches no function state.
cudaError_t kernel_smem(const void *func, size_t bytes, bool max_carveout = false);
template <typename F>
cudaError_t kernel_smem(F *func, size_t bytes, bool max_carveout = false) {
  return kernel_smem(reinterpret_cast<const void *>(func), bytes, max_carveout);
}

// Pattern tile widths compiled per precision and pass (preferred first).
// FP32 plans: both passes use one tile width (the stored partials are laid
// out per tile): forward kTlFwdThreads threads x (kTlTile / kTlFwdThreads)
// patterns each, adjoint one pattern per thread.
constexpr int kTlTile = 64;
constexpr int kTlFwdThreads = 64;
constexpr int kTlBwdThreads = 64;
constexpr int kFwdTilesF32[2] = {kTlTile, kTlTile};
constexpr int kBwdTilesF32[2] = {kTlTile, kTlTile};
constexpr int kFwdTilesF64[2] = {64, 32};
constexpr int kBwdTilesF64[2] = {64, 32};
constexpr int kStages = 4;
// default staging-ring depths of the FP32 kernels (reduced to fit shared memory)
constexpr int kTlFwdStages = 3;
constexpr int kTlBwdStages = 2;

// category pairs of the FP32 kernels (K padded to an even count)
inline int kpairs_for(int K) { return (K + 1) / 2; }
// Tip-code rows are padded to a multiple of this many patterns.
constexpr int kCodeAlign = 128;

inline int kmax_for(int K) { return K <= 1 ? 1 : (K <= 4 ? 4 : 8); }

template <typename T>
size_t prune_smem_bytes(int S, int K, int C, int slots, int tile, bool backward) {
  return stack_layout<T>(S, K, C, slots, tile, kStages, kmax_for(K), backward).total;
}

// patterns per CTA of the producer-warp post-order (kTlPartTile-wide stored tiles)
constexpr int kTlWsPatterns = 128;
static_assert(kTlTile == kTlPartTile, "stored tile width");

// FP32 kernels (packed FP32x2, category pairs)
inline size_t tl_ws_smem_bytes(int K, int C, int slots, int nstage) {
  return size_t(tl_layout(kpairs_for(K), C, slots, kTlWsPatterns, kTlWsPatterns, nstage, false).total);
}
inline size_t tl_smem_bytes(int K, int C, int slots, bool backward, int nstage) {
  return size_t(tl_layout(kpairs_for(K), C, slots, kTlTile, backward ? kTlBwdThreads : kTlFwdThreads, nstage,
                          backward)
                    .total);
}

// Launch the pruning kernels (S = 4) with a tile width from the pass's
// candidate list.  Return cudaSuccess or the launch error.
// flags: kF32PairThreads = one thread per (pattern, category pair) kernels
// (K in 1-4 or 7-8); kF32ProducerWarp = post-order with a producer warp;
// kF32InPlaceAdjoint = adjoint that stores outside partials over the
// post-order tiles (consumes them) instead of a shared-memory stack;
// kF32PairAdjoint = that adjoint with one thread per (pattern, category pair)
// (K in 1-2, 3-4 or 7-8)
constexpr int kF32PairThreads = 1, kF32ProducerWarp = 2, kF32InPlaceAdjoint = 4, kF32PairAdjoint = 8;
cudaError_t launch_prune_f32(const PruneArgs<float> &a, bool backward, int tile, int batch, int flags,
                             cudaStream_t stream);
size_t tq_smem_bytes(int K, int C, int slots, bool backward, int nstage);
size_t ta_smem_bytes(int K, int C, int nstage);
size_t tp_smem_bytes(int K, int C, int nstage);
bool pair_threads_supported(int K);
bool pair_adjoint_supported(int K);
// One launch over the plans of `m` (all with the same category-pair count):
// the producer-warp post-order (`total` CTAs, kTlWsPatterns patterns each),
// or the in-place adjoint (one stored tile per CTA; `pair_adjoint` selects
// the pair-thread kernel).  `smem` = the largest dynamic shared memory any
// of the plans needs.
cudaError_t launch_forward_multi(const MultiPrune<float> &m, int total, size_t smem, cudaStream_t stream);
cudaError_t launch_adjoint_multi(const MultiPrune<float> &m, int total, size_t smem, bool pair_adjoint,
                                 cudaStream_t stream);
cudaError_t launch_prune_f64(const PruneArgs<double> &a, bool backward, int tile, int batch,
                             cudaStream_t stream);

// Sum the per-tile gradient blocks into G / dfreq / dprop; accumulate = 1
// adds to what is there (pattern slabs after the first).
cudaError_t launch_reduce_f32(const float *gpart, const float *rootpart, double *G, double *dfreq,
                              double *dprop, int batch, int B, int ntiles, int S, int K, int accumulate,
                              cudaStream_t stream);
cudaError_t launch_reduce_f64(const double *gpart, const double *rootpart, double *G,
                              double *dfreq, double *dprop, int batch, int B, int ntiles, int S,
                              int K, int accumulate, cudaStream_t stream);
// one bounded wait that nothing completes (limit_ns), reported in *status
cudaError_t launch_wait_selftest(int *status, unsigned long long limit_ns, cudaStream_t stream);
// lnL[b] = sum over tiles (fixed order); accumulate = 1 adds to lnl[b]
cudaError_t launch_reduce_lnl(const double *tile_lnl, double *lnl, int batch, int ntiles, int accumulate,
                              cudaStream_t stream);

cudaError_t launch_pmatrix_f32(const double *lam, const double *U, const double *W,
                               const double *bl, const double *rates, const int *branch_pos,
                               float *pmat, int S, int B, int K, int n_steps, int batch,
                               cudaStream_t stream);
cudaError_t launch_pmatrix_f64(const double *lam, const double *U, const double *W,
                               const double *bl, const double *rates, const int *branch_pos,
                               double *pmat, int S, int B, int K, int n_steps, int batch,
                               cudaStream_t stream);
cudaError_t launch_scatter_f32(const double *src, const int *branch_pos, float *pmat, int B,
                               int KSS, int n_steps, int batch, cudaStream_t stream);
cudaError_t launch_scatter_f64(const double *src, const int *branch_pos, double *pmat, int B,
                               int KSS, int n_steps, int batch, cudaStream_t stream);
cudaError_t launch_pmatrix_backward(const double *G, const double *lam, const double *U,
                                    const double *W, const double *bl, const double *rates, int S,
                                    int B, int K, int batch, double *dlam, double *dU, double *dW,
                                    double *dbl, double *drates, cudaStream_t stream);

}  // namespace tt
