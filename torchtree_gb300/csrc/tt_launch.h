// Host-side launchers implemented in the per-precision translation units.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "tt_prune.cuh"

namespace tt {

// Set the calling thread's tt_last_error() message; returns `code`.
int record_error(int code, const char *msg);

// Pattern tile widths compiled per precision (largest first).
constexpr int kTilesF32[2] = {128, 64};
constexpr int kTilesF64[2] = {64, 32};
constexpr int kStages = 4;

inline int kmax_for(int K) { return K <= 1 ? 1 : (K <= 4 ? 4 : 8); }

template <typename T>
size_t prune_smem_bytes(int S, int K, int C, int slots, int tile, bool backward) {
  return stack_layout<T>(S, K, C, slots, tile, kStages, kmax_for(K), backward).total;
}

// Launch the pruning kernels (S = 4).  Return cudaSuccess or the launch error.
cudaError_t launch_prune_f32(const PruneArgs<float> &a, bool backward, int tile, int batch,
                             cudaStream_t stream);
cudaError_t launch_prune_f64(const PruneArgs<double> &a, bool backward, int tile, int batch,
                             cudaStream_t stream);

cudaError_t launch_reduce_f32(const float *gpart, const float *rootpart, double *G, double *dfreq,
                              double *dprop, int batch, int B, int ntiles, int S, int K,
                              cudaStream_t stream);
cudaError_t launch_reduce_f64(const double *gpart, const double *rootpart, double *G,
                              double *dfreq, double *dprop, int batch, int B, int ntiles, int S,
                              int K, cudaStream_t stream);
cudaError_t launch_reduce_lnl(const double *tile_lnl, double *lnl, int batch, int ntiles,
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
