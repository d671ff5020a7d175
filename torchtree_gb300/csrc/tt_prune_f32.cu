// FP32 (rescaled) instantiations of the pruning kernels, S = 4.
#include "tt_launch.h"
#include "tt_pmatrix.cuh"
#include "tt_prune.cuh"

namespace tt {

namespace {

template <int KMAX, int TILE>
cudaError_t launch_one(const PruneArgs<float> &a, bool backward, int batch, cudaStream_t stream) {
  const size_t smem = prune_smem_bytes<float>(4, a.K, a.C, a.slots, TILE, backward);
  const dim3 grid(a.ntiles, batch);
  if (backward) {
    auto kern = prune_backward_kernel<float, 4, KMAX, TILE, kStages>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    kern<<<grid, TILE, smem, stream>>>(a);
  } else {
    auto kern = prune_forward_kernel<float, 4, KMAX, TILE, kStages>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    kern<<<grid, TILE, smem, stream>>>(a);
  }
  return cudaGetLastError();
}

template <int TILE>
cudaError_t by_k(const PruneArgs<float> &a, bool backward, int batch, cudaStream_t stream) {
  switch (kmax_for(a.K)) {
    case 1: return launch_one<1, TILE>(a, backward, batch, stream);
    case 4: return launch_one<4, TILE>(a, backward, batch, stream);
    default: return launch_one<8, TILE>(a, backward, batch, stream);
  }
}

}  // namespace

cudaError_t launch_prune_f32(const PruneArgs<float> &a, bool backward, int tile, int batch,
                             cudaStream_t stream) {
  if (tile == kTilesF32[0]) return by_k<kTilesF32[0]>(a, backward, batch, stream);
  return by_k<kTilesF32[1]>(a, backward, batch, stream);
}

cudaError_t launch_reduce_f32(const float *gpart, const float *rootpart, double *G, double *dfreq,
                              double *dprop, int batch, int B, int ntiles, int S, int K,
                              cudaStream_t stream) {
  const int kss = K * S * S;
  reduce_branch_grads_kernel<float><<<dim3(B, batch), kss <= 64 ? 64 : 128, 0, stream>>>(
      gpart, G, B, ntiles, kss);
  reduce_root_grads_kernel<float><<<batch, 32, 0, stream>>>(rootpart, dfreq, dprop, ntiles, S, K);
  return cudaGetLastError();
}

cudaError_t launch_pmatrix_f32(const double *lam, const double *U, const double *W,
                               const double *bl, const double *rates, const int *branch_pos,
                               float *pmat, int S, int B, int K, int n_steps, int batch,
                               cudaStream_t stream) {
  const long long total = (long long)batch * B * K;
  const int threads = 128;
  const unsigned blocks = unsigned((total + threads - 1) / threads);
  pmatrix_from_eigen_kernel<float, 4><<<blocks, threads, 0, stream>>>(lam, U, W, bl, rates, branch_pos,
                                                                      pmat, B, K, n_steps, batch);
  return cudaGetLastError();
}

cudaError_t launch_scatter_f32(const double *src, const int *branch_pos, float *pmat, int B,
                               int KSS, int n_steps, int batch, cudaStream_t stream) {
  const long long total = (long long)batch * B * KSS;
  const unsigned blocks = unsigned((total + 255) / 256);
  pmatrix_scatter_kernel<float><<<blocks, 256, 0, stream>>>(src, branch_pos, pmat, B, KSS, n_steps,
                                                            batch);
  return cudaGetLastError();
}

}  // namespace tt
