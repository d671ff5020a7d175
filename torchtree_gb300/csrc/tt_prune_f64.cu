// FP64 instantiations of the pruning kernels (S = 4), the P-matrix
// backward and the likelihood reduction.
#include "tt_launch.h"
#include "tt_pmatrix.cuh"
#include "tt_prune.cuh"

namespace tt {

namespace {

template <int KMAX, int TILE, bool BACKWARD>
cudaError_t launch_one(const PruneArgs<double> &a, int batch, cudaStream_t stream) {
  const size_t smem = prune_smem_bytes<double>(4, a.K, a.C, a.slots, TILE, BACKWARD);
  const dim3 grid(a.ntiles, batch);
  if (BACKWARD) {
    auto kern = prune_backward_kernel<double, 4, KMAX, TILE, kStages>;
    cudaError_t e = kernel_smem(kern, smem);
    if (e != cudaSuccess) return e;
    kern<<<grid, TILE, smem, stream>>>(a);
  } else {
    auto kern = prune_forward_kernel<double, 4, KMAX, TILE, kStages>;
    cudaError_t e = kernel_smem(kern, smem);
    if (e != cudaSuccess) return e;
    kern<<<grid, TILE, smem, stream>>>(a);
  }
  return cudaGetLastError();
}

template <int TILE, bool BACKWARD>
cudaError_t by_k(const PruneArgs<double> &a, int batch, cudaStream_t stream) {
  switch (kmax_for(a.K)) {
    case 1: return launch_one<1, TILE, BACKWARD>(a, batch, stream);
    case 4: return launch_one<4, TILE, BACKWARD>(a, batch, stream);
    default: return launch_one<8, TILE, BACKWARD>(a, batch, stream);
  }
}

}  // namespace

__global__ void reduce_lnl_kernel(const double *tile_lnl, double *lnl, int ntiles, int accumulate) {
  __shared__ double part[8];
  const int b = blockIdx.x;
  double acc = 0.0;
  for (int t = threadIdx.x; t < ntiles; t += blockDim.x) acc += tile_lnl[size_t(b) * ntiles + t];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) s += part[w];
    lnl[b] = accumulate ? lnl[b] + s : s;
  }
}

cudaError_t launch_prune_f64(const PruneArgs<double> &a, bool backward, int tile, int batch,
                             cudaStream_t stream) {
  if (backward) {
    if (tile == kBwdTilesF64[0]) return by_k<kBwdTilesF64[0], true>(a, batch, stream);
    if (tile == kBwdTilesF64[1]) return by_k<kBwdTilesF64[1], true>(a, batch, stream);
  } else {
    if (tile == kFwdTilesF64[0]) return by_k<kFwdTilesF64[0], false>(a, batch, stream);
    if (tile == kFwdTilesF64[1]) return by_k<kFwdTilesF64[1], false>(a, batch, stream);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_reduce_f64(const double *gpart, const double *rootpart, double *G,
                              double *dfreq, double *dprop, int batch, int B, int ntiles, int S,
                              int K, int accumulate, cudaStream_t stream) {
  const int kss = K * S * S;
  reduce_branch_grads_kernel<double><<<dim3(B, batch), kss <= 64 ? 64 : 128, 0, stream>>>(
      gpart, G, B, ntiles, kss, accumulate);
  reduce_root_grads_kernel<double><<<batch, 32, 0, stream>>>(rootpart, dfreq, dprop, ntiles, S, K, accumulate);
  return cudaGetLastError();
}

// Self-test of the failure path of every staged kernel: one thread waits on
// an mbarrier that nothing arrives at, with the same bounded wait, gives up
// after limit_ns and records the timeout in the status word.
__global__ void wait_selftest_kernel(int *status, unsigned long long limit_ns) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_barrier_init();
    if (!mbar_wait_bounded(&bar, 0, limit_ns)) atomicExch(status, kDeviceTimeout);
  }
}

cudaError_t launch_wait_selftest(int *status, unsigned long long limit_ns, cudaStream_t stream) {
  wait_selftest_kernel<<<1, 32, 0, stream>>>(status, limit_ns);
  return cudaGetLastError();
}

cudaError_t launch_reduce_lnl(const double *tile_lnl, double *lnl, int batch, int ntiles, int accumulate,
                              cudaStream_t stream) {
  reduce_lnl_kernel<<<batch, 256, 0, stream>>>(tile_lnl, lnl, ntiles, accumulate);
  return cudaGetLastError();
}

cudaError_t launch_pmatrix_f64(const double *lam, const double *U, const double *W,
                               const double *bl, const double *rates, const int *branch_pos,
                               double *pmat, int S, int B, int K, int n_steps, int batch,
                               cudaStream_t stream) {
  const long long total = (long long)batch * B * K;
  const int threads = 128;
  const unsigned blocks = unsigned((total + threads - 1) / threads);
  pmatrix_from_eigen_kernel<double, 4><<<blocks, threads, 0, stream>>>(
      lam, U, W, bl, rates, branch_pos, pmat, B, K, n_steps, batch, 16);
  return cudaGetLastError();
}

cudaError_t launch_scatter_f64(const double *src, const int *branch_pos, double *pmat, int B,
                               int KSS, int n_steps, int batch, cudaStream_t stream) {
  const long long total = (long long)batch * B * KSS;
  const unsigned blocks = unsigned((total + 255) / 256);
  pmatrix_scatter_kernel<double><<<blocks, 256, 0, stream>>>(src, branch_pos, pmat, B, KSS, n_steps,
                                                             batch, 16, 16);
  return cudaGetLastError();
}

cudaError_t launch_pmatrix_backward(const double *G, const double *lam, const double *U,
                                    const double *W, const double *bl, const double *rates, int S,
                                    int B, int K, int batch, double *dlam, double *dU, double *dW,
                                    double *dbl, double *drates, cudaStream_t stream) {
  if (K <= 4)
    pmatrix_backward_kernel<4, 4, 128><<<batch, 128, 0, stream>>>(G, lam, U, W, bl, rates, B, K,
                                                                   dlam, dU, dW, dbl, drates);
  else
    pmatrix_backward_kernel<4, 8, 128><<<batch, 128, 0, stream>>>(G, lam, U, W, bl, rates, B, K,
                                                                   dlam, dU, dW, dbl, drates);
  return cudaGetLastError();
}

}  // namespace tt
