// FP32 (rescaled) pruning kernels on packed FP32x2 arithmetic, S = 4.
#include <cstdlib>

#include "tt_launch.h"
#include "tt_pmatrix.cuh"
#include "tt_prune_ta.cuh"
#include "tt_prune_tl.cuh"
#include "tt_prune_tp.cuh"
#include "tt_prune_tq.cuh"

namespace tt {

namespace {

// dynamic shared memory of a kernel, with the largest carveout so that the
// CTAs the shared memory allows per SM are all resident
template <typename F>
cudaError_t set_smem(F kern, size_t smem) {
  return kernel_smem(kern, smem, true);
}

template <int KQ>
cudaError_t launch_tl(const PruneArgs<float> &a, bool backward, int batch, cudaStream_t stream) {
  const size_t smem = tl_smem_bytes(a.K, a.C, a.slots, backward, a.nstage);
  const dim3 grid(a.ntiles, batch);
  if (backward) {
    auto kern = tl_backward_kernel<KQ, kTlBwdThreads>;
    cudaError_t e = set_smem(kern, smem);
    if (e != cudaSuccess) return e;
    kern<<<grid, kTlBwdThreads, smem, stream>>>(a);
  } else {
    auto kern = tl_forward_kernel<KQ, kTlFwdThreads, kTlTile / kTlFwdThreads>;
    cudaError_t e = set_smem(kern, smem);
    if (e != cudaSuccess) return e;
    kern<<<grid, kTlFwdThreads, smem, stream>>>(a);
  }
  return cudaGetLastError();
}

template <int KQ>
cudaError_t launch_tq(const PruneArgs<float> &a, bool backward, int batch, cudaStream_t stream) {
  const size_t smem = tq_smem_bytes(a.K, a.C, a.slots, backward, a.nstage);
  const dim3 grid(a.ntiles, batch);
  if (backward) {
    auto kern = tq_backward_kernel<KQ>;
    cudaError_t e = set_smem(kern, smem);
    if (e != cudaSuccess) return e;
    kern<<<grid, kTqTile * KQ, smem, stream>>>(a);
  } else {
    auto kern = tq_forward_kernel<KQ>;
    cudaError_t e = set_smem(kern, smem);
    if (e != cudaSuccess) return e;
    kern<<<grid, kTqTile * KQ, smem, stream>>>(a);
  }
  return cudaGetLastError();
}

}  // namespace

size_t tq_smem_bytes(int K, int C, int slots, bool backward, int nstage) {
  const int KQ = kpairs_for(K);
  return size_t(tl_layout(KQ, C, slots, kTqTile, kTqTile * KQ, nstage, backward, kTqRed2).total);
}

bool pair_threads_supported(int K) {
  const int KQ = kpairs_for(K);
  return KQ == 1 || KQ == 2 || KQ == 4;
}

template <int KQ>
cudaError_t launch_tl_ws(const PruneArgs<float> &a, int batch, cudaStream_t stream) {
  const size_t smem = tl_ws_smem_bytes(a.K, a.C, a.slots, a.nstage);
  constexpr int TPC = kTlWsPatterns / kTlTile;
  const dim3 grid((a.ntiles + TPC - 1) / TPC, batch);
  auto kern = tl_forward_ws_kernel<KQ, kTlWsPatterns>;
  cudaError_t e = set_smem(kern, smem);
  if (e != cudaSuccess) return e;
  kern<<<grid, kTlWsPatterns + 32, smem, stream>>>(a);
  return cudaGetLastError();
}

size_t ta_smem_bytes(int K, int C, int nstage) {
  return size_t(ta_layout(kpairs_for(K), C, kTlTile, kTlBwdThreads, nstage).total);
}

template <int KQ>
cudaError_t launch_ta(const PruneArgs<float> &a, int batch, cudaStream_t stream) {
  const size_t smem = ta_smem_bytes(a.K, a.C, a.nstage);
  const dim3 grid(a.ntiles, batch);
  auto kern = ta_backward_kernel<KQ, kTlBwdThreads>;
  cudaError_t e = set_smem(kern, smem);
  if (e != cudaSuccess) return e;
  kern<<<grid, kTlBwdThreads, smem, stream>>>(a);
  return cudaGetLastError();
}

size_t tp_smem_bytes(int K, int C, int nstage) {
  const int KQ = kpairs_for(K);
  return size_t(ta_layout(KQ, C, kTpTile, kTpTile * KQ, nstage).total);
}

bool pair_adjoint_supported(int K) {
  const int KQ = kpairs_for(K);
  return KQ == 1 || KQ == 2 || KQ == 4;
}

template <int KQ, int MB = tp_min_blocks(KQ)>
cudaError_t launch_tp(const PruneArgs<float> &a, int batch, cudaStream_t stream) {
  const size_t smem = tp_smem_bytes(a.K, a.C, a.nstage);
  const dim3 grid(a.ntiles, batch);
  auto kern = tp_backward_kernel<KQ, MB>;
  cudaError_t e = set_smem(kern, smem);
  if (e != cudaSuccess) return e;
  kern<<<grid, kTpTile * KQ, smem, stream>>>(a);
  return cudaGetLastError();
}

namespace {

template <int KQ>
cudaError_t launch_forward_multi_k(const MultiPrune<float> &m, int total, size_t smem, cudaStream_t stream) {
  auto kern = tl_forward_ws_multi_kernel<KQ, kTlWsPatterns>;
  cudaError_t e = set_smem(kern, smem);
  if (e != cudaSuccess) return e;
  kern<<<total, kTlWsPatterns + 32, smem, stream>>>(m);
  return cudaGetLastError();
}

template <int KQ>
cudaError_t launch_adjoint_multi_k(const MultiPrune<float> &m, int total, size_t smem, bool pair_adjoint,
                                   cudaStream_t stream) {
  if constexpr (KQ == 1 || KQ == 2 || KQ == 4) {
    if (pair_adjoint) {
      auto kern = tp_backward_multi_kernel<KQ>;
      cudaError_t e = set_smem(kern, smem);
      if (e != cudaSuccess) return e;
      kern<<<total, kTpTile * KQ, smem, stream>>>(m);
      return cudaGetLastError();
    }
  }
  auto kern = ta_backward_multi_kernel<KQ, kTlBwdThreads>;
  cudaError_t e = set_smem(kern, smem);
  if (e != cudaSuccess) return e;
  kern<<<total, kTlBwdThreads, smem, stream>>>(m);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_forward_multi(const MultiPrune<float> &m, int total, size_t smem, cudaStream_t stream) {
  switch (kpairs_for(m.a[0].K)) {
    case 1: return launch_forward_multi_k<1>(m, total, smem, stream);
    case 2: return launch_forward_multi_k<2>(m, total, smem, stream);
    case 3: return launch_forward_multi_k<3>(m, total, smem, stream);
    default: return launch_forward_multi_k<4>(m, total, smem, stream);
  }
}

cudaError_t launch_adjoint_multi(const MultiPrune<float> &m, int total, size_t smem, bool pair_adjoint,
                                 cudaStream_t stream) {
  switch (kpairs_for(m.a[0].K)) {
    case 1: return launch_adjoint_multi_k<1>(m, total, smem, pair_adjoint, stream);
    case 2: return launch_adjoint_multi_k<2>(m, total, smem, pair_adjoint, stream);
    case 3: return launch_adjoint_multi_k<3>(m, total, smem, false, stream);
    default: return launch_adjoint_multi_k<4>(m, total, smem, pair_adjoint, stream);
  }
}

cudaError_t launch_prune_f32(const PruneArgs<float> &a, bool backward, int tile, int batch, int flags,
                             cudaStream_t stream) {
  if (tile != kTlTile) return cudaErrorInvalidValue;
  const bool pair_threads = flags & kF32PairThreads;
  if (backward && !pair_threads && (flags & kF32InPlaceAdjoint) && (flags & kF32PairAdjoint) &&
      pair_adjoint_supported(a.K)) {
    switch (kpairs_for(a.K)) {
      case 1: return launch_tp<1>(a, batch, stream);
      case 2:  // register budget for 7 CTAs per SM (72 registers), or 8 (64, a few spills) on request
        return getenv("TT_TP_MINBLOCKS") && atoi(getenv("TT_TP_MINBLOCKS")) == 8 ? launch_tp<2, 8>(a, batch, stream)
                                                                                 : launch_tp<2>(a, batch, stream);
      default: return launch_tp<4>(a, batch, stream);
    }
  }
  if (backward && !pair_threads && (flags & kF32InPlaceAdjoint)) {
    switch (kpairs_for(a.K)) {
      case 1: return launch_ta<1>(a, batch, stream);
      case 2: return launch_ta<2>(a, batch, stream);
      case 3: return launch_ta<3>(a, batch, stream);
      default: return launch_ta<4>(a, batch, stream);
    }
  }
  if (!backward && !pair_threads && (flags & kF32ProducerWarp) && a.nstage <= 8) {
    switch (kpairs_for(a.K)) {
      case 1: return launch_tl_ws<1>(a, batch, stream);
      case 2: return launch_tl_ws<2>(a, batch, stream);
      case 3: return launch_tl_ws<3>(a, batch, stream);
      default: return launch_tl_ws<4>(a, batch, stream);
    }
  }
  if (pair_threads) {
    switch (kpairs_for(a.K)) {
      case 1: return launch_tq<1>(a, backward, batch, stream);
      case 2: return launch_tq<2>(a, backward, batch, stream);
      case 4: return launch_tq<4>(a, backward, batch, stream);
      default: return cudaErrorInvalidValue;
    }
  }
  switch (kpairs_for(a.K)) {
    case 1: return launch_tl<1>(a, backward, batch, stream);
    case 2: return launch_tl<2>(a, backward, batch, stream);
    case 3: return launch_tl<3>(a, backward, batch, stream);
    default: return launch_tl<4>(a, backward, batch, stream);
  }
}

cudaError_t launch_reduce_f32(const float *gpart, const float *rootpart, double *G, double *dfreq,
                              double *dprop, int batch, int B, int ntiles, int S, int K, int accumulate,
                              cudaStream_t stream) {
  const int kss = K * S * S;
  reduce_branch_grads_kernel<float><<<dim3(B, batch), kss <= 64 ? 64 : 128, 0, stream>>>(
      gpart, G, B, ntiles, kss, accumulate);
  reduce_root_grads_kernel<float><<<batch, 32, 0, stream>>>(rootpart, dfreq, dprop, ntiles, S, K, accumulate);
  return cudaGetLastError();
}

cudaError_t launch_pmatrix_f32(const double *lam, const double *U, const double *W,
                               const double *bl, const double *rates, const int *branch_pos,
                               float *pmat, int S, int B, int K, int n_steps, int batch,
                               cudaStream_t stream) {
  const long long total = (long long)batch * B * K;
  const int threads = 128;
  const unsigned blocks = unsigned((total + threads - 1) / threads);
  pmatrix_pairs_from_eigen_kernel<<<blocks, threads, 0, stream>>>(lam, U, W, bl, rates, branch_pos, pmat, B, K,
                                                                  kpairs_for(K), n_steps, batch);
  return cudaGetLastError();
}

cudaError_t launch_scatter_f32(const double *src, const int *branch_pos, float *pmat, int B,
                               int KSS, int n_steps, int batch, cudaStream_t stream) {
  const long long total = (long long)batch * B * KSS;
  const unsigned blocks = unsigned((total + 255) / 256);
  const int K = KSS / 16;
  pmatrix_pairs_scatter_kernel<<<blocks, 256, 0, stream>>>(src, branch_pos, pmat, B, K, kpairs_for(K), n_steps,
                                                           batch);
  return cudaGetLastError();
}

}  // namespace tt
