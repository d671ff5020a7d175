// Host side of the wide-state path (S != 4: amino acids, codons): level
// schedule, workspace and launch sequences behind the C entry points.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <string>
#include <vector>

#include <cudaTypedefs.h>

#include "../../include/torchtree_gb300.h"
#include "tt_plan.h"
#include "tt_wide.cuh"
#include "tt_wide_tc.cuh"
#include "tt_wide_tc_bwd.cuh"

namespace tt {

__global__ void wide_root_kernel(const double *root_site, const int *root_expo, const double *props,
                                 const double *weights, double *site_lnl, double *log2L, double *block_lnl,
                                 int K, int N, int Npad) {
  __shared__ double part[8];
  const int b = blockIdx.y, n = blockIdx.x * 256 + threadIdx.x;
  double contrib = 0.0;
  if (n < N) {
    int emax = INT_MIN;
    for (int k = 0; k < K; ++k) emax = max(emax, root_expo[(size_t(b) * K + k) * Npad + n]);
    double s = 0.0;
    for (int k = 0; k < K; ++k) {
      const size_t o = (size_t(b) * K + k) * Npad + n;
      s += props[size_t(b) * K + k] * ldexp(root_site[o], root_expo[o] - emax);
    }
    const double l2 = log2(s) + double(emax);
    const double ll = l2 * 0.69314718055994530942;
    if (site_lnl) site_lnl[size_t(b) * N + n] = ll;
    log2L[size_t(b) * Npad + n] = l2;
    contrib = weights[n] * ll;
  }
  contrib = warp_sum(contrib);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = contrib;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += part[w];
    block_lnl[size_t(b) * gridDim.x + blockIdx.x] = t;
  }
}

__global__ void wide_pmatrix_grad_reduce_kernel(const double *part, int nchunks, int S, int K, double *dlam,
                                                double *dU, double *dW, double *drates) {
  const int b = blockIdx.x;
  const int width = 2 * S * S + S + K;
  for (int e = threadIdx.x; e < width; e += blockDim.x) {
    double s = 0.0;
    for (int c = 0; c < nchunks; ++c) s += part[(size_t(b) * nchunks + c) * width + e];
    if (e < S * S) {
      if (dU) dU[size_t(b) * S * S + e] = s;
    } else if (e < 2 * S * S) {
      if (dW) dW[size_t(b) * S * S + e - S * S] = s;
    } else if (e < 2 * S * S + S) {
      if (dlam) dlam[size_t(b) * S + e - 2 * S * S] = s;
    } else if (drates) {
      drates[size_t(b) * K + e - 2 * S * S - S] = s;
    }
  }
}

struct WideState {
  int SP = 0, PTf = 0, PTb = 0;
  int Npad = 0;  // whole alignment padded to 128 patterns: the tip-code row stride
  int bchunk = 8, nbchunks = 1;
  bool tc = false;  // FP32 codon post-order on the tensor cores
  bool store_products = false;  // FP32 codon: the adjoint reads the post-order's children's products
  bool tc_bwd = false;  // FP32 codon adjoint on the tensor cores (needs the stored products)
  float *d_pimg = nullptr;  // its GEMM2 operands: split P^T images [b][B][K][2][64][64]
  float *d_pimg_f = nullptr;  // the tensor-core post-order's B operands: split P images, same shape
  // the images hold the current transition matrices (written right after them, in one pass)
  bool img_f_valid = false, img_b_valid = false;
  // pattern slabs (p->slab != 0): the pattern-sized buffers below hold one
  // slab; tail_valid = they still hold the last slab's post-order (from a
  // tt_log_likelihood with keep_partials), which the gradient then reuses
  bool tail_valid = false;
  size_t slab_bytes = 0;     // of p->bytes: the pattern-sized buffers
  double *d_site = nullptr;  // slab mode: one slab's site log-likelihoods [b][slab]
  std::vector<int> fwd_off, bwd_off;  // level boundaries in d_fwd / d_bwd
  int *d_left = nullptr, *d_right = nullptr, *d_fwd = nullptr, *d_bwd = nullptr;
  int *d_branch_lvn = nullptr;  // [B] node count of each branch's parent level (adjoint chunking)
  void *d_part = nullptr;
  int *d_expo = nullptr;
  double *d_root_site = nullptr;
  int *d_root_expo = nullptr;
  double *d_log2L = nullptr;
  double *d_block_lnl = nullptr;
  void *d_gpart = nullptr;
  void *d_rootpart = nullptr;
  double *d_pgpart = nullptr;
  void *d_prod = nullptr;  // FP32: the children's products of the post-order, read by the adjoint
};

namespace {

int wfail(int code, const std::string &m) { return record_error(code, m.c_str()); }

// Launch geometry of a pass over `n` patterns (the whole alignment or one
// slab): padded width, tiles of the two passes, root blocks, and the
// adjoint's chunks of tiles (about two CTAs per SM over batch x categories;
// cmax bounds the chunk count of any pass over at most n patterns).
struct WideGeo {
  int Npad, ntiles_f, ntiles_b, nblk, nchunks, tpc, cmax;
};

WideGeo wide_geo(const tt_plan *p, int n) {
  const WideState &w = *p->wide;
  WideGeo g;
  g.Npad = (n + 127) / 128 * 128;
  g.ntiles_f = g.Npad / w.PTf;
  g.ntiles_b = g.Npad / w.PTb;
  g.nblk = (n + 255) / 256;
  const int want = (2 * 152 + p->batch * p->K - 1) / (p->batch * p->K);
  g.cmax = std::max(1, std::min({want, g.ntiles_b, 64}));
  g.tpc = (g.ntiles_b + g.cmax - 1) / g.cmax;
  g.nchunks = (g.ntiles_b + g.tpc - 1) / g.tpc;
  return g;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda link)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *ptr = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
  }
  return fn;
}

// A row-major FP32 array [rows][cols] (cols a multiple of 4) as a 2-D tensor
// map with bx x by boxes, no swizzle.
bool encode_rows(CUtensorMap *m, const float *base, uint64_t rows, uint64_t cols, uint32_t bx, uint32_t by,
                 CUtensorMapSwizzle swizzle = CU_TENSOR_MAP_SWIZZLE_NONE) {
  const PFN_cuTensorMapEncodeTiled_v12000 fn = tensor_map_encoder();
  if (!fn) return false;
  const cuuint64_t dims[2] = {cols, rows};
  const cuuint64_t strides[1] = {cols * sizeof(float)};
  const cuuint32_t box[2] = {bx, by};
  const cuuint32_t elem[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(base), dims, strides, box, elem,
            CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Both split images of the FP32 codon transition matrices that the tensor-core
// kernels use, from d_pmat in one pass (either may be skipped).
cudaError_t launch_pimages(tt_plan *p, bool fwd, bool bwd, cudaStream_t s) {
  WideState &w = *p->wide;
  float *f = fwd ? w.d_pimg_f : nullptr, *b = bwd ? w.d_pimg : nullptr;
  if (!f && !b) return cudaSuccess;
  const long long count = (long long)p->batch * p->B * p->K;
  wide_pimages_kernel<<<unsigned(count), 256, 0, s>>>(static_cast<const float *>(p->d_pmat), f, b);
  p->launches += 1;
  if (f) w.img_f_valid = true;
  if (b) w.img_b_valid = true;
  return cudaGetLastError();
}

int wcuda(cudaError_t e, const char *where) {
  return wfail(e == cudaErrorMemoryAllocation ? TT_ERR_OUT_OF_MEMORY : TT_ERR_CUDA,
               std::string(where) + ": " + cudaGetErrorString(e));
}

template <typename P>
int walloc(tt_plan *p, P **ptr, size_t bytes, const char *what) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(ptr), bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return wfail(TT_ERR_OUT_OF_MEMORY, std::string("cudaMalloc of ") + what + " (" + std::to_string(bytes) +
                                           " bytes) failed: " + cudaGetErrorString(e));
  }
  p->bytes += bytes;
  return TT_OK;
}

// compiled (precision, padded states) -> pattern tiles of the two passes
void tiles_for(bool f32, int SP, int &ptf, int &ptb) {
  if (SP == 20) {
    ptf = ptb = 128;
  } else {
    ptf = ptb = f32 ? 64 : 32;
  }
}

template <typename T, int SP, int PTF, int PTB>
struct Wide {
  static cudaError_t prepare() {
    cudaError_t e = cudaFuncSetAttribute(wide_forward_kernel<T, SP, PTF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         int(wide_fwd_smem<T, SP, PTF>()));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(wide_backward_kernel<T, SP, PTB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               int(wide_bwd_smem<T, SP, PTB>()));
    if (e == cudaSuccess)  // the CTAs the shared memory allows per SM all resident
      e = cudaFuncSetAttribute(wide_backward_kernel<T, SP, PTB>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               int(cudaSharedmemCarveoutMaxShared));
    if (std::is_same<T, float>::value && SP == 64 && e == cudaSuccess)
      e = cudaFuncSetAttribute(wide_forward_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::kSmem);
    if (std::is_same<T, float>::value && SP == 64 && e == cudaSuccess)  // two CTAs per SM
      e = cudaFuncSetAttribute(wide_forward_tc_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                               int(cudaSharedmemCarveoutMaxShared));
    if (std::is_same<T, float>::value && SP == 64 && e == cudaSuccess)
      e = cudaFuncSetAttribute(wide_backward_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, tcb::kSmem);
    if (std::is_same<T, float>::value && SP == 64 && e == cudaSuccess)
      e = cudaFuncSetAttribute(wide_backward_tc_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                               int(cudaSharedmemCarveoutMaxShared));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(wide_pmatrix_kernel<T, SP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               int(3 * SP * SP * sizeof(T) + SP * sizeof(T)));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(wide_pmatrix_backward_kernel<double, SP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               int(Wide<double, SP, PTF, PTB>::pback_smem()));
    return e;
  }
  static size_t pback_smem() { return 4 * SP * SP * sizeof(T) + (SP / 4 * SP + 3 * SP + 8) * sizeof(double); }

  // arguments of a pass over patterns [p0, p0 + n) with geometry g: tip
  // codes and weights from the slab's first pattern, every pattern-sized
  // buffer with the slab's own width
  static WideArgs<T> args(tt_plan *p, const double *props, const double *freqs, int rescale, const WideGeo &g,
                          int p0, int n) {
    WideState &w = *p->wide;
    WideArgs<T> a;
    a.tips = p->T;
    a.N = n;
    a.Npad = g.Npad;
    a.K = p->K;
    a.B = p->B;
    a.I = p->I;
    a.S = p->S;
    a.code_stride = p->code_stride;
    a.rescale = rescale;
    a.nchunks = g.nchunks;
    a.tiles_per_chunk = g.tpc;
    a.ntiles = g.ntiles_b;
    a.nodes = nullptr;
    a.left = w.d_left;
    a.right = w.d_right;
    a.codes = p->d_codes + p0;
    a.table = static_cast<const T *>(p->d_table);
    a.pmat = static_cast<const T *>(p->d_pmat);
    a.part = static_cast<T *>(w.d_part);
    a.expo = w.d_expo;
    a.props = props;
    a.freqs = freqs;
    a.weights = p->d_weights + p0;
    a.root_site = w.d_root_site;
    a.root_expo = w.d_root_expo;
    a.log2L = w.d_log2L;
    a.gpart = static_cast<T *>(w.d_gpart);
    a.rootpart = static_cast<T *>(w.d_rootpart);
    a.prod = nullptr;
    return a;
  }

  // post-order over patterns [p0, p0 + n), root sums, and lnL (added to
  // lnl when accumulate; no lnL when lnl is NULL).  site_lnl [b][n].
  static cudaError_t forward(tt_plan *p, const double *props, const double *freqs, int rescale, bool keep,
                             double *lnl, double *site_lnl, int p0, int n, int accumulate, cudaStream_t s) {
    WideState &w = *p->wide;
    const WideGeo g = wide_geo(p, n);
    WideArgs<T> a = args(p, props, freqs, rescale, g, p0, n);
    if (keep) a.prod = static_cast<T *>(w.d_prod);
    constexpr int NT = WideCfg<T, SP, PTF>::NT;
    const size_t smem = wide_fwd_smem<T, SP, PTF>();
    if constexpr (std::is_same<T, float>::value && SP == 64) {
      if (w.tc && w.d_pimg_f && !w.img_f_valid) {  // the post-order's split P images, if not written with P
        const cudaError_t e = launch_pimages(p, true, false, s);
        if (e != cudaSuccess) return e;
      }
    }
    for (size_t lv = 0; lv + 1 < w.fwd_off.size(); ++lv) {
      a.nodes = w.d_fwd + w.fwd_off[lv];
      if constexpr (std::is_same<T, float>::value && SP == 64) {
        if (w.tc) {  // tiles per CTA by level: about sixteen waves of two CTAs per SM
          const int nodes = w.fwd_off[lv + 1] - w.fwd_off[lv], ntf = g.Npad / tc::kPT;
          const int chunks = tc_level_chunks(nodes, p->batch * p->K, ntf, ntf, 16 * 152 * 2);
          WideArgs<T> at = a;
          at.ntiles = ntf;
          at.tiles_per_chunk = (ntf + chunks - 1) / chunks;
          const dim3 grid(chunks, nodes, plan_run_samples(p) * p->K);
          wide_forward_tc_kernel<<<grid, tc::kThreads, tc::kSmem, s>>>(at, w.d_pimg_f, p->d_status, 2000000000ull);
          p->launches += 1;
          continue;
        }
      }
      const dim3 grid(g.ntiles_f, w.fwd_off[lv + 1] - w.fwd_off[lv], plan_run_samples(p) * p->K);
      wide_forward_kernel<T, SP, PTF><<<grid, NT, smem, s>>>(a);
      p->launches += 1;
    }
    wide_root_kernel<<<dim3(g.nblk, plan_run_samples(p)), 256, 0, s>>>(w.d_root_site, w.d_root_expo, props, a.weights,
                                                           site_lnl, w.d_log2L, w.d_block_lnl, p->K, n, g.Npad);
    p->launches += 1;
    cudaError_t e = cudaSuccess;
    if (lnl) {
      e = launch_reduce_lnl(w.d_block_lnl, lnl, plan_run_samples(p), g.nblk, accumulate, s);
      p->launches += 1;
    }
    return e == cudaSuccess ? cudaGetLastError() : e;
  }

  // adjoint over patterns [p0, p0 + n) after that range's post-order; the
  // chunk sums are added to the previous slabs' when accumulate
  static cudaError_t backward(tt_plan *p, const double *props, const double *freqs, int p0, int n, int accumulate,
                              cudaStream_t s) {
    WideState &w = *p->wide;
    const WideGeo g = wide_geo(p, n);
    WideArgs<T> a = args(p, props, freqs, 1, g, p0, n);
    a.prod = static_cast<T *>(w.d_prod);
    if constexpr (std::is_same<T, float>::value && SP == 64) {
      if (w.tc_bwd && a.prod && w.d_pimg) return backward_tc(p, a, g, accumulate, s);
    }
    constexpr int NT = WideCfg<T, SP, PTB>::NT;
    const size_t smem = wide_bwd_smem<T, SP, PTB>(a.prod != nullptr);
    // FP32 20-state plans: a chunk count per level (three CTAs per SM), as the tensor-core adjoint does
    constexpr bool per_level = std::is_same<T, float>::value && SP == 20;
    const int bk = p->batch * p->K, target = 8 * 152 * 3;
    for (size_t lv = 0; lv + 1 < w.bwd_off.size(); ++lv) {
      const int nodes = w.bwd_off[lv + 1] - w.bwd_off[lv];
      const int chunks = per_level ? tc_level_chunks(nodes, bk, g.ntiles_b, g.cmax, target) : g.nchunks;
      a.nodes = w.d_bwd + w.bwd_off[lv];
      a.tiles_per_chunk = per_level ? (g.ntiles_b + chunks - 1) / chunks : g.tpc;
      const dim3 grid(chunks, nodes, plan_run_samples(p) * p->K);
      wide_backward_kernel<T, SP, PTB><<<grid, NT, smem, s>>>(a);
      p->launches += 1;
    }
    wide_grad_reduce_kernel<T><<<dim3(p->B, plan_run_samples(p)), 256, 0, s>>>(
        static_cast<const T *>(w.d_gpart), p->d_G, p->B, g.nchunks, p->K, p->S, SP, accumulate,
        per_level ? w.d_branch_lvn : nullptr, bk, g.ntiles_b, g.cmax, target);
    wide_root_reduce_kernel<T><<<plan_run_samples(p), 64, 0, s>>>(static_cast<const T *>(w.d_rootpart), p->d_rootgrad,
                                                       p->d_rootgrad + size_t(p->batch) * p->S, g.nchunks, p->K,
                                                       p->S, SP, accumulate);
    p->launches += 2;
    return cudaGetLastError();
  }

  // the tensor-core adjoint (FP32 codon plans): split P^T images, then one
  // launch per depth level over chunks of 128-pattern tiles
  static cudaError_t backward_tc(tt_plan *p, WideArgs<float> a, const WideGeo &g, int accumulate, cudaStream_t s) {
    WideState &w = *p->wide;
    if (!w.img_b_valid) {  // the split P^T images, if not written with P
      const cudaError_t e = launch_pimages(p, false, true, s);
      if (e != cudaSuccess) return e;
    }
    const int ntc = g.Npad / tcb::kPT;
    const int want = (2 * 152 + p->batch * p->K - 1) / (p->batch * p->K);
    const int cmax = std::max(1, std::min({want, ntc, g.cmax}));
    const int tpc = (ntc + cmax - 1) / cmax;
    a.ntiles = ntc;
    a.tiles_per_chunk = tpc;
    a.nchunks = (ntc + tpc - 1) / tpc;
    // the raw rows as 2-D tensors: partials [b I K 64][Npad], products [b I K 128][Npad]
    TcbMaps maps;
    const uint64_t blocks = uint64_t(p->batch) * p->I * p->K;
    if (!encode_rows(&maps.part32, a.part, blocks * 64, uint64_t(g.Npad), 32, 64, CU_TENSOR_MAP_SWIZZLE_128B) ||
        !encode_rows(&maps.prod32, a.prod, blocks * 128, uint64_t(g.Npad), 32, 128, CU_TENSOR_MAP_SWIZZLE_128B) ||
        !encode_rows(&maps.part128, a.part, blocks * 64, uint64_t(g.Npad), 128, 32) ||
        !encode_rows(&maps.prod128, a.prod, blocks * 128, uint64_t(g.Npad), 128, 32))
      return cudaErrorInvalidValue;
    // a.nchunks stays the chunk stride of the gradient blocks; each level launches
    // tc_level_chunks(...) <= a.nchunks chunks (the root's level all of them)
    const int bk = p->batch * p->K;
    for (size_t lv = 0; lv + 1 < w.bwd_off.size(); ++lv) {
      const int nodes = w.bwd_off[lv + 1] - w.bwd_off[lv];
      const int chunks = tc_level_chunks(nodes, bk, ntc, cmax);
      a.nodes = w.d_bwd + w.bwd_off[lv];
      a.tiles_per_chunk = (ntc + chunks - 1) / chunks;
      const dim3 grid(chunks, nodes, plan_run_samples(p) * p->K);
      wide_backward_tc_kernel<<<grid, tcb::kThreads, tcb::kSmem, s>>>(a, maps, w.d_pimg, p->C, p->d_status,
                                                                       2000000000ull);
      p->launches += 1;
    }
    wide_grad_reduce_kernel<float><<<dim3(p->B, plan_run_samples(p)), 256, 0, s>>>(static_cast<const float *>(w.d_gpart),
                                                                         p->d_G, p->B, a.nchunks, p->K, p->S, 64,
                                                                         accumulate, w.d_branch_lvn, bk, ntc, cmax);
    wide_root_reduce_kernel<float><<<plan_run_samples(p), 64, 0, s>>>(static_cast<const float *>(w.d_rootpart), p->d_rootgrad,
                                                           p->d_rootgrad + size_t(p->batch) * p->S, a.nchunks, p->K,
                                                           p->S, 64, accumulate);
    p->launches += 2;
    return cudaGetLastError();
  }

  static cudaError_t pmatrix(tt_plan *p, const double *lam, const double *U, const double *W, const double *bl,
                             const double *rates, cudaStream_t s) {
    wide_pmatrix_kernel<T, SP><<<dim3(p->B, p->batch), 256, 3 * SP * SP * sizeof(T) + SP * sizeof(T), s>>>(
        lam, U, W, bl, rates, static_cast<T *>(p->d_pmat), p->S, p->B, p->K);
    p->launches += 1;
    p->wide->img_f_valid = p->wide->img_b_valid = false;
    if constexpr (std::is_same<T, float>::value && SP == 64) {  // the tensor-core kernels' images with P
      const cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
      return launch_pimages(p, p->wide->tc, p->wide->tc_bwd, s);
    }
    return cudaGetLastError();
  }

  static cudaError_t pmatrix_backward(tt_plan *p, const double *lam, const double *U, const double *W,
                                      const double *bl, const double *rates, double *dlam, double *dU, double *dW,
                                      double *dbl, double *drates, cudaStream_t s) {
    WideState &w = *p->wide;
    wide_pmatrix_backward_kernel<double, SP><<<dim3(w.nbchunks, p->batch), 256, Wide<double, SP, PTF, PTB>::pback_smem(), s>>>(
        p->d_G, lam, U, W, bl, rates, p->S, p->B, p->K, w.bchunk, dbl, w.d_pgpart);
    wide_pmatrix_grad_reduce_kernel<<<p->batch, 256, 0, s>>>(w.d_pgpart, w.nbchunks, p->S, p->K, dlam, dU, dW,
                                                             drates);
    p->launches += 2;
    return cudaGetLastError();
  }
};

// dispatch on (precision, SP)
template <typename F>
cudaError_t dispatch(tt_plan *p, F &&f) {
  const bool f32 = p->precision == TT_PRECISION_F32;
  if (p->wide->SP == 20) {
    if (f32) return f(Wide<float, 20, 128, 128>());
    return f(Wide<double, 20, 128, 128>());
  }
  if (f32) return f(Wide<float, 64, 64, 64>());
  return f(Wide<double, 64, 32, 32>());
}

}  // namespace

int wide_create(tt_plan *p) {
  if (p->S < 2 || p->S > 64) return wfail(TT_ERR_UNSUPPORTED, "state_count must be in [2, 64]");
  WideState *w = new WideState();
  p->wide = w;
  const bool f32 = p->precision == TT_PRECISION_F32;
  w->SP = p->S <= 20 ? 20 : 64;
  tiles_for(f32, w->SP, w->PTf, w->PTb);
  w->Npad = (p->N + 127) / 128 * 128;
  if (size_t(p->batch) * p->K > 65535) return wfail(TT_ERR_INVALID_ARGUMENT, "batch * category_count must be <= 65535");
  w->nbchunks = (p->B + w->bchunk - 1) / w->bchunk;
  {  // tensor-core post-order for FP32 codon plans (TT_WIDE_TC=0 selects the CUDA-core kernel)
    const char *env = getenv("TT_WIDE_TC");
    w->tc = f32 && w->SP == 64 && !(env && atoi(env) == 0);
  }
  p->code_stride = w->Npad;

  // children, levels by height (forward) and by depth (adjoint); the postorder
  // was validated by build_schedule
  const int T = p->T, I = p->I, NN = 2 * T - 1;
  std::vector<int> left(I), right(I), height(NN, 0), depth(NN, 0);
  // the schedule holds (node, left, right) in an evaluation order that is a post-order
  for (int s = 0; s < I; ++s) {
    const int *rec = &p->steps[size_t(s) * kStepInts];
    const int v = rec[0], l = rec[1], r = rec[2];
    left[v - T] = l;
    right[v - T] = r;
    height[v] = 1 + std::max(height[l], height[r]);
  }
  for (int s = I - 1; s >= 0; --s) {
    const int *rec = &p->steps[size_t(s) * kStepInts];
    depth[rec[1]] = depth[rec[0]] + 1;
    depth[rec[2]] = depth[rec[0]] + 1;
  }
  int H = 0, D = 0;
  for (int v = T; v < NN; ++v) {
    H = std::max(H, height[v]);
    D = std::max(D, depth[v]);
  }
  std::vector<int> fwd, bwd;
  w->fwd_off.push_back(0);
  for (int h = 1; h <= H; ++h) {
    for (int v = T; v < NN; ++v)
      if (height[v] == h) fwd.push_back(v);
    w->fwd_off.push_back(int(fwd.size()));
  }
  w->bwd_off.push_back(0);
  std::vector<int> branch_lvn(size_t(p->B), 1);
  for (int d = 0; d <= D; ++d) {
    const size_t first = bwd.size();
    for (int v = T; v < NN; ++v)
      if (depth[v] == d) bwd.push_back(v);
    const int n = int(bwd.size() - first);
    for (size_t i = first; i < bwd.size(); ++i) {
      const int v = bwd[i];
      branch_lvn[left[v - T]] = n;
      branch_lvn[right[v - T]] = n;
    }
    w->bwd_off.push_back(int(bwd.size()));
  }
  const size_t es = p->elem, SP = size_t(w->SP), b = size_t(p->batch), K = size_t(p->K);
  int rc = TT_OK;
  if (!rc) rc = walloc(p, &w->d_left, I * sizeof(int), "children");
  if (!rc) rc = walloc(p, &w->d_right, I * sizeof(int), "children");
  if (!rc) rc = walloc(p, &w->d_fwd, I * sizeof(int), "levels");
  if (!rc) rc = walloc(p, &w->d_bwd, I * sizeof(int), "levels");
  if (!rc) rc = walloc(p, &w->d_branch_lvn, size_t(p->B) * sizeof(int), "branch levels");
  if (!rc) rc = walloc(p, &p->d_codes, size_t(T) * p->code_stride, "tip codes");
  if (!rc) rc = walloc(p, &p->d_table, 256 * SP * es, "code table");
  if (!rc) rc = walloc(p, &p->d_weights, size_t(p->N) * sizeof(double), "weights");
  if (!rc) rc = walloc(p, &p->d_pmat, b * p->B * K * SP * SP * es, "transition matrices");
  {  // FP32 codon plans keep the children's products for the adjoint (TT_WIDE_STORE_PRODUCTS=0
     // recomputes them): 84.1 -> 80.2 ms per call at 200 tips x 2,608 codon patterns x 16; with 20
     // states the extra stores cost more than the products they save
    const char *env = getenv("TT_WIDE_STORE_PRODUCTS");
    w->store_products = f32 && SP == 64 && !(env && atoi(env) == 0);
  }
  {  // tensor-core adjoint for those plans (TT_WIDE_TC_BWD=0 selects the CUDA-core kernel)
    const char *env = getenv("TT_WIDE_TC_BWD");
    if (!rc && w->store_products && !(env && atoi(env) == 0)) rc = wide_set_tensor_core_adjoint(p, true);
  }
  if (!rc && w->tc) rc = wide_set_tensor_cores(p, true);  // its split P images
  // the pattern-sized buffers (partials, exponents, products, root and
  // gradient chunks) come from wide_alloc_slab once the slab size is chosen
  if (!rc)
    rc = walloc(p, &w->d_pgpart, b * w->nbchunks * (2 * p->S * p->S + p->S + K) * sizeof(double),
                "matrix gradient chunks");
  if (!rc) rc = walloc(p, &p->d_G, b * p->B * K * p->S * p->S * sizeof(double), "dlnL/dP");
  if (!rc) rc = walloc(p, &p->d_rootgrad, b * (p->S + K) * sizeof(double), "root grads");
  if (!rc) rc = walloc(p, &p->d_status, sizeof(int), "status");
  if (rc) return rc;
  cudaError_t e = cudaMemcpy(w->d_left, left.data(), I * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(w->d_right, right.data(), I * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(w->d_fwd, fwd.data(), I * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(w->d_bwd, bwd.data(), I * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(w->d_branch_lvn, branch_lvn.data(), size_t(p->B) * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(p->d_status, 0, sizeof(int));
  if (e == cudaSuccess)
    e = dispatch(p, [](auto W) { return decltype(W)::prepare(); });
  if (e != cudaSuccess) return wcuda(e, "wide-state plan set-up");
  return TT_OK;
}

namespace {

struct SlabBuffers {
  size_t part, expo, prod, root_site, root_expo, log2L, block, gpart, rootpart, site;
  size_t total() const {
    size_t t = 0;
    for (size_t x : {part, expo, prod, root_site, root_expo, log2L, block, gpart, rootpart, site})
      t += x ? std::max(x, size_t(16)) : 0;
    return t;
  }
};

// Pattern-sized buffers for passes over at most n patterns (slab = n when
// the plan works in slabs, 0 for the whole alignment).
SlabBuffers slab_buffers(const tt_plan *p, int n, bool slab) {
  const WideState &w = *p->wide;
  const WideGeo g = wide_geo(p, n);
  const size_t es = p->elem, SP = size_t(w.SP), b = size_t(p->batch), K = size_t(p->K), I = size_t(p->I);
  SlabBuffers x;
  x.part = b * I * K * SP * g.Npad * es;
  x.expo = b * I * K * g.Npad * sizeof(int);
  x.prod = w.store_products ? b * I * K * 2 * SP * g.Npad * es : 0;
  x.root_site = b * K * g.Npad * sizeof(double);
  x.root_expo = b * K * g.Npad * sizeof(int);
  x.log2L = b * g.Npad * sizeof(double);
  x.block = b * g.nblk * sizeof(double);
  x.gpart = b * p->B * g.cmax * K * SP * SP * es;
  x.rootpart = b * g.cmax * K * (SP + 1) * es;
  x.site = slab ? b * size_t(n) * sizeof(double) : 0;
  return x;
}

void free_slab_buffers(tt_plan *p) {
  WideState &w = *p->wide;
  for (void **x : {reinterpret_cast<void **>(&w.d_part), reinterpret_cast<void **>(&w.d_expo),
                   reinterpret_cast<void **>(&w.d_prod), reinterpret_cast<void **>(&w.d_root_site),
                   reinterpret_cast<void **>(&w.d_root_expo), reinterpret_cast<void **>(&w.d_log2L),
                   reinterpret_cast<void **>(&w.d_block_lnl), reinterpret_cast<void **>(&w.d_gpart),
                   reinterpret_cast<void **>(&w.d_rootpart), reinterpret_cast<void **>(&w.d_site)})
    if (*x) {
      cudaFree(*x);
      *x = nullptr;
    }
  p->bytes -= std::min(p->bytes, w.slab_bytes);
  w.slab_bytes = 0;
}

}  // namespace

size_t wide_pattern_bytes(const tt_plan *p, int n) { return slab_buffers(p, n, false).total(); }

int wide_alloc_slab(tt_plan *p, int slab) {
  WideState &w = *p->wide;
  free_slab_buffers(p);
  p->partials_valid = false;
  p->grads_valid = false;
  w.tail_valid = false;
  const SlabBuffers x = slab_buffers(p, slab ? slab : p->N, slab != 0);
  const size_t before = p->bytes;
  int rc = walloc(p, &w.d_part, x.part, "partials");
  if (!rc) rc = walloc(p, &w.d_expo, x.expo, "scale exponents");
  if (!rc && x.prod) rc = walloc(p, &w.d_prod, x.prod, "children's products");
  if (!rc) rc = walloc(p, &w.d_root_site, x.root_site, "root sums");
  if (!rc) rc = walloc(p, &w.d_root_expo, x.root_expo, "root exponents");
  if (!rc) rc = walloc(p, &w.d_log2L, x.log2L, "site log-likelihoods");
  if (!rc) rc = walloc(p, &w.d_block_lnl, x.block, "block sums");
  if (!rc) rc = walloc(p, &w.d_gpart, x.gpart, "gradient chunks");
  if (!rc) rc = walloc(p, &w.d_rootpart, x.rootpart, "root gradient chunks");
  if (!rc && x.site) rc = walloc(p, &w.d_site, x.site, "slab site log-likelihoods");
  w.slab_bytes = p->bytes - before;
  if (rc) {
    free_slab_buffers(p);
    return rc;
  }
  p->slab = slab;
  return TT_OK;
}

bool wide_has_buffers(const tt_plan *p) { return p->wide && p->wide->d_part; }

int wide_set_tensor_cores(tt_plan *p, bool on) {
  WideState *w = p->wide;
  if (!w || p->precision != TT_PRECISION_F32 || w->SP != 64)
    return on ? wfail(TT_ERR_UNSUPPORTED, "the tensor-core post-order serves FP32 codon (> 20-state) plans") : TT_OK;
  const size_t bytes = size_t(p->batch) * p->B * p->K * tcb::kImgFloats * sizeof(float);
  if (on && !w->d_pimg_f) {  // the split P images: 32 KB per (sample, branch, category)
    const int rc = walloc(p, &w->d_pimg_f, bytes, "split transition-matrix images");
    if (rc) return rc;
    w->img_f_valid = false;
  } else if (!on && w->d_pimg_f) {
    cudaFree(w->d_pimg_f);
    w->d_pimg_f = nullptr;
    p->bytes -= std::min(p->bytes, bytes);
  }
  w->tc = on;
  return TT_OK;
}

bool wide_tensor_cores(const tt_plan *p) { return p->wide && p->wide->tc; }

int wide_set_tensor_core_adjoint(tt_plan *p, bool on) {
  WideState *w = p->wide;
  if (!w || p->precision != TT_PRECISION_F32 || w->SP != 64 || !w->store_products)
    return on ? wfail(TT_ERR_UNSUPPORTED,
                      "the tensor-core adjoint serves FP32 codon (> 20-state) plans that keep the children's products")
              : TT_OK;
  if (on && !w->d_pimg) {  // the split P^T images: 32 KB per (sample, branch, category)
    const size_t bytes = size_t(p->batch) * p->B * p->K * tcb::kImgFloats * sizeof(float);
    const int rc = walloc(p, &w->d_pimg, bytes, "split transition-matrix images");
    if (rc) return rc;
    w->img_b_valid = false;
  } else if (!on && w->d_pimg) {
    cudaFree(w->d_pimg);
    w->d_pimg = nullptr;
    p->bytes -= std::min(p->bytes, size_t(p->batch) * p->B * p->K * tcb::kImgFloats * sizeof(float));
  }
  w->tc_bwd = on;
  return TT_OK;
}

bool wide_tensor_core_adjoint(const tt_plan *p) { return p->wide && p->wide->tc_bwd; }

void wide_destroy(tt_plan *p) {
  WideState *w = p->wide;
  if (!w) return;
  void *bufs[] = {w->d_left, w->d_right, w->d_fwd, w->d_bwd, w->d_branch_lvn, w->d_part, w->d_expo, w->d_root_site, w->d_root_expo,
                  w->d_log2L, w->d_block_lnl, w->d_gpart, w->d_rootpart, w->d_pgpart, w->d_prod, w->d_site,
                  w->d_pimg, w->d_pimg_f};
  for (void *x : bufs)
    if (x) cudaFree(x);
  delete w;
  p->wide = nullptr;
}

int wide_set_tips(tt_plan *p, const uint8_t *codes, const double *code_table, int code_count,
                  const double *weights) {
  const int SP = p->wide->SP;
  std::vector<unsigned char> table(size_t(code_count) * SP * p->elem, 0);
  for (int c = 0; c < code_count; ++c)
    for (int j = 0; j < p->S; ++j) {
      const double v = code_table[size_t(c) * p->S + j];
      if (p->precision == TT_PRECISION_F32) {
        const float f = float(v);
        std::memcpy(&table[(size_t(c) * SP + j) * 4], &f, 4);
      } else {
        std::memcpy(&table[(size_t(c) * SP + j) * 8], &v, 8);
      }
    }
  cudaError_t e = cudaMemset(p->d_codes, 0, size_t(p->T) * p->code_stride);
  if (e == cudaSuccess)
    e = cudaMemcpy2D(p->d_codes, p->code_stride, codes, p->N, p->N, p->T, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(p->d_table, table.data(), table.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(p->d_weights, weights, size_t(p->N) * sizeof(double), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return wcuda(e, "tt_plan_set_tips upload");
  return TT_OK;
}

int wide_update_matrices(tt_plan *p, const double *lam, const double *U, const double *W, const double *bl,
                         const double *rates, cudaStream_t s) {
  cudaError_t e = dispatch(p, [&](auto X) { return decltype(X)::pmatrix(p, lam, U, W, bl, rates, s); });
  return e == cudaSuccess ? TT_OK : wcuda(e, "transition-matrix launch");
}

int wide_set_matrices(tt_plan *p, const double *matrices, cudaStream_t s) {
  const int SP = p->wide->SP;
  const long long count = (long long)p->batch * p->B * p->K * SP * SP;
  const unsigned blocks = unsigned((count + 255) / 256);
  if (p->precision == TT_PRECISION_F32)
    wide_pmatrix_copy_kernel<float><<<blocks, 256, 0, s>>>(matrices, static_cast<float *>(p->d_pmat), p->S, SP, count);
  else
    wide_pmatrix_copy_kernel<double><<<blocks, 256, 0, s>>>(matrices, static_cast<double *>(p->d_pmat), p->S, SP,
                                                            count);
  p->launches += 1;
  p->wide->img_f_valid = p->wide->img_b_valid = false;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && p->precision == TT_PRECISION_F32 && SP == 64)  // the tensor-core kernels' images
    e = launch_pimages(p, p->wide->tc, p->wide->tc_bwd, s);
  return e == cudaSuccess ? TT_OK : wcuda(e, "transition-matrix copy launch");
}

int wide_log_likelihood(tt_plan *p, const double *props, const double *freqs, int rescale, bool keep, double *lnl,
                        double *site_lnl, cudaStream_t s) {
  WideState &w = *p->wide;
  if (!p->slab) {
    cudaError_t e = dispatch(
        p, [&](auto X) { return decltype(X)::forward(p, props, freqs, rescale, keep, lnl, site_lnl, 0, p->N, 0, s); });
    return e == cudaSuccess ? TT_OK : wcuda(e, "wide-state post-order launch");
  }
  // slab by slab, lnL summed over slabs; the last slab's post-order stays in
  // the buffers for the gradient
  cudaError_t e = cudaSuccess;
  for (int p0 = 0; p0 < p->N && e == cudaSuccess; p0 += p->slab) {
    const int n = std::min(p->slab, p->N - p0);
    const bool last = p0 + n == p->N;
    e = dispatch(p, [&](auto X) {
      return decltype(X)::forward(p, props, freqs, rescale, keep && last, lnl, site_lnl ? w.d_site : nullptr, p0, n,
                                  p0 > 0, s);
    });
    if (e == cudaSuccess && site_lnl)  // [b][n] rows into columns p0.. of [b][N]
      e = cudaMemcpy2DAsync(site_lnl + p0, size_t(p->N) * sizeof(double), w.d_site, size_t(n) * sizeof(double),
                            size_t(n) * sizeof(double), p->batch, cudaMemcpyDeviceToDevice, s);
  }
  if (e != cudaSuccess) return wcuda(e, "wide-state post-order launch");
  w.tail_valid = keep;
  return TT_OK;
}

int wide_gradient(tt_plan *p, const double *props, const double *freqs, double *grad_matrices,
                  double *grad_frequencies, double *grad_weights, cudaStream_t s) {
  WideState &w = *p->wide;
  cudaError_t e = cudaSuccess;
  if (!p->slab) {
    e = dispatch(p, [&](auto X) { return decltype(X)::backward(p, props, freqs, 0, p->N, 0, s); });
  } else {
    // slabs from the last: its post-order is still in the buffers after a
    // tt_log_likelihood with keep_partials; every other slab's is recomputed
    const int nslab = (p->N + p->slab - 1) / p->slab;
    for (int j = nslab - 1; j >= 0 && e == cudaSuccess; --j) {
      const int p0 = j * p->slab, n = std::min(p->slab, p->N - p0);
      if (!(j == nslab - 1 && w.tail_valid)) {
        e = dispatch(p, [&](auto X) {
          return decltype(X)::forward(p, props, freqs, p->last_rescale, true, nullptr, nullptr, p0, n, 0, s);
        });
        if (e != cudaSuccess) break;
      }
      e = dispatch(p, [&](auto X) { return decltype(X)::backward(p, props, freqs, p0, n, j != nslab - 1, s); });
    }
    w.tail_valid = false;  // the adjoint wrote over the partials
  }
  if (e != cudaSuccess) return wcuda(e, "wide-state adjoint launch");
  const size_t kss = size_t(p->K) * p->S * p->S;
  if (grad_matrices)
    e = cudaMemcpyAsync(grad_matrices, p->d_G, size_t(p->batch) * p->B * kss * sizeof(double),
                        cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess && grad_frequencies)
    e = cudaMemcpyAsync(grad_frequencies, p->d_rootgrad, size_t(p->batch) * p->S * sizeof(double),
                        cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess && grad_weights)
    e = cudaMemcpyAsync(grad_weights, p->d_rootgrad + size_t(p->batch) * p->S,
                        size_t(p->batch) * p->K * sizeof(double), cudaMemcpyDeviceToDevice, s);
  return e == cudaSuccess ? TT_OK : wcuda(e, "gradient copy");
}

int wide_matrices_gradient(tt_plan *p, const double *lam, const double *U, const double *W, const double *bl,
                           const double *rates, double *dlam, double *dU, double *dW, double *dbl, double *drates,
                           cudaStream_t s) {
  cudaError_t e = dispatch(p, [&](auto X) {
    return decltype(X)::pmatrix_backward(p, lam, U, W, bl, rates, dlam, dU, dW, dbl, drates, s);
  });
  return e == cudaSuccess ? TT_OK : wcuda(e, "transition-matrix gradient launch");
}

}  // namespace tt
