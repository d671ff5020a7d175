// Time-tree operations around the likelihood, batched over samples:
//
// * node-height ratio transform and its log-determinant
//   (torchtree/evolution/tree_height_transform.py:7-99, GeneralNodeHeightTransform):
//     h[root] = x[root];  h[v] = lb[v] + x[v] (h[parent v] - lb[v]) in pre-order,
//     log|J| = sum over non-root internal v of log(h[parent v] - lb[v]),
//   with lb[v] the largest sampling time below v, plus branch lengths
//   h[parent] - h[child] (tree_model.py:23-40);
// * constant-size coalescent log-density
//   (torchtree/evolution/coalescent.py:86-134, ConstantCoalescent.log_prob):
//     log p = -sum_i C(l_i, 2) (t_(i+1) - t_i) / theta - (T - 1) log theta
//   over the sorted node heights t with l_i lineages between t_i and t_(i+1).
//
// One CTA per sample. The transform walks the tree level by level (all nodes
// of one depth in parallel, a barrier between depths) on the sample's row in
// shared memory, loaded and stored coalesced; its adjoint walks the levels
// back, each parent gathering its internal children's terms (fixed order, no
// atomics). The coalescent sorts the sample's internal heights (bitonic sort
// in shared memory), merges them by rank with the tip times sorted once at
// set-up, and sums over the merged order with a block prefix sum of the
// lineage counts.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/torchtree_gb300.h"
#include "tt_common.cuh"
#include "tt_launch.h"

struct tt_time_tree {
  int device = 0;
  int T = 0;
  int levels = 0;               // depths of internal nodes (root: depth 0)
  int *d_lvl_nodes = nullptr;   // [T-1] internal nodes (index - T) by depth, root first
  int *d_lvl_off = nullptr;     // [levels + 1] offsets into d_lvl_nodes
  int2 *d_kids = nullptr;       // [T-1] children (node indices) of internal node index - T
  int *d_parent = nullptr;      // [2T-2] parent node index of every non-root node
  double *d_lb = nullptr;       // [T-1] lower bounds of internal nodes
  double *d_times = nullptr;    // [T] sampling times
  double *d_tip_t = nullptr;    // [T] sampling times in ascending (time, tip) order
  int *d_tip_i = nullptr;       // [T] the tips in that order
};

namespace {

constexpr int kTimeTreeThreads = 128;  // threads of the per-sample transform CTAs

int tfail(int code, const std::string &m) { return tt::record_error(code, m.c_str()); }

// sum of v over the CTA in a fixed order (warps, then warp totals); valid in thread 0
__device__ __forceinline__ double cta_sum(double v, double *wred) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) wred[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < nw; ++w) t += wred[w];
  return t;
}

__global__ void ratio_forward_kernel(const int *lvl_nodes, const int *lvl_off, int levels, const int *parent,
                                     const double *lb, const double *times, const double *x, double *h,
                                     double *bl, double *logdet, int T) {
  extern __shared__ __align__(16) double rs[];
  __shared__ double wred[32];
  const int b = blockIdx.x, tid = threadIdx.x, NT = blockDim.x, I = T - 1;
  double *xs = rs, *hs = rs + I;  // this sample's ratios and heights
  for (int v = tid; v < I; v += NT) xs[v] = x[size_t(b) * I + v];
  __syncthreads();
  if (tid == 0) hs[I - 1] = xs[I - 1];  // root height
  __syncthreads();
  double ld = 0.0;
  for (int d = 1; d < levels; ++d) {  // one depth at a time, parents before children
    for (int e = lvl_off[d] + tid; e < lvl_off[d + 1]; e += NT) {
      const int v = lvl_nodes[e], pv = parent[v + T] - T;
      const double span = hs[pv] - lb[v];
      hs[v] = lb[v] + xs[v] * span;
      ld += log(span);
    }
    __syncthreads();
  }
  const double tot = cta_sum(ld, wred);
  if (tid == 0) logdet[b] = tot;
  for (int v = tid; v < I; v += NT) h[size_t(b) * I + v] = hs[v];
  if (bl)
    for (int n = tid; n < 2 * T - 2; n += NT) {
      const double hn = n < T ? times[n] : hs[n - T];
      bl[size_t(b) * (2 * T - 2) + n] = hs[parent[n] - T] - hn;
    }
}

// dlnL/dx from dlnL/dh, dlnL/dbranch lengths and dlnL/dlog|J|
__global__ void ratio_backward_kernel(const int *lvl_nodes, const int *lvl_off, int levels, const int2 *kids,
                                      const double *lb, const double *x, const double *h, const double *gh_in,
                                      const double *gbl, const double *gld, double *gx, int T) {
  extern __shared__ __align__(16) double rs[];
  const int b = blockIdx.x, tid = threadIdx.x, NT = blockDim.x, I = T - 1, B = 2 * T - 2;
  double *xs = rs, *hs = rs + I, *g = rs + 2 * I;
  for (int v = tid; v < I; v += NT) {
    xs[v] = x[size_t(b) * I + v];
    hs[v] = h[size_t(b) * I + v];
    double gv = gh_in ? gh_in[size_t(b) * I + v] : 0.0;
    if (gbl) {  // branch c above node c has length h[parent c] - h[c]
      const int2 k = kids[v];
      gv += gbl[size_t(b) * B + k.x] + gbl[size_t(b) * B + k.y];
      if (v < I - 1) gv -= gbl[size_t(b) * B + v + T];
    }
    g[v] = gv;
  }
  __syncthreads();
  const double gl = gld ? gld[b] : 0.0;
  // deepest parents first: a parent gathers d/dh of its internal children,
  // which are final, then turns them into d/dx
  for (int d = levels - 2; d >= 0; --d) {
    for (int e = lvl_off[d] + tid; e < lvl_off[d + 1]; e += NT) {
      const int p = lvl_nodes[e];
      const int2 k = kids[p];
      double gp = g[p];
      const int c2[2] = {k.x, k.y};
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        if (c2[c] < T) continue;
        const int cv = c2[c] - T;
        const double span = hs[p] - lb[cv], gc = g[cv];
        g[cv] = gc * span;                   // dh_c/dx_c = span
        gp += gc * xs[cv] + gl / span;       // dh_c/dh_p = x_c; d log(span)/dh_p
      }
      g[p] = gp;
    }
    __syncthreads();
  }
  // the root entry keeps d/dh[root] (h_root = x_root)
  for (int v = tid; v < I; v += NT) gx[size_t(b) * I + v] = g[v];
}

// one CTA per sample: the internal heights sorted in shared memory (bitonic,
// ties by node index), merged by rank with the tips (sorted at set-up; a tip
// precedes an internal node of equal height, as its index is smaller)
__global__ void coalescent_kernel(const double *tip_t, const int *tip_i, const double *hint, const double *theta,
                                  int T, int m2, double *logp, double *gh, double *gtheta) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int b = blockIdx.x, tid = threadIdx.x, NT = blockDim.x;
  const int n = 2 * T - 1, I = T - 1;
  double *ik = reinterpret_cast<double *>(sm);  // [m2] internal heights
  double *key = ik + m2;                        // [n] merged heights
  double *tk = key + n;                         // [T] tip times, sorted
  int *ii = reinterpret_cast<int *>(tk + T);    // [m2] internal node indices
  int *idx = ii + m2;                           // [n] merged node indices
  for (int e = tid; e < m2; e += NT) {
    ik[e] = e < I ? hint[size_t(b) * I + e] : INFINITY;
    ii[e] = T + e;
  }
  for (int e = tid; e < T; e += NT) tk[e] = tip_t[e];
  __syncthreads();
  for (int k = 2; k <= m2; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int e = tid; e < m2; e += NT) {
        const int o = e ^ j;
        if (o > e) {
          const bool up = (e & k) == 0;
          const double ke = ik[e], ko = ik[o];
          const int ie = ii[e], io = ii[o];
          const bool gt = ke > ko || (ke == ko && ie > io);
          if (gt == up) {
            ik[e] = ko, ik[o] = ke;
            ii[e] = io, ii[o] = ie;
          }
        }
      }
      __syncthreads();
    }
  for (int a = tid; a < I; a += NT) {  // tips at or below this height come first
    const double v = ik[a];
    int lo = 0, hi = T;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (tk[mid] <= v) lo = mid + 1;
      else hi = mid;
    }
    key[a + lo] = v;
    idx[a + lo] = ii[a];
  }
  for (int t = tid; t < T; t += NT) {  // internal nodes strictly below this time come first
    const double v = tk[t];
    int lo = 0, hi = I;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (ik[mid] < v) lo = mid + 1;
      else hi = mid;
    }
    key[t + lo] = v;
    idx[t + lo] = tip_i[t];
  }
  __syncthreads();
  // Lineages through sorted position p: L_p = (#tips at or before p) - (#internal
  // nodes at or before p), a block-wide prefix sum over contiguous chunks of
  // positions.  With c_p = L_p (L_p - 1) / 2 for p < n - 1 (0 at the last):
  //   log p = -sum_p c_p (t_{p+1} - t_p) / theta - (T - 1) log theta,
  //   d/dt_p = (c_p - c_{p-1}) / theta  (each internal node written once),
  //   d/dtheta = sum_p c_p (t_{p+1} - t_p) / theta^2 - (T - 1) / theta.
  // The sum runs in a fixed order (per-thread chunks, then warps, then warp totals).
  const double th = theta[b], inv_th = 1.0 / th;
  const int E = (n + NT - 1) / NT;
  const int p0 = min(n, tid * E), p1 = min(n, p0 + E);
  int dsum = 0;
  for (int p = p0; p < p1; ++p) dsum += idx[p] < T ? 1 : -1;
  const int lane = tid & 31, warp = tid >> 5, NW = (NT + 31) >> 5;
  int incl = dsum;  // inclusive warp scan
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  __shared__ int wsum[32];
  __shared__ double wacc[32];
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  int off = incl - dsum;
  for (int w = 0; w < warp; ++w) off += wsum[w];
  int L = off;
  double c_prev = 0.5 * double(off) * double(off - 1);  // c_{p0 - 1} (0 before the first position)
  if (p0 == 0) c_prev = 0.0;
  double acc = 0.0;
  for (int p = p0; p < p1; ++p) {
    L += idx[p] < T ? 1 : -1;
    const double c = p < n - 1 ? 0.5 * double(L) * double(L - 1) : 0.0;
    if (p < n - 1) acc = fma(c, key[p + 1] - key[p], acc);
    if (gh && idx[p] >= T) gh[size_t(b) * I + idx[p] - T] = (c - c_prev) * inv_th;
    c_prev = c;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) wacc[warp] = acc;
  __syncthreads();
  if (tid == 0) {
    double total = 0.0;
    for (int w = 0; w < NW; ++w) total += wacc[w];
    logp[b] = -total * inv_th - double(T - 1) * log(th);
    if (gtheta) gtheta[b] = total * inv_th * inv_th - double(T - 1) * inv_th;
  }
}

}  // namespace

extern "C" {

int tt_time_tree_create(tt_time_tree **tree, int32_t tip_count, const int32_t *postorder,
                        const double *sampling_times) {
  if (!tree || !postorder || !sampling_times) return tfail(TT_ERR_INVALID_ARGUMENT, "NULL argument");
  *tree = nullptr;
  const int T = tip_count, I = T - 1, NN = 2 * T - 1;
  if (T < 2) return tfail(TT_ERR_INVALID_ARGUMENT, "a tree needs at least 2 tips");
  std::vector<int> parent(NN, -1), left(NN, -1), right(NN, -1);
  std::vector<char> done(NN, 0);
  for (int t = 0; t < T; ++t) done[t] = 1;
  for (int s = 0; s < I; ++s) {
    const int v = postorder[3 * s], l = postorder[3 * s + 1], r = postorder[3 * s + 2];
    if (v < T || v >= NN || l < 0 || l >= NN || r < 0 || r >= NN || done[v] || !done[l] || !done[r] ||
        parent[l] >= 0 || parent[r] >= 0 || l == r)
      return tfail(TT_ERR_INVALID_ARGUMENT, "postorder is not a valid post-order of a binary tree");
    parent[l] = v, parent[r] = v, left[v] = l, right[v] = r, done[v] = 1;
  }
  if (postorder[3 * (I - 1)] != NN - 1) return tfail(TT_ERR_INVALID_ARGUMENT, "the root must be node 2T-2, last");
  std::vector<double> lb(I, 0.0);
  for (int s = 0; s < I; ++s) {
    const int v = postorder[3 * s];
    auto h = [&](int c) { return c < T ? sampling_times[c] : lb[c - T]; };
    lb[v - T] = std::max(h(left[v]), h(right[v]));
  }
  // internal nodes by depth (root at depth 0; a parent precedes its children)
  std::vector<int> depth(NN, 0);
  int levels = 1;
  for (int s = I - 1; s >= 0; --s) {  // reversed post-order: parents first
    const int v = postorder[3 * s];
    if (v != NN - 1) depth[v] = depth[parent[v]] + 1;
    levels = std::max(levels, depth[v] + 1);
  }
  std::vector<int> lvl_off(levels + 1, 0), lvl_nodes;
  lvl_nodes.reserve(I);
  for (int d = 0; d < levels; ++d) {
    lvl_off[d] = int(lvl_nodes.size());
    for (int v = T; v < NN; ++v)
      if (depth[v] == d) lvl_nodes.push_back(v - T);
  }
  lvl_off[levels] = int(lvl_nodes.size());
  std::vector<int2> kids(I);
  for (int v = T; v < NN; ++v) kids[v - T] = make_int2(left[v], right[v]);
  // tips in ascending (sampling time, index) order
  std::vector<int> tip_i(T);
  for (int i = 0; i < T; ++i) tip_i[i] = i;
  std::sort(tip_i.begin(), tip_i.end(), [&](int a, int b) {
    return sampling_times[a] != sampling_times[b] ? sampling_times[a] < sampling_times[b] : a < b;
  });
  std::vector<double> tip_t(T);
  for (int i = 0; i < T; ++i) tip_t[i] = sampling_times[tip_i[i]];
  tt_time_tree *t = new tt_time_tree();
  cudaGetDevice(&t->device);
  t->T = T;
  t->levels = levels;
  cudaError_t e = cudaSuccess;
  auto up = [&](auto **dst, const auto *src, size_t n) {
    if (e != cudaSuccess) return;
    e = cudaMalloc(reinterpret_cast<void **>(dst), std::max<size_t>(n, 1) * sizeof(**dst));
    if (e == cudaSuccess && n) e = cudaMemcpy(*dst, src, n * sizeof(**dst), cudaMemcpyHostToDevice);
  };
  up(&t->d_lvl_nodes, lvl_nodes.data(), lvl_nodes.size());
  up(&t->d_lvl_off, lvl_off.data(), lvl_off.size());
  up(&t->d_kids, kids.data(), kids.size());
  up(&t->d_parent, parent.data(), size_t(2 * T - 2));
  up(&t->d_lb, lb.data(), lb.size());
  up(&t->d_times, sampling_times, size_t(T));
  up(&t->d_tip_t, tip_t.data(), tip_t.size());
  up(&t->d_tip_i, tip_i.data(), tip_i.size());
  if (e != cudaSuccess) {
    tt_time_tree_destroy(t);
    return tfail(TT_ERR_OUT_OF_MEMORY, std::string("time-tree upload: ") + cudaGetErrorString(e));
  }
  *tree = t;
  return TT_OK;
}

int tt_time_tree_destroy(tt_time_tree *t) {
  if (!t) return TT_OK;
  void *bufs[] = {t->d_lvl_nodes, t->d_lvl_off, t->d_kids, t->d_parent, t->d_lb, t->d_times, t->d_tip_t, t->d_tip_i};
  for (void *p : bufs)
    if (p) cudaFree(p);
  delete t;
  return TT_OK;
}

int tt_ratio_transform(tt_time_tree *t, int32_t batch, const double *ratios, double *heights,
                       double *branch_lengths, double *log_det_jacobian, void *stream) {
  if (!t || !ratios || !heights || !log_det_jacobian || batch < 1)
    return tfail(TT_ERR_INVALID_ARGUMENT, "NULL argument or empty batch");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t smem = 2 * size_t(t->T - 1) * sizeof(double);
  if (3 * size_t(t->T - 1) * sizeof(double) > 227 * 1024)
    return tfail(TT_ERR_UNSUPPORTED, "the ratio transform holds a sample's rows in shared memory: at most 9,600 tips");
  cudaError_t e = tt::kernel_smem(ratio_forward_kernel, smem);
  if (e == cudaSuccess) {
    ratio_forward_kernel<<<batch, kTimeTreeThreads, smem, s>>>(t->d_lvl_nodes, t->d_lvl_off, t->levels, t->d_parent,
                                                               t->d_lb, t->d_times, ratios, heights, branch_lengths,
                                                               log_det_jacobian, t->T);
    e = cudaGetLastError();
  }
  return e == cudaSuccess ? TT_OK : tfail(TT_ERR_CUDA, std::string("ratio transform launch: ") + cudaGetErrorString(e));
}

int tt_ratio_transform_backward(tt_time_tree *t, int32_t batch, const double *ratios, const double *heights,
                                const double *grad_heights, const double *grad_branch_lengths,
                                const double *grad_log_det, double *grad_ratios, void *stream) {
  if (!t || !ratios || !heights || !grad_ratios || batch < 1)
    return tfail(TT_ERR_INVALID_ARGUMENT, "NULL argument or empty batch");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t smem = 3 * size_t(t->T - 1) * sizeof(double);
  if (smem > 227 * 1024)
    return tfail(TT_ERR_UNSUPPORTED, "the ratio transform holds a sample's rows in shared memory: at most 9,600 tips");
  cudaError_t e = tt::kernel_smem(ratio_backward_kernel, smem);
  if (e == cudaSuccess) {
    ratio_backward_kernel<<<batch, kTimeTreeThreads, smem, s>>>(t->d_lvl_nodes, t->d_lvl_off, t->levels, t->d_kids,
                                                                t->d_lb, ratios, heights, grad_heights,
                                                                grad_branch_lengths, grad_log_det, grad_ratios, t->T);
    e = cudaGetLastError();
  }
  return e == cudaSuccess ? TT_OK
                          : tfail(TT_ERR_CUDA, std::string("ratio transform backward launch: ") + cudaGetErrorString(e));
}

int tt_constant_coalescent(tt_time_tree *t, int32_t batch, const double *heights, const double *theta,
                           double *log_prob, double *grad_heights, double *grad_theta, void *stream) {
  if (!t || !heights || !theta || !log_prob || batch < 1)
    return tfail(TT_ERR_INVALID_ARGUMENT, "NULL argument or empty batch");
  const int T = t->T, I = T - 1, n = 2 * T - 1;
  if (T > 4096) return tfail(TT_ERR_UNSUPPORTED, "the coalescent kernel sorts at most 4,096 tips");
  int m2 = 1;
  while (m2 < I) m2 <<= 1;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t smem = size_t(m2 + n + T) * sizeof(double) + size_t(m2 + n) * sizeof(int);
  cudaError_t e = tt::kernel_smem(coalescent_kernel, smem);
  if (e == cudaSuccess) {  // every internal node's gradient is written once: no clearing needed
    coalescent_kernel<<<batch, 256, smem, s>>>(t->d_tip_t, t->d_tip_i, heights, theta, T, m2, log_prob,
                                               grad_heights, grad_theta);
    e = cudaGetLastError();
  }
  return e == cudaSuccess ? TT_OK : tfail(TT_ERR_CUDA, std::string("coalescent launch: ") + cudaGetErrorString(e));
}

}  // extern "C"
