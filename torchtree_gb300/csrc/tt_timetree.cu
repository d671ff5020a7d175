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
// One thread per sample walks the pre-order (the transform is a chain along
// each root-to-tip path); one CTA per sample sorts the node heights for the
// coalescent (bitonic sort in shared memory, then one ordered scan for the
// lineage counts and sums).
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
  int *d_pre_child = nullptr;   // [T-2] internal non-root nodes (index - T) in pre-order
  int *d_pre_parent = nullptr;  // [T-2] their parents (index - T)
  int *d_parent = nullptr;      // [2T-2] parent node index of every non-root node
  double *d_lb = nullptr;       // [T-1] lower bounds of internal nodes
  double *d_times = nullptr;    // [T] sampling times
};

namespace {

int tfail(int code, const std::string &m) { return tt::record_error(code, m.c_str()); }

__global__ void ratio_forward_kernel(const int *pre_child, const int *pre_parent, const int *parent,
                                     const double *lb, const double *times, const double *x, double *h,
                                     double *bl, double *logdet, int T, int batch) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  const int I = T - 1;
  const double *xb = x + size_t(b) * I;
  double *hb = h + size_t(b) * I;
  hb[I - 1] = xb[I - 1];  // root height
  double ld = 0.0;
  for (int s = 0; s < I - 1; ++s) {
    const int v = pre_child[s], pv = pre_parent[s];
    const double span = hb[pv] - lb[v];
    hb[v] = lb[v] + xb[v] * span;
    ld += log(span);
  }
  logdet[b] = ld;
  if (bl)
    for (int n = 0; n < 2 * T - 2; ++n) {
      const double hn = n < T ? times[n] : hb[n - T];
      bl[size_t(b) * (2 * T - 2) + n] = hb[parent[n] - T] - hn;
    }
}

// gx holds g_h on entry (filled here), dlnL/dx on exit
__global__ void ratio_backward_kernel(const int *pre_child, const int *pre_parent, const int *parent,
                                      const double *lb, const double *x, const double *h, const double *gh_in,
                                      const double *gbl, const double *gld, double *gx, int T, int batch) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  const int I = T - 1;
  const double *xb = x + size_t(b) * I, *hb = h + size_t(b) * I;
  double *g = gx + size_t(b) * I;
  for (int v = 0; v < I; ++v) g[v] = gh_in ? gh_in[size_t(b) * I + v] : 0.0;
  if (gbl)
    for (int n = 0; n < 2 * T - 2; ++n) {
      const double gn = gbl[size_t(b) * (2 * T - 2) + n];
      g[parent[n] - T] += gn;
      if (n >= T) g[n - T] -= gn;
    }
  const double gl = gld ? gld[b] : 0.0;
  for (int s = I - 2; s >= 0; --s) {
    const int v = pre_child[s], pv = pre_parent[s];
    const double span = hb[pv] - lb[v];
    const double gv = g[v];
    g[v] = gv * span;                          // dh_v/dx_v = span
    g[pv] += gv * xb[v] + gl / span;           // dh_v/dh_p = x_v; d log(span)/dh_p
  }
  // the root entry keeps g_h[root] (h_root = x_root)
}

// one CTA per sample: heights of all 2T-1 nodes, bitonic sort in shared memory
__global__ void coalescent_kernel(const double *times, const double *hint, const double *theta, int T, int n2,
                                  double *logp, double *gh, double *gtheta) {
  extern __shared__ __align__(16) unsigned char sm[];
  double *key = reinterpret_cast<double *>(sm);  // [n2]
  int *idx = reinterpret_cast<int *>(key + n2);  // [n2]
  const int b = blockIdx.x, tid = threadIdx.x, NT = blockDim.x;
  const int n = 2 * T - 1, I = T - 1;
  for (int e = tid; e < n2; e += NT) {
    if (e < n) {
      key[e] = e < T ? times[e] : hint[size_t(b) * I + e - T];
      idx[e] = e;
    } else {
      key[e] = INFINITY;
      idx[e] = e;
    }
  }
  __syncthreads();
  for (int k = 2; k <= n2; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int e = tid; e < n2; e += NT) {
        const int o = e ^ j;
        if (o > e) {
          const bool up = (e & k) == 0;
          const double ke = key[e], ko = key[o];
          const int ie = idx[e], io = idx[o];
          const bool gt = ke > ko || (ke == ko && ie > io);
          if (gt == up) {
            key[e] = ko, key[o] = ke;
            idx[e] = io, idx[o] = ie;
          }
        }
      }
      __syncthreads();
    }
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
  // pre-order of the non-root internal nodes: reversed post-order
  std::vector<int> pc, pp;
  for (int s = I - 2; s >= 0; --s) {
    const int v = postorder[3 * s];
    pc.push_back(v - T);
    pp.push_back(parent[v] - T);
  }
  tt_time_tree *t = new tt_time_tree();
  cudaGetDevice(&t->device);
  t->T = T;
  cudaError_t e = cudaSuccess;
  auto up = [&](auto **dst, const auto *src, size_t n) {
    if (e != cudaSuccess) return;
    e = cudaMalloc(reinterpret_cast<void **>(dst), std::max<size_t>(n, 1) * sizeof(**dst));
    if (e == cudaSuccess && n) e = cudaMemcpy(*dst, src, n * sizeof(**dst), cudaMemcpyHostToDevice);
  };
  up(&t->d_pre_child, pc.data(), pc.size());
  up(&t->d_pre_parent, pp.data(), pp.size());
  up(&t->d_parent, parent.data(), size_t(2 * T - 2));
  up(&t->d_lb, lb.data(), lb.size());
  up(&t->d_times, sampling_times, size_t(T));
  if (e != cudaSuccess) {
    tt_time_tree_destroy(t);
    return tfail(TT_ERR_OUT_OF_MEMORY, std::string("time-tree upload: ") + cudaGetErrorString(e));
  }
  *tree = t;
  return TT_OK;
}

int tt_time_tree_destroy(tt_time_tree *t) {
  if (!t) return TT_OK;
  void *bufs[] = {t->d_pre_child, t->d_pre_parent, t->d_parent, t->d_lb, t->d_times};
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
  ratio_forward_kernel<<<(batch + 127) / 128, 128, 0, s>>>(t->d_pre_child, t->d_pre_parent, t->d_parent, t->d_lb,
                                                          t->d_times, ratios, heights, branch_lengths,
                                                          log_det_jacobian, t->T, batch);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? TT_OK : tfail(TT_ERR_CUDA, std::string("ratio transform launch: ") + cudaGetErrorString(e));
}

int tt_ratio_transform_backward(tt_time_tree *t, int32_t batch, const double *ratios, const double *heights,
                                const double *grad_heights, const double *grad_branch_lengths,
                                const double *grad_log_det, double *grad_ratios, void *stream) {
  if (!t || !ratios || !heights || !grad_ratios || batch < 1)
    return tfail(TT_ERR_INVALID_ARGUMENT, "NULL argument or empty batch");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  ratio_backward_kernel<<<(batch + 127) / 128, 128, 0, s>>>(t->d_pre_child, t->d_pre_parent, t->d_parent, t->d_lb,
                                                           ratios, heights, grad_heights, grad_branch_lengths,
                                                           grad_log_det, grad_ratios, t->T, batch);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? TT_OK
                          : tfail(TT_ERR_CUDA, std::string("ratio transform backward launch: ") + cudaGetErrorString(e));
}

int tt_constant_coalescent(tt_time_tree *t, int32_t batch, const double *heights, const double *theta,
                           double *log_prob, double *grad_heights, double *grad_theta, void *stream) {
  if (!t || !heights || !theta || !log_prob || batch < 1)
    return tfail(TT_ERR_INVALID_ARGUMENT, "NULL argument or empty batch");
  const int n = 2 * t->T - 1;
  if (n > 8191) return tfail(TT_ERR_UNSUPPORTED, "the coalescent kernel sorts at most 4,096 tips");
  int n2 = 1;
  while (n2 < n) n2 <<= 1;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t smem = size_t(n2) * (sizeof(double) + sizeof(int));
  cudaError_t e = cudaFuncSetAttribute(coalescent_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e == cudaSuccess) {  // every internal node's gradient is written once: no clearing needed
    coalescent_kernel<<<batch, 256, smem, s>>>(t->d_times, heights, theta, t->T, n2, log_prob, grad_heights,
                                               grad_theta);
    e = cudaGetLastError();
  }
  return e == cudaSuccess ? TT_OK : tfail(TT_ERR_CUDA, std::string("coalescent launch: ") + cudaGetErrorString(e));
}

}  // extern "C"
