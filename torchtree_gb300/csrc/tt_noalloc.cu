// tt_log_likelihood_static: the FP64 log-likelihood without any device
// allocation.
//
// Some callers cannot call cudaMalloc: code that runs inside an
// application's own memory manager (which owns every device byte and
// forbids other allocations), and embedding hosts that give a plug-in
// device pointers but no permission to allocate.  The plan-based entry
// points allocate their workspace in tt_plan_create, so they are closed
// to those callers.  This entry point takes every input and output from
// the caller and keeps its scratch (step table, transition matrices in
// step order, padded tip-code table, per-tile sums, status word) in one
// file-scope __device__ array of kScratchBytes, which every GPU that loads
// the library holds until the process exits.
//
// Every call looks up the array's device address on the current device with
// cudaGetSymbolAddress (the first call on a device loads the module), so a
// context that was torn down and rebuilt gets the array's new address.  The
// host-side schedule is built in static host arrays, not on the caller's
// stack, under one lock that serialises the host side of every call.  The
// call refuses a stream that is being captured (its host-to-device copies
// come from pageable memory), and it synchronises the stream before it
// returns so that the kernel's status word is read back: a bounded wait that
// gave up is returned as TT_ERR_DEVICE_TIMEOUT.  All calls share the array
// and it keeps the last call's contents; calls whose work overlaps on the
// GPU (two streams, two processes' worth of host threads bypassing the lock)
// race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/torchtree_gb300.h"
#include "tt_launch.h"

namespace {

constexpr size_t kScratchBytes = size_t(8) << 20;  // 8 MiB of scratch
constexpr int kMaxTips = 1024;
constexpr int kTableRows = 256;  // codes are uint8: pad the table to every value

}  // namespace

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

namespace {

// Serialises the host side of every call: the static host arrays below and
// the order of the copies into the shared device array.
std::mutex g_scratch_lock;

int fail(int code, const char *msg) { return tt::record_error(code, msg); }

int fail_cuda(const char *what, cudaError_t e) {
  char buf[240];
  snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
  return fail(TT_ERR_CUDA, buf);
}

// Device address of g_scratch in the current device's context, looked up on
// every call (cheap once the module is loaded) so that it is never stale.
int scratch_address(unsigned char **out) {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
  if (e != cudaSuccess) return fail_cuda("cudaGetSymbolAddress of the static scratch failed", e);
  *out = static_cast<unsigned char *>(p);
  return TT_OK;
}

// Host working arrays of one call (about 120 KB), kept off the caller's stack:
// plug-in hosts may run this on worker threads with small stacks.  Guarded by
// g_scratch_lock.
struct HostTables {
  int left[2 * kMaxTips], right[2 * kMaxTips], parent[2 * kMaxTips], need[2 * kMaxTips];
  int first[2 * kMaxTips], slot[2 * kMaxTips], order[kMaxTips];
  int stk_node[2 * kMaxTips];
  unsigned char stk_state[2 * kMaxTips], done[2 * kMaxTips];
  int steps[(kMaxTips - 1) * tt::kStepInts];
  int branch_pos[2 * kMaxTips - 2];
};
HostTables g_host;

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Post-order schedule with shared-memory slots (forward only), built in
// the static host arrays: the child whose subtree needs more slots is
// evaluated first, so at most log2(T)+1 slots are live.
int static_schedule(int T, const int32_t *post, HostTables &h, int *slots_out) {
  const int I = T - 1, NN = 2 * T - 1;
  int *left = h.left, *right = h.right, *parent = h.parent, *need = h.need;
  int *first = h.first, *slot = h.slot, *order = h.order, *stk_node = h.stk_node;
  unsigned char *stk_state = h.stk_state, *done = h.done;
  int *steps = h.steps, *branch_pos = h.branch_pos;
  for (int v = 0; v < NN; ++v) {
    left[v] = right[v] = parent[v] = first[v] = slot[v] = -1;
    need[v] = 0;
    done[v] = v < T;
  }
  for (int s = 0; s < I; ++s) {
    const int v = post[3 * s], l = post[3 * s + 1], r = post[3 * s + 2];
    if (v < T || v >= NN || l < 0 || l >= NN || r < 0 || r >= NN || l == r || l == v || r == v)
      return fail(TT_ERR_INVALID_ARGUMENT, "postorder triple out of range");
    if (done[v]) return fail(TT_ERR_INVALID_ARGUMENT, "a node appears twice as a parent");
    if (!done[l] || !done[r]) return fail(TT_ERR_INVALID_ARGUMENT, "postorder uses a child before it is computed");
    if (parent[l] >= 0 || parent[r] >= 0) return fail(TT_ERR_INVALID_ARGUMENT, "a child has two parents");
    left[v] = l;
    right[v] = r;
    parent[l] = parent[r] = v;
    done[v] = 1;
    const int f = need[l] >= need[r] ? l : r, g = f == l ? r : l;
    first[v] = f;
    int n = need[f] > (f >= T) + need[g] ? need[f] : (f >= T) + need[g];
    need[v] = n > 1 ? n : 1;
  }
  const int root = post[3 * (I - 1)];
  if (root != 2 * T - 2) return fail(TT_ERR_INVALID_ARGUMENT, "the last postorder triple must be the root 2T-2");
  for (int v = 0; v < NN; ++v)
    if (v != root && parent[v] < 0) return fail(TT_ERR_INVALID_ARGUMENT, "a node is not connected to the root");
  int top = 0, count = 0;
  stk_node[0] = root;
  stk_state[0] = 0;
  while (top >= 0) {
    const int v = stk_node[top];
    if (v < T) {
      --top;
    } else if (stk_state[top] == 0) {
      stk_state[top] = 1;
      ++top;
      stk_node[top] = first[v];
      stk_state[top] = 0;
    } else if (stk_state[top] == 1) {
      stk_state[top] = 2;
      ++top;
      stk_node[top] = first[v] == left[v] ? right[v] : left[v];
      stk_state[top] = 0;
    } else {
      order[count++] = v;
      --top;
    }
  }
  unsigned long long used = 0;
  int slots = 1;
  for (int s = 0; s < I; ++s) {
    const int v = order[s], l = left[v], r = right[v];
    int *rec = steps + s * tt::kStepInts;
    for (int k = 0; k < tt::kStepInts; ++k) rec[k] = -1;
    rec[0] = v;
    rec[1] = l;
    rec[2] = r;
    rec[3] = l >= T ? slot[l] : -1;
    rec[4] = r >= T ? slot[r] : -1;
    if (rec[3] >= 0) used &= ~(1ull << rec[3]);
    if (rec[4] >= 0) used &= ~(1ull << rec[4]);
    if (v != root) {
      int f = 0;
      while (f < 64 && (used >> f) & 1ull) ++f;
      if (f == 64) return fail(TT_ERR_UNSUPPORTED, "tree needs more than 64 shared-memory slots");
      used |= 1ull << f;
      rec[5] = f;
      slot[v] = f;
      if (f + 1 > slots) slots = f + 1;
    }
    branch_pos[l] = 2 * s;
    branch_pos[r] = 2 * s + 1;
  }
  *slots_out = slots;
  return TT_OK;
}

}  // namespace

extern "C" int tt_log_likelihood_static(int32_t tip_count, const int32_t *postorder, int32_t state_count,
                                        int32_t category_count, int32_t pattern_count, int32_t batch,
                                        const uint8_t *codes, const double *code_table, int32_t code_count,
                                        const double *weights, const double *matrices,
                                        const double *category_weights, const double *frequencies,
                                        int32_t rescale, double *log_likelihood, void *stream) {
  if (!postorder || !codes || !code_table || !weights || !matrices || !category_weights || !frequencies ||
      !log_likelihood)
    return fail(TT_ERR_INVALID_ARGUMENT, "NULL argument");
  if (tip_count < 2 || tip_count > kMaxTips)
    return fail(TT_ERR_INVALID_ARGUMENT, "tt_log_likelihood_static supports 2 to 1024 tips");
  if (state_count != 4) return fail(TT_ERR_UNSUPPORTED, "tt_log_likelihood_static supports 4 states");
  if (category_count < 1 || category_count > 8)
    return fail(TT_ERR_INVALID_ARGUMENT, "category_count must be in [1, 8]");
  if (pattern_count < 1 || batch < 1 || batch > 65535)
    return fail(TT_ERR_INVALID_ARGUMENT, "pattern_count and batch must be >= 1 (batch <= 65535)");
  if (code_count < 1 || code_count > kTableRows)
    return fail(TT_ERR_INVALID_ARGUMENT, "code_count must be in [1, 256]");

  const int T = tip_count, I = T - 1, B = 2 * T - 2, S = 4, K = category_count, N = pattern_count;
  const int kss = K * S * S;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(s, &capture);
  if (e != cudaSuccess) return fail_cuda("cudaStreamIsCapturing failed", e);
  if (capture != cudaStreamCaptureStatusNone)
    return fail(TT_ERR_UNSUPPORTED,
                "tt_log_likelihood_static must not be called on a capturing stream (its schedule is copied "
                "from pageable host memory and its status is read back synchronously)");
  int smem_max = 0, dev = 0;
  e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail_cuda("cudaGetDevice failed", e);
  e = cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return fail_cuda("cudaDeviceGetAttribute failed", e);

  std::lock_guard<std::mutex> guard(g_scratch_lock);
  const int *steps = g_host.steps, *branch_pos = g_host.branch_pos;
  int slots = 0;
  int rc = static_schedule(T, postorder, g_host, &slots);
  if (rc != TT_OK) return rc;
  int tile = 0;
  for (int t : tt::kFwdTilesF64)
    if (!tile && tt::prune_smem_bytes<double>(S, K, kTableRows, slots, t, false) <= size_t(smem_max)) tile = t;
  if (!tile) return fail(TT_ERR_UNSUPPORTED, "tree needs more shared memory than one CTA can hold");
  const int ntiles = (N + tile - 1) / tile;
  const int code_stride = (N + tt::kCodeAlign - 1) / tt::kCodeAlign * tt::kCodeAlign;

  // carve the scratch
  size_t off = 0;
  const size_t o_status = off;
  off = align256(off + sizeof(int));
  const size_t o_table = off;
  off = align256(off + size_t(kTableRows) * S * sizeof(double));
  const size_t o_steps = off;
  off = align256(off + size_t(I) * tt::kStepInts * sizeof(int));
  const size_t o_bpos = off;
  off = align256(off + size_t(B) * sizeof(int));
  const size_t o_pmat = off;
  off = align256(off + size_t(batch) * I * 2 * kss * sizeof(double));
  const size_t o_tiles = off;
  off = align256(off + size_t(batch) * ntiles * sizeof(double));
  const size_t o_codes = off;  // tip codes with rows padded for 16-byte-aligned bulk copies
  off = align256(off + size_t(T) * code_stride);
  if (off > kScratchBytes) {
    char buf[240];
    snprintf(buf, sizeof buf,
             "problem needs %zu bytes of scratch, more than the %zu-byte static scratch of "
             "tt_log_likelihood_static (fewer tips, categories, samples or patterns, or use the plan API)",
             off, kScratchBytes);
    return fail(TT_ERR_INVALID_ARGUMENT, buf);
  }
  unsigned char *scratch = nullptr;
  rc = scratch_address(&scratch);
  if (rc != TT_OK) return rc;
  int *d_status = reinterpret_cast<int *>(scratch + o_status);
  double *d_table = reinterpret_cast<double *>(scratch + o_table);
  int *d_steps = reinterpret_cast<int *>(scratch + o_steps);
  int *d_bpos = reinterpret_cast<int *>(scratch + o_bpos);
  double *d_pmat = reinterpret_cast<double *>(scratch + o_pmat);
  double *d_tiles = reinterpret_cast<double *>(scratch + o_tiles);
  uint8_t *d_codes = scratch + o_codes;

  // Start-of-call state: status cleared; table rows past code_count and the
  // tile sums set to NaN, so an out-of-range code or a CTA that gave up on a
  // bounded wait shows up as a NaN log-likelihood instead of stale data.
  e = cudaMemsetAsync(d_status, 0, sizeof(int), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_table, 0xff, size_t(kTableRows) * S * sizeof(double), s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_table, code_table, size_t(code_count) * S * sizeof(double), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_tiles, 0xff, size_t(batch) * ntiles * sizeof(double), s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_steps, steps, size_t(I) * tt::kStepInts * sizeof(int), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_bpos, branch_pos, size_t(B) * sizeof(int), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_codes, 0, size_t(T) * code_stride, s);
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(d_codes, code_stride, codes, N, N, T, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = tt::launch_scatter_f64(matrices, d_bpos, d_pmat, B, kss, I, batch, s);
  if (e != cudaSuccess) return fail(TT_ERR_CUDA, cudaGetErrorString(e));

  tt::PruneArgs<double> a;
  std::memset(&a, 0, sizeof a);
  a.steps = reinterpret_cast<const int4 *>(d_steps);
  a.n_steps = I;
  a.tip_count = T;
  a.branch_count = B;
  a.N = N;
  a.K = K;
  a.C = kTableRows;
  a.slots = slots;
  a.rescale = rescale ? 1 : 0;
  a.ntiles = ntiles;
  a.code_stride = code_stride;
  a.nstage = tt::kStages;
  a.codes = d_codes;
  a.table = d_table;
  a.pmat = d_pmat;
  a.props = category_weights;
  a.freqs = frequencies;
  a.weights = weights;
  a.partials = nullptr;
  a.site_lnl = nullptr;
  a.tile_lnl = d_tiles;
  a.status = d_status;
  a.timeout_ns = 2000000000ull;
  e = tt::launch_prune_f64(a, false, tile, batch, s);
  if (e == cudaSuccess) e = tt::launch_reduce_lnl(d_tiles, log_likelihood, batch, ntiles, 0, s);
  if (e != cudaSuccess) return fail(TT_ERR_CUDA, cudaGetErrorString(e));
  // read the status word back (this synchronises the stream)
  int status = 0;
  e = cudaMemcpyAsync(&status, d_status, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail_cuda("reading the status word back failed", e);
  if (status != TT_OK)
    return fail(status == TT_ERR_DEVICE_TIMEOUT ? TT_ERR_DEVICE_TIMEOUT : TT_ERR_CUDA,
                "tt_log_likelihood_static: a bounded wait in the kernel gave up (status word set); the "
                "log-likelihoods are not valid");
  return TT_OK;
}
