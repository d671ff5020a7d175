// C ABI of the engine: plan construction (schedule + shared-memory slot
// assignment), device workspace and the entry points declared in
// include/torchtree_gb300.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "../../include/torchtree_gb300.h"
#include "tt_launch.h"
#include "tt_plan.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char *where) {
  return fail(e == cudaErrorMemoryAllocation ? TT_ERR_OUT_OF_MEMORY : TT_ERR_CUDA,
              std::string(where) + ": " + cudaGetErrorString(e));
}

constexpr unsigned long long kTimeoutNs = 2000000000ull;  // bounded device waits: 2 s

}  // namespace

namespace tt {
// Error reporting for entry points defined in other translation units.
int record_error(int code, const char *msg) { return fail(code, msg); }

cudaError_t kernel_smem(const void *func, size_t bytes, bool max_carveout) {
  static std::mutex mu;
  static std::map<std::pair<const void *, int>, size_t> done;  // largest size set per (kernel, device)
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  auto it = done.find({func, dev});
  if (it != done.end() && it->second >= bytes) return cudaSuccess;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
  if (e == cudaSuccess && max_carveout)
    e = cudaFuncSetAttribute(func, cudaFuncAttributePreferredSharedMemoryCarveout, int(cudaSharedmemCarveoutMaxShared));
  if (e == cudaSuccess) done[{func, dev}] = bytes;
  return e;
}
}  // namespace tt



namespace {

template <typename P>
int dev_alloc(tt_plan *p, P **ptr, size_t bytes, const char *what) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(ptr), bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(TT_ERR_OUT_OF_MEMORY,
                std::string("cudaMalloc of ") + what + " (" + std::to_string(bytes) + " bytes) failed: " +
                    cudaGetErrorString(e));
  }
  p->bytes += bytes;
  return TT_OK;
}

void release(tt_plan *p) {
  void *bufs[] = {p->d_steps, p->d_steps_rev, p->d_steps_ws, p->d_branch_pos, p->d_codes,    p->d_table,   p->d_weights,
                  p->d_pmat,  p->d_partials,   p->d_tile_lnl, p->d_gpart,   p->d_rootpart,
                  p->d_G,     p->d_rootgrad,   p->d_status, p->d_qpart};
  for (void *b : bufs)
    if (b) cudaFree(b);
  tt::wide_destroy(p);
}

// Build the execution order and the shared-memory slot plan.
// Post-order: at every node the child whose subtree needs more stack slots
// is evaluated first (Sethi-Ullman), so the forward stack depth is at most
// log2(T)+1.  The adjoint walks the same list backwards.
int build_schedule(tt_plan *p, const int32_t *post) {
  const int T = p->T, I = p->I, NN = 2 * T - 1;
  std::vector<int> left(NN, -1), right(NN, -1), parent(NN, -1);
  std::vector<char> done(NN, 0);
  for (int t = 0; t < T; ++t) done[t] = 1;
  for (int s = 0; s < I; ++s) {
    const int v = post[3 * s], l = post[3 * s + 1], r = post[3 * s + 2];
    char buf[160];
    if (v < T || v >= NN || l < 0 || l >= NN || r < 0 || r >= NN || l == r || l == v || r == v) {
      snprintf(buf, sizeof buf, "postorder triple %d = (%d, %d, %d) is out of range for %d tips", s, v,
               l, r, T);
      return fail(TT_ERR_INVALID_ARGUMENT, buf);
    }
    if (done[v]) {
      snprintf(buf, sizeof buf, "node %d appears twice as a parent", v);
      return fail(TT_ERR_INVALID_ARGUMENT, buf);
    }
    if (!done[l] || !done[r]) {
      snprintf(buf, sizeof buf, "triple %d uses child before it is computed (not a post-order)", s);
      return fail(TT_ERR_INVALID_ARGUMENT, buf);
    }
    if (parent[l] >= 0 || parent[r] >= 0) {
      snprintf(buf, sizeof buf, "triple %d reuses a child that already has a parent", s);
      return fail(TT_ERR_INVALID_ARGUMENT, buf);
    }
    left[v] = l;
    right[v] = r;
    parent[l] = v;
    parent[r] = v;
    done[v] = 1;
  }
  const int root = post[3 * (I - 1)];
  if (root != 2 * T - 2)
    return fail(TT_ERR_INVALID_ARGUMENT,
                "the last postorder triple must be the root with index 2T-2 (branch i is the branch "
                "above node i, so B = 2T-2)");
  for (int v = 0; v < NN; ++v)
    if (v != root && parent[v] < 0)
      return fail(TT_ERR_INVALID_ARGUMENT, "node " + std::to_string(v) + " is not connected to the root");

  // stack need per node and child order
  std::vector<int> need(NN, 0), first(NN, -1);
  for (int s = 0; s < I; ++s) {
    const int v = post[3 * s], l = left[v], r = right[v];
    const int f = need[l] >= need[r] ? l : r;
    const int g = f == l ? r : l;
    first[v] = f;
    need[v] = std::max({need[f], (f >= T ? 1 : 0) + need[g], 1});
  }
  std::vector<int> order;
  order.reserve(I);
  {
    std::vector<std::pair<int, int>> st;  // (node, visited children)
    st.push_back({root, 0});
    while (!st.empty()) {
      auto &top = st.back();
      const int v = top.first;
      if (v < T) {
        st.pop_back();
        continue;
      }
      if (top.second == 0) {
        top.second = 1;
        st.push_back({first[v], 0});
      } else if (top.second == 1) {
        top.second = 2;
        st.push_back({first[v] == left[v] ? right[v] : left[v], 0});
      } else {
        order.push_back(v);
        st.pop_back();
      }
    }
  }
  // forward slots
  p->steps.assign(size_t(I) * tt::kStepInts, -1);
  std::vector<int> fslot(NN, -1), bslot(NN, -1);
  std::set<int> free_slots;
  int next_slot = 0;
  auto alloc = [&]() {
    if (!free_slots.empty()) {
      int s = *free_slots.begin();
      free_slots.erase(free_slots.begin());
      return s;
    }
    return next_slot++;
  };
  for (int s = 0; s < I; ++s) {
    const int v = order[s], l = left[v], r = right[v];
    int *rec = &p->steps[size_t(s) * tt::kStepInts];
    rec[0] = v;
    rec[1] = l;
    rec[2] = r;
    rec[3] = l >= T ? fslot[l] : -1;
    rec[4] = r >= T ? fslot[r] : -1;
    if (rec[3] >= 0) free_slots.insert(rec[3]);
    if (rec[4] >= 0) free_slots.insert(rec[4]);
    rec[5] = v == root ? -1 : alloc();
    fslot[v] = rec[5];
  }
  p->slots_fwd = std::max(next_slot, 1);
  free_slots.clear();
  next_slot = 0;
  for (int s = I - 1; s >= 0; --s) {
    const int v = order[s], l = left[v], r = right[v];
    int *rec = &p->steps[size_t(s) * tt::kStepInts];
    rec[6] = v == root ? -1 : bslot[v];
    if (rec[6] >= 0) free_slots.insert(rec[6]);
    rec[7] = l >= T ? alloc() : -1;
    rec[8] = r >= T ? alloc() : -1;
    bslot[l] = rec[7];
    bslot[r] = rec[8];
  }
  p->slots_bwd = std::max(next_slot, 1);
  // In-place FP32 adjoint.  The reversed walk visits, right after a node with
  // an internal child, one of its children (the one that precedes it in the
  // post-order): that child's outside partial stays in registers.  The other
  // internal child's outside partial overwrites the child's own post-order
  // tile, read for the last time at this step, and is staged back at the
  // child's step, which must not be staged before this step has written it.
  std::vector<int> pos(NN, -1);
  for (int s = 0; s < I; ++s) pos[order[s]] = s;
  for (int s = 0; s < I; ++s) {
    const int v = order[s], l = left[v], r = right[v];
    int *rec = &p->steps[size_t(s) * tt::kStepInts];
    const int nxt = s > 0 ? order[s - 1] : -1;
    int flags = 0;
    if (l >= T) flags |= nxt == l ? tt::kTaCarryLeft : tt::kTaStoreLeft;
    if (r >= T) flags |= nxt == r ? tt::kTaCarryRight : tt::kTaStoreRight;
    rec[9] = flags;
    rec[10] = -1;
  }
  for (int s = 0; s < I; ++s) {
    const int v = order[s];
    if (v == root) continue;
    const int ps = pos[parent[v]];
    const int pf = p->steps[size_t(ps) * tt::kStepInts + 9];
    if (pf & (v == left[parent[v]] ? tt::kTaStoreLeft : tt::kTaStoreRight)) {
      p->steps[size_t(s) * tt::kStepInts + 9] |= tt::kTaPreStored;
      p->steps[size_t(s) * tt::kStepInts + 10] = I - 1 - ps;
    }
  }
  // producer-warp post-order: a node whose next step is its parent hands its
  // partial over in registers and takes no stack slot
  p->steps_ws.assign(size_t(I) * tt::kStepInts, -1);
  {
    std::vector<int> wslot(NN, -1);
    free_slots.clear();
    next_slot = 0;
    for (int s = 0; s < I; ++s) {
      const int v = order[s], l = left[v], r = right[v];
      int *rec = &p->steps_ws[size_t(s) * tt::kStepInts];
      rec[0] = v;
      rec[1] = l;
      rec[2] = r;
      const int kid[2] = {l, r};
      for (int c = 0; c < 2; ++c) {
        const int k = kid[c];
        if (k < T) continue;
        const bool carried = s > 0 && order[s - 1] == k;
        rec[3 + c] = carried ? tt::kWsCarry : wslot[k];
        if (!carried) free_slots.insert(wslot[k]);
      }
      const bool carry_out = s + 1 < I && parent[v] == order[s + 1];
      rec[5] = v == root ? -1 : (carry_out ? tt::kWsCarry : alloc());
      wslot[v] = rec[5];
    }
    p->slots_ws = std::max(next_slot, 1);
  }
  p->branch_pos.assign(p->B, -1);
  for (int s = 0; s < I; ++s) {
    const int *rec = &p->steps[size_t(s) * tt::kStepInts];
    p->branch_pos[rec[1]] = 2 * s;
    p->branch_pos[rec[2]] = 2 * s + 1;
  }
  return TT_OK;
}

int check_device(const tt_plan *p) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev != p->device)
    return fail(TT_ERR_INVALID_ARGUMENT, "the current CUDA device differs from the plan's device");
  return TT_OK;
}

template <typename T>
tt::PruneArgs<T> make_args(tt_plan *p, const double *props, const double *freqs, int rescale,
                           bool keep, double *site_lnl) {
  tt::PruneArgs<T> a;
  a.steps = p->d_steps;
  a.n_steps = p->I;
  a.tip_count = p->T;
  a.branch_count = p->B;
  a.N = p->N;
  a.K = p->K;
  a.C = p->C;
  a.rescale = rescale;
  a.ntiles = p->ntiles_f;
  a.code_stride = p->code_stride;
  a.nstage = p->nstage_f;
  a.steps_rev = p->d_steps_rev;
  a.steps_ws = p->d_steps_ws;
  a.codes = p->d_codes;
  a.table = static_cast<const T *>(p->d_table);
  a.pmat = static_cast<const T *>(p->d_pmat);
  a.props = props;
  a.freqs = freqs;
  a.weights = p->d_weights;
  a.partials = keep ? static_cast<T *>(p->d_partials) : nullptr;
  a.site_lnl = site_lnl;
  a.tile_lnl = p->d_tile_lnl;
  a.gpart = static_cast<T *>(p->d_gpart);
  a.rootpart = static_cast<T *>(p->d_rootpart);
  a.status = p->d_status;
  a.timeout_ns = kTimeoutNs;
  a.slots = 0;
  return a;
}

// ------------------------------------------------------------ pattern slabs
// Patterns are independent, so the post-order and adjoint of one slab of
// patterns equal the corresponding tiles of a whole-alignment pass.  A slab
// starts at a multiple of kSlabAlign patterns: a whole number of 64- and
// 32-pattern tiles, of the tile-sum blocks of 8 tiles, and of 128-byte code
// runs (so every code copy stays inside the padded tip row).
constexpr int kSlabAlign = 512;

int slab_round(long long patterns, int N) {
  if (patterns <= 0) return 0;
  const long long r = (patterns + kSlabAlign - 1) / kSlabAlign * kSlabAlign;
  return r >= N ? 0 : int(r);
}

// Bytes of the gradient buffers (stored partials, per-tile gradient blocks,
// per-tile root blocks) for `npat` patterns, with dev_alloc's 16-byte floor.
struct GradBytes {
  size_t partials, gpart, rootpart;
  size_t total() const { return std::max(partials, size_t(16)) + std::max(gpart, size_t(16)) + std::max(rootpart, size_t(16)); }
};

GradBytes grad_bytes(const tt_plan *p, int npat) {
  const bool f32 = p->precision == TT_PRECISION_F32;
  const size_t kss = size_t(p->K) * p->S * p->S;
  const size_t I1 = size_t(std::max(p->I - 1, 1));
  // FP32 plans: category pairs (K padded to even), partials per tile (N padded to whole tiles)
  const size_t kpad = f32 ? size_t(2 * tt::kpairs_for(p->K)) : size_t(p->K);
  const size_t ntb = (size_t(npat) + p->tile_b - 1) / p->tile_b;
  const size_t npad = f32 ? ntb * p->tile_b : size_t(npat);
  GradBytes g;
  g.partials = size_t(p->batch) * I1 * kpad * npad * p->S * p->elem;
  g.gpart = size_t(p->batch) * p->B * ntb * kss * p->elem;
  g.rootpart = size_t(p->batch) * ntb * (p->S + p->K) * p->elem;
  return g;
}

void free_grad_buffers(tt_plan *p) {
  for (void **b : {&p->d_partials, &p->d_gpart, &p->d_rootpart})
    if (*b) {
      cudaFree(*b);
      *b = nullptr;
    }
  p->bytes -= std::min(p->bytes, p->grad_bytes);
  p->grad_bytes = 0;
}

// (Re)allocate the gradient buffers for slabs of `slab` patterns (0 = all).
// On failure the plan keeps no gradient buffers: tt_log_likelihood without
// keep_partials still works, and a smaller slab may be set.
int alloc_grad_buffers(tt_plan *p, int slab) {
  free_grad_buffers(p);
  p->partials_valid = false;
  p->grads_valid = false;
  const GradBytes g = grad_bytes(p, slab ? slab : p->N);
  const size_t before = p->bytes;
  int rc = dev_alloc(p, &p->d_partials, g.partials, "partials");
  if (!rc) rc = dev_alloc(p, &p->d_gpart, g.gpart, "gradient tiles");
  if (!rc) rc = dev_alloc(p, &p->d_rootpart, g.rootpart, "root tiles");
  p->grad_bytes = p->bytes - before;
  if (rc) {
    const std::string msg = g_last_error;
    free_grad_buffers(p);
    return fail(rc, msg + " (a smaller TT_OPT_SLAB_PATTERNS holds fewer patterns' partials at once)");
  }
  p->slab = slab;
  return TT_OK;
}

// Slab size of a new plan whose pattern-sized buffers take `full` bytes for
// the whole alignment: none when they fit in 7/8 of the free device memory
// (or TT_GRADIENT_BUDGET_BYTES), else slabs sized to that budget.
// TT_SLAB_PATTERNS sets the slab explicitly.
int choose_slab(const tt_plan *p, size_t full) {
  if (const char *env = getenv("TT_SLAB_PATTERNS")) return slab_round(atoll(env), p->N);
  size_t free_b = 0, total_b = 0;
  size_t budget = SIZE_MAX;  // no slabs when the free memory cannot be read
  if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess)
    budget = free_b - free_b / 8;
  else
    cudaGetLastError();
  if (const char *env = getenv("TT_GRADIENT_BUDGET_BYTES")) budget = std::min(budget, size_t(atoll(env)));
  if (full <= budget) return 0;
  const double per_pattern = double(full) / p->N;
  const long long fit = (long long)(double(budget) / per_pattern) / kSlabAlign * kSlabAlign;
  return slab_round(std::max<long long>(kSlabAlign, fit), p->N);
}

// Restrict pruning arguments to patterns [p0, p0 + n) with `tile`-pattern tiles.
template <typename T>
void slab_args(tt::PruneArgs<T> &a, int p0, int n, int tile) {
  a.codes += p0;
  a.weights += p0;
  a.N = n;
  a.ntiles = (n + tile - 1) / tile;
  a.site_lnl = nullptr;
}

// Post-order pass over patterns [p0, p0 + n) in the plan's kernel shape;
// store = keep the partials of that range (for the adjoint).
template <typename T>
cudaError_t post_order(tt_plan *p, const double *props, const double *freqs, int rescale, bool store,
                       double *site_lnl, int p0, int n, cudaStream_t s) {
  auto a = make_args<T>(p, props, freqs, rescale, store, site_lnl);
  if (p0 != 0 || n != p->N) slab_args(a, p0, n, p->tile_f);
  if constexpr (sizeof(T) == 4) {
    a.slots = p->producer_warp && !p->pair_threads ? p->slots_ws : p->slots_fwd;
    return tt::launch_prune_f32(a, false, p->tile_f, plan_run_samples(p),
                                (p->pair_threads ? tt::kF32PairThreads : 0) | (p->producer_warp ? tt::kF32ProducerWarp : 0), s);
  } else {
    a.slots = p->slots_fwd;
    return tt::launch_prune_f64(a, false, p->tile_f, plan_run_samples(p), s);
  }
}

}  // namespace

extern "C" {

const char *tt_version(void) { return "torchtree_gb300 0.1.0 (sm_103a)"; }

const char *tt_last_error(void) { return g_last_error.c_str(); }

int tt_plan_create(tt_plan **plan, int32_t tip_count, const int32_t *postorder,
                   int32_t state_count, int32_t category_count, int32_t pattern_count,
                   int32_t batch, int32_t precision) {
  if (!plan || !postorder) return fail(TT_ERR_INVALID_ARGUMENT, "plan and postorder must not be NULL");
  *plan = nullptr;
  if (tip_count < 2) return fail(TT_ERR_INVALID_ARGUMENT, "a tree needs at least 2 tips");
  if (state_count < 2 || state_count > 64)
    return fail(TT_ERR_UNSUPPORTED, "state_count must be in [2, 64]");
  if (category_count < 1 || category_count > 8)
    return fail(TT_ERR_INVALID_ARGUMENT, "category_count must be in [1, 8]");
  if (pattern_count < 1) return fail(TT_ERR_INVALID_ARGUMENT, "pattern_count must be >= 1");
  if (batch < 1 || batch > 65535) return fail(TT_ERR_INVALID_ARGUMENT, "batch must be in [1, 65535]");
  if (precision != TT_PRECISION_F32 && precision != TT_PRECISION_F64)
    return fail(TT_ERR_INVALID_ARGUMENT, "precision must be TT_PRECISION_F32 or TT_PRECISION_F64");

  tt_plan *p = new tt_plan();
  cudaError_t ce = cudaGetDevice(&p->device);
  if (ce != cudaSuccess) {
    delete p;
    return cuda_fail(ce, "cudaGetDevice");
  }
  p->T = tip_count;
  p->I = tip_count - 1;
  p->B = 2 * tip_count - 2;
  p->S = state_count;
  p->K = category_count;
  p->N = pattern_count;
  p->batch = batch;
  p->precision = precision;
  p->elem = precision == TT_PRECISION_F32 ? 4 : 8;
  int rc = build_schedule(p, postorder);
  if (rc != TT_OK) {
    delete p;
    return rc;
  }
  if (p->S != 4) {  // amino-acid / codon / general models: level-scheduled wide-state kernels
    rc = tt::wide_create(p);
    if (rc == TT_OK) rc = tt::wide_alloc_slab(p, choose_slab(p, tt::wide_pattern_bytes(p, p->N)));
    if (rc != TT_OK) {
      release(p);
      delete p;
      return rc;
    }
    *plan = p;
    return TT_OK;
  }
  int smem_max = 0;
  cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->device);
  const bool f32 = precision == TT_PRECISION_F32;
  const int *ftiles = f32 ? tt::kFwdTilesF32 : tt::kFwdTilesF64;
  const int *btiles = f32 ? tt::kBwdTilesF32 : tt::kBwdTilesF64;
  if (f32) {  // ring depths of the FP32 kernels; TT_FWD_STAGES / TT_BWD_STAGES override
    p->nstage_f = getenv("TT_FWD_STAGES") ? std::max(2, atoi(getenv("TT_FWD_STAGES"))) : tt::kTlFwdStages;
    p->nstage_b = getenv("TT_BWD_STAGES") ? std::max(2, atoi(getenv("TT_BWD_STAGES"))) : tt::kTlBwdStages;
  }
  auto smem_of = [&](int tile, bool bwd) {
    const int slots = bwd ? p->slots_bwd : p->slots_fwd;
    const int ns = bwd ? p->nstage_b : p->nstage_f;
    return f32 ? std::max({tt::tl_smem_bytes(p->K, 256, slots, bwd, ns), tt::tq_smem_bytes(p->K, 256, slots, bwd, ns),
                           bwd ? size_t(0) : tt::tl_ws_smem_bytes(p->K, 256, p->slots_ws, ns),
                           bwd ? std::max(tt::ta_smem_bytes(p->K, 256, ns), tt::tp_smem_bytes(p->K, 256, ns))
                               : size_t(0)})
               : tt::prune_smem_bytes<double>(4, p->K, 256, slots, tile, bwd);
  };
  // optional overrides for tuning sweeps: TT_FWD_TILE / TT_BWD_TILE.  FP32 rings
  // shrink (down to 3 stages) before a smaller tile is tried.
  auto fits = [&](int tile, bool bwd) {
    int &ns = bwd ? p->nstage_b : p->nstage_f;
    const int want = ns;
    for (; ns >= (f32 ? std::min(3, want) : want); --ns)
      if (smem_of(tile, bwd) <= size_t(smem_max)) return true;
    ns = want;
    return false;
  };
  auto pick = [&](const int *cand, bool bwd, const char *env) {
    const char *o = getenv(env);
    if (o) {
      const int want = atoi(o);
      for (int i = 0; i < 2; ++i)
        if (cand[i] == want && fits(want, bwd)) return want;
    }
    for (int i = 0; i < 2; ++i)
      if (fits(cand[i], bwd)) return cand[i];
    return 0;
  };
  p->tile_f = pick(ftiles, false, "TT_FWD_TILE");
  p->tile_b = pick(btiles, true, "TT_BWD_TILE");
  if (!p->tile_f || !p->tile_b) {
    delete p;
    return fail(TT_ERR_UNSUPPORTED, "tree needs " + std::to_string(std::max(p->slots_fwd, p->slots_bwd)) +
                                        " shared-memory slots, more than one CTA can hold");
  }
  {
    const char *env = getenv("TT_PRODUCER_WARP");
    p->producer_warp = f32 && !(env && atoi(env) == 0);
  }
  {
    const char *env = getenv("TT_INPLACE_ADJOINT");
    p->inplace_adjoint = f32 && !(env && atoi(env) == 0);
  }
  if (f32 && tt::pair_adjoint_supported(p->K)) {
    const char *env = getenv("TT_PAIR_ADJOINT");
    p->pair_adjoint = env && atoi(env) == 1;
  }
  if (f32 && tt::pair_threads_supported(p->K)) {  // measured slower on GB300: off unless TT_PAIR_THREADS=1
    const char *env = getenv("TT_PAIR_THREADS");
    p->pair_threads = env && atoi(env) == 1;
  }
  p->ntiles_f = (p->N + p->tile_f - 1) / p->tile_f;
  p->ntiles_b = (p->N + p->tile_b - 1) / p->tile_b;
  p->code_stride = (p->N + tt::kCodeAlign - 1) / tt::kCodeAlign * tt::kCodeAlign;

  const size_t kss = size_t(p->K) * p->S * p->S;
  rc = TT_OK;
  if (!rc) rc = dev_alloc(p, &p->d_steps, p->steps.size() * sizeof(int), "schedule");
  if (!rc) rc = dev_alloc(p, &p->d_steps_rev, p->steps.size() * sizeof(int), "reversed schedule");
  if (!rc) rc = dev_alloc(p, &p->d_steps_ws, p->steps_ws.size() * sizeof(int), "post-order schedule");
  if (!rc) rc = dev_alloc(p, &p->d_branch_pos, size_t(p->B) * sizeof(int), "branch map");
  if (!rc) rc = dev_alloc(p, &p->d_codes, size_t(p->T) * p->code_stride, "tip codes");
  if (!rc) rc = dev_alloc(p, &p->d_table, size_t(256) * p->S * p->elem, "code table");
  if (!rc) rc = dev_alloc(p, &p->d_weights, size_t(p->N) * sizeof(double), "weights");
  // FP32 plans: category pairs (K padded to even)
  const size_t kpad = f32 ? size_t(2 * tt::kpairs_for(p->K)) : size_t(p->K);
  if (!rc) rc = dev_alloc(p, &p->d_pmat, size_t(batch) * p->I * 2 * kpad * p->S * p->S * p->elem, "transition matrices");
  if (!rc) rc = dev_alloc(p, &p->d_tile_lnl, size_t(batch) * p->ntiles_f * sizeof(double), "tile sums");
  if (!rc) rc = dev_alloc(p, &p->d_G, size_t(batch) * p->B * kss * sizeof(double), "dlnL/dP");
  if (!rc) rc = dev_alloc(p, &p->d_rootgrad, size_t(batch) * (p->S + p->K) * sizeof(double), "root grads");
  if (!rc) rc = dev_alloc(p, &p->d_status, sizeof(int), "status");
  if (!rc) {
    rc = alloc_grad_buffers(p, choose_slab(p, grad_bytes(p, p->N).total()));
  }
  if (rc) {
    release(p);
    delete p;
    return rc;
  }
  ce = cudaMemcpy(p->d_steps, p->steps.data(), p->steps.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) {
    std::vector<int> rev(p->steps.size());
    for (int s2 = 0; s2 < p->I; ++s2)
      std::memcpy(&rev[size_t(s2) * tt::kStepInts], &p->steps[size_t(p->I - 1 - s2) * tt::kStepInts],
                  tt::kStepInts * sizeof(int));
    ce = cudaMemcpy(p->d_steps_rev, rev.data(), rev.size() * sizeof(int), cudaMemcpyHostToDevice);
  }
  if (ce == cudaSuccess)
    ce = cudaMemcpy(p->d_steps_ws, p->steps_ws.data(), p->steps_ws.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess)
    ce = cudaMemcpy(p->d_branch_pos, p->branch_pos.data(), p->branch_pos.size() * sizeof(int),
                    cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMemset(p->d_status, 0, sizeof(int));
  if (ce == cudaSuccess)  // padded category pairs must read as zero matrices
    ce = cudaMemset(p->d_pmat, 0, size_t(batch) * p->I * 2 * kpad * p->S * p->S * p->elem);
  if (ce != cudaSuccess) {
    release(p);
    delete p;
    return cuda_fail(ce, "plan upload");
  }
  *plan = p;
  return TT_OK;
}

int tt_plan_destroy(tt_plan *plan) {
  if (!plan) return TT_OK;
  release(plan);
  delete plan;
  return TT_OK;
}

int tt_plan_workspace_bytes(const tt_plan *plan, size_t *bytes) {
  if (!plan || !bytes) return fail(TT_ERR_INVALID_ARGUMENT, "NULL argument");
  *bytes = plan->bytes;
  return TT_OK;
}

int tt_plan_set_tips(tt_plan *p, const uint8_t *codes, const double *code_table, int32_t code_count,
                     const double *weights) {
  if (!p || !codes || !code_table || !weights) return fail(TT_ERR_INVALID_ARGUMENT, "NULL argument");
  if (code_count < 1 || code_count > 256)
    return fail(TT_ERR_INVALID_ARGUMENT, "code_count must be in [1, 256]");
  int rc = check_device(p);
  if (rc) return rc;
  const size_t tn = size_t(p->T) * p->N;
  for (size_t i = 0; i < tn; ++i)
    if (codes[i] >= code_count)
      return fail(TT_ERR_INVALID_ARGUMENT, "tip code " + std::to_string(codes[i]) + " at position " +
                                               std::to_string(i) + " is >= code_count");
  for (int n = 0; n < p->N; ++n)
    if (!(weights[n] >= 0.0)) return fail(TT_ERR_INVALID_ARGUMENT, "pattern weights must be >= 0");
  if (p->wide) {
    rc = tt::wide_set_tips(p, codes, code_table, code_count, weights);
    if (rc) return rc;
    p->C = code_count;
    p->tips_set = true;
    p->partials_valid = false;
    return TT_OK;
  }
  std::vector<unsigned char> table(size_t(code_count) * p->S * p->elem);
  for (size_t i = 0; i < size_t(code_count) * p->S; ++i) {
    if (p->precision == TT_PRECISION_F32) {
      float f = float(code_table[i]);
      std::memcpy(&table[i * 4], &f, 4);
    } else {
      std::memcpy(&table[i * 8], &code_table[i], 8);
    }
  }
  cudaError_t e = cudaMemset(p->d_codes, 0, size_t(p->T) * p->code_stride);
  if (e == cudaSuccess)
    e = cudaMemcpy2D(p->d_codes, p->code_stride, codes, p->N, p->N, p->T, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(p->d_table, table.data(), table.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(p->d_weights, weights, size_t(p->N) * sizeof(double), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "tt_plan_set_tips upload");
  p->C = code_count;
  p->tips_set = true;
  p->partials_valid = false;
  return TT_OK;
}

int tt_update_transition_matrices(tt_plan *p, const double *lam, const double *U, const double *W,
                                  const double *bl, const double *rates, void *stream) {
  if (!p || !lam || !U || !W || !bl || !rates) return fail(TT_ERR_INVALID_ARGUMENT, "NULL argument");
  int rc = check_device(p);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (p->wide) {
    rc = tt::wide_update_matrices(p, lam, U, W, bl, rates, s);
    if (rc) return rc;
    p->pmat_set = true;
    p->partials_valid = false;
    return TT_OK;
  }
  cudaError_t e =
      p->precision == TT_PRECISION_F32
          ? tt::launch_pmatrix_f32(lam, U, W, bl, rates, p->d_branch_pos, static_cast<float *>(p->d_pmat),
                                   p->S, p->B, p->K, p->I, p->batch, s)
          : tt::launch_pmatrix_f64(lam, U, W, bl, rates, p->d_branch_pos, static_cast<double *>(p->d_pmat),
                                   p->S, p->B, p->K, p->I, p->batch, s);
  if (e != cudaSuccess) return cuda_fail(e, "transition-matrix launch");
  p->launches += 1;
  p->pmat_set = true;
  p->partials_valid = false;
  return TT_OK;
}

int tt_set_transition_matrices(tt_plan *p, const double *matrices, void *stream) {
  if (!p || !matrices) return fail(TT_ERR_INVALID_ARGUMENT, "NULL argument");
  int rc = check_device(p);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (p->wide) {
    rc = tt::wide_set_matrices(p, matrices, s);
    if (rc) return rc;
    p->pmat_set = true;
    p->partials_valid = false;
    return TT_OK;
  }
  const int kss = p->K * p->S * p->S;
  cudaError_t e = p->precision == TT_PRECISION_F32
                      ? tt::launch_scatter_f32(matrices, p->d_branch_pos, static_cast<float *>(p->d_pmat),
                                               p->B, kss, p->I, p->batch, s)
                      : tt::launch_scatter_f64(matrices, p->d_branch_pos, static_cast<double *>(p->d_pmat),
                                               p->B, kss, p->I, p->batch, s);
  if (e != cudaSuccess) return cuda_fail(e, "transition-matrix scatter launch");
  p->launches += 1;
  p->pmat_set = true;
  p->partials_valid = false;
  return TT_OK;
}

int tt_log_likelihood(tt_plan *p, const double *props, const double *freqs, int32_t rescale,
                      int32_t keep_partials, double *lnl, double *site_lnl, void *stream) {
  if (!p || !props || !freqs || !lnl) return fail(TT_ERR_INVALID_ARGUMENT, "NULL argument");
  if (!p->tips_set) return fail(TT_ERR_NOT_READY, "tt_plan_set_tips has not been called");
  if (!p->pmat_set) return fail(TT_ERR_NOT_READY, "transition matrices have not been set");
  int rc = check_device(p);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (p->wide) {
    if (!tt::wide_has_buffers(p))
      return fail(TT_ERR_OUT_OF_MEMORY, "the plan holds no partial buffers: set TT_OPT_SLAB_PATTERNS to a size that fits");
    rc = tt::wide_log_likelihood(p, props, freqs, rescale ? 1 : 0, keep_partials != 0, lnl, site_lnl, s);
    if (rc) return rc;
    p->last_rescale = rescale ? 1 : 0;
    p->partials_valid = keep_partials != 0;
    return TT_OK;
  }
  if (keep_partials && !p->d_partials)
    return fail(TT_ERR_OUT_OF_MEMORY, "the plan holds no gradient buffers: set TT_OPT_SLAB_PATTERNS to a size that fits");
  // in slab mode the partials are recomputed by tt_gradient, slab by slab
  const bool store = keep_partials != 0 && !p->slab;
  cudaError_t e = p->precision == TT_PRECISION_F32 ? post_order<float>(p, props, freqs, rescale ? 1 : 0, store, site_lnl, 0, p->N, s)
                                                   : post_order<double>(p, props, freqs, rescale ? 1 : 0, store, site_lnl, 0, p->N, s);
  if (e != cudaSuccess) return cuda_fail(e, "post-order launch");
  e = tt::launch_reduce_lnl(p->d_tile_lnl, lnl, plan_run_samples(p), p->ntiles_f, 0, s);
  if (e != cudaSuccess) return cuda_fail(e, "likelihood reduction launch");
  p->launches += 2;
  p->last_rescale = rescale ? 1 : 0;
  p->partials_valid = keep_partials != 0;
  return TT_OK;
}

}  // extern "C"

namespace {

// Whether plan p runs the default FP32 4-state kernels that a multi-plan
// launch can merge: producer-warp post-order and in-place adjoint, one
// pattern per thread in the post-order, the whole alignment resident.
bool mergeable(const tt_plan *p) {
  return p->precision == TT_PRECISION_F32 && !p->wide && p->S == 4 && !p->slab && p->producer_warp &&
         !p->pair_threads && p->inplace_adjoint && p->nstage_f <= 8;
}

int check_multi(int32_t count, tt_plan *const *plans, const double *const *props, const double *const *freqs) {
  if (count < 1 || !plans || !props || !freqs) return fail(TT_ERR_INVALID_ARGUMENT, "NULL argument or empty plan list");
  for (int i = 0; i < count; ++i) {
    if (!plans[i] || !props[i] || !freqs[i]) return fail(TT_ERR_INVALID_ARGUMENT, "NULL plan or argument");
    for (int j = 0; j < i; ++j)
      if (plans[j] == plans[i]) return fail(TT_ERR_INVALID_ARGUMENT, "a plan appears twice in one call");
    const int rc = check_device(plans[i]);
    if (rc) return rc;
  }
  return TT_OK;
}

// Groups of up to kMaxMultiPlans mergeable plans with one category-pair count
// (and, for the adjoint, one adjoint kernel) among the plans `todo`.
std::vector<std::vector<int>> merge_groups(const std::vector<int> &todo, tt_plan *const *plans, bool adjoint) {
  std::vector<std::vector<int>> groups;
  for (int i : todo) {
    const tt_plan *p = plans[i];
    bool placed = false;
    for (auto &g : groups) {
      const tt_plan *q = plans[g[0]];
      if (int(g.size()) < tt::kMaxMultiPlans && tt::kpairs_for(q->K) == tt::kpairs_for(p->K) &&
          (!adjoint || q->pair_adjoint == p->pair_adjoint)) {
        g.push_back(i);
        placed = true;
        break;
      }
    }
    if (!placed) groups.push_back({i});
  }
  return groups;
}

}  // namespace

extern "C" {

int tt_plans_log_likelihood(int32_t count, tt_plan *const *plans, const double *const *category_weights,
                            const double *const *frequencies, int32_t rescale, int32_t keep_partials,
                            double *const *log_likelihood, void *stream) {
  int rc = check_multi(count, plans, category_weights, frequencies);
  if (rc) return rc;
  if (!log_likelihood) return fail(TT_ERR_INVALID_ARGUMENT, "NULL argument");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::vector<int> merge;
  for (int i = 0; i < count; ++i) {
    tt_plan *p = plans[i];
    if (!log_likelihood[i]) return fail(TT_ERR_INVALID_ARGUMENT, "NULL log_likelihood");
    if (!p->tips_set) return fail(TT_ERR_NOT_READY, "tt_plan_set_tips has not been called");
    if (!p->pmat_set) return fail(TT_ERR_NOT_READY, "transition matrices have not been set");
    if (mergeable(p) && (!keep_partials || p->d_partials)) {
      merge.push_back(i);
    } else {  // other kernel shapes: the plan's own call
      rc = tt_log_likelihood(p, category_weights[i], frequencies[i], rescale, keep_partials, log_likelihood[i],
                             nullptr, stream);
      if (rc) return rc;
    }
  }
  constexpr int TPC = tt::kTlWsPatterns / tt::kTlTile;  // stored tiles per post-order CTA
  for (const auto &g : merge_groups(merge, plans, false)) {
    tt::MultiPrune<float> m;
    std::memset(&m, 0, sizeof m);
    m.count = int(g.size());
    size_t smem = 0;
    long long total = 0;
    for (int k = 0; k < m.count; ++k) {
      tt_plan *p = plans[g[k]];
      auto a = make_args<float>(p, category_weights[g[k]], frequencies[g[k]], rescale ? 1 : 0, keep_partials != 0,
                                nullptr);
      a.slots = p->slots_ws;
      m.a[k] = a;
      m.first[k] = int(total);
      m.per_sample[k] = (p->ntiles_f + TPC - 1) / TPC;
      total += (long long)m.per_sample[k] * plan_run_samples(p);
      smem = std::max(smem, tt::tl_ws_smem_bytes(p->K, p->C, p->slots_ws, p->nstage_f));
    }
    if (total > 0x7fffffffll) return fail(TT_ERR_UNSUPPORTED, "too many CTAs for one merged launch");
    m.first[m.count] = int(total);
    cudaError_t e = tt::launch_forward_multi(m, int(total), smem, s);
    if (e != cudaSuccess) return cuda_fail(e, "merged post-order launch");
    for (int k = 0; k < m.count; ++k) {
      tt_plan *p = plans[g[k]];
      e = tt::launch_reduce_lnl(p->d_tile_lnl, log_likelihood[g[k]], plan_run_samples(p), p->ntiles_f, 0, s);
      if (e != cudaSuccess) return cuda_fail(e, "likelihood reduction launch");
      p->launches += 1;
      p->last_rescale = rescale ? 1 : 0;
      p->partials_valid = keep_partials != 0;
    }
    plans[g[0]]->launches += 1;  // the merged post-order, counted once
  }
  return TT_OK;
}

int tt_plans_gradient(int32_t count, tt_plan *const *plans, const double *const *category_weights,
                      const double *const *frequencies, double *const *grad_frequencies,
                      double *const *grad_weights, void *stream) {
  int rc = check_multi(count, plans, category_weights, frequencies);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::vector<int> merge;
  for (int i = 0; i < count; ++i) {
    tt_plan *p = plans[i];
    double *gf = grad_frequencies ? grad_frequencies[i] : nullptr;
    double *gw = grad_weights ? grad_weights[i] : nullptr;
    if (!p->partials_valid)
      return fail(TT_ERR_NOT_READY,
                  "tt_plans_gradient needs a preceding log-likelihood with keep_partials=1 for the same matrices");
    if (mergeable(p) && p->d_partials && p->d_gpart && p->d_rootpart) {
      merge.push_back(i);
    } else {
      rc = tt_gradient(p, category_weights[i], frequencies[i], nullptr, gf, gw, stream);
      if (rc) return rc;
    }
  }
  for (const auto &g : merge_groups(merge, plans, true)) {
    tt::MultiPrune<float> m;
    std::memset(&m, 0, sizeof m);
    m.count = int(g.size());
    size_t smem = 0;
    long long total = 0;
    const bool pair = plans[g[0]]->pair_adjoint && tt::pair_adjoint_supported(plans[g[0]]->K);
    for (int k = 0; k < m.count; ++k) {
      tt_plan *p = plans[g[k]];
      auto a = make_args<float>(p, category_weights[g[k]], frequencies[g[k]], 1, true, nullptr);
      a.slots = p->slots_bwd;
      a.nstage = p->nstage_b;
      a.ntiles = (p->N + p->tile_b - 1) / p->tile_b;
      a.site_lnl = nullptr;
      m.a[k] = a;
      m.first[k] = int(total);
      m.per_sample[k] = a.ntiles;
      total += (long long)a.ntiles * plan_run_samples(p);
      smem = std::max(smem, pair ? tt::tp_smem_bytes(p->K, p->C, p->nstage_b) : tt::ta_smem_bytes(p->K, p->C, p->nstage_b));
    }
    if (total > 0x7fffffffll) return fail(TT_ERR_UNSUPPORTED, "too many CTAs for one merged launch");
    m.first[m.count] = int(total);
    cudaError_t e = tt::launch_adjoint_multi(m, int(total), smem, pair, s);
    if (e != cudaSuccess) return cuda_fail(e, "merged adjoint launch");
    plans[g[0]]->launches += 1;
    for (int k = 0; k < m.count; ++k) {
      const int i = g[k];
      tt_plan *p = plans[i];
      const int ntiles = m.per_sample[k];
      e = tt::launch_reduce_f32(static_cast<const float *>(p->d_gpart), static_cast<const float *>(p->d_rootpart),
                                p->d_G, p->d_rootgrad, p->d_rootgrad + size_t(p->batch) * p->S, plan_run_samples(p), p->B, ntiles,
                                p->S, p->K, 0, s);
      if (e == cudaSuccess && grad_frequencies && grad_frequencies[i])
        e = cudaMemcpyAsync(grad_frequencies[i], p->d_rootgrad, size_t(p->batch) * p->S * sizeof(double),
                            cudaMemcpyDeviceToDevice, s);
      if (e == cudaSuccess && grad_weights && grad_weights[i])
        e = cudaMemcpyAsync(grad_weights[i], p->d_rootgrad + size_t(p->batch) * p->S,
                            size_t(p->batch) * p->K * sizeof(double), cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return cuda_fail(e, "merged adjoint reductions");
      p->launches += 2;
      p->partials_valid = false;  // the outside partials overwrote the post-order tiles
      p->grads_valid = true;
    }
  }
  return TT_OK;
}

int tt_gradient(tt_plan *p, const double *props, const double *freqs, double *grad_matrices,
                double *grad_frequencies, double *grad_weights, void *stream) {
  if (!p || !props || !freqs) return fail(TT_ERR_INVALID_ARGUMENT, "NULL argument");
  if (!p->partials_valid)
    return fail(TT_ERR_NOT_READY,
                "tt_gradient needs a preceding tt_log_likelihood with keep_partials=1 for the same matrices");
  int rc = check_device(p);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (p->wide) {  // the wide-state adjoint overwrites the stored partials (slab mode recomputes them)
    if (!tt::wide_has_buffers(p))
      return fail(TT_ERR_OUT_OF_MEMORY, "the plan holds no partial buffers: set TT_OPT_SLAB_PATTERNS to a size that fits");
    rc = tt::wide_gradient(p, props, freqs, grad_matrices, grad_frequencies, grad_weights, s);
    if (rc) return rc;
    p->partials_valid = p->slab != 0;
    p->grads_valid = true;
    return TT_OK;
  }
  if (!p->d_partials || !p->d_gpart || !p->d_rootpart)
    return fail(TT_ERR_OUT_OF_MEMORY, "the plan holds no gradient buffers: set TT_OPT_SLAB_PATTERNS to a size that fits");
  // one pass over all patterns, or per slab: post-order (storing) + adjoint +
  // tile sums added to the previous slabs'
  const int span = p->slab ? p->slab : p->N;
  cudaError_t e = cudaSuccess;
  for (int p0 = 0; p0 < p->N && e == cudaSuccess; p0 += span) {
    const int n = std::min(span, p->N - p0);
    if (p->slab) {
      e = p->precision == TT_PRECISION_F32 ? post_order<float>(p, props, freqs, p->last_rescale, true, nullptr, p0, n, s)
                                           : post_order<double>(p, props, freqs, p->last_rescale, true, nullptr, p0, n, s);
      p->launches += 1;
      if (e != cudaSuccess) break;
    }
    const int ntiles = (n + p->tile_b - 1) / p->tile_b;
    if (p->precision == TT_PRECISION_F32) {
      auto a = make_args<float>(p, props, freqs, 1, true, nullptr);
      a.slots = p->slots_bwd;
      a.nstage = p->nstage_b;
      slab_args(a, p0, n, p->tile_b);
      e = tt::launch_prune_f32(a, true, p->tile_b, plan_run_samples(p),
                               p->pair_threads ? tt::kF32PairThreads
                                               : (p->inplace_adjoint ? tt::kF32InPlaceAdjoint |
                                                                           (p->pair_adjoint ? tt::kF32PairAdjoint : 0)
                                                                     : 0),
                               s);
      if (e == cudaSuccess)
        e = tt::launch_reduce_f32(static_cast<const float *>(p->d_gpart),
                                  static_cast<const float *>(p->d_rootpart), p->d_G, p->d_rootgrad,
                                  p->d_rootgrad + size_t(p->batch) * p->S, plan_run_samples(p), p->B, ntiles, p->S,
                                  p->K, p0 > 0, s);
    } else {
      auto a = make_args<double>(p, props, freqs, 1, true, nullptr);
      a.slots = p->slots_bwd;
      slab_args(a, p0, n, p->tile_b);
      e = tt::launch_prune_f64(a, true, p->tile_b, plan_run_samples(p), s);
      if (e == cudaSuccess)
        e = tt::launch_reduce_f64(static_cast<const double *>(p->d_gpart),
                                  static_cast<const double *>(p->d_rootpart), p->d_G, p->d_rootgrad,
                                  p->d_rootgrad + size_t(p->batch) * p->S, plan_run_samples(p), p->B, ntiles, p->S,
                                  p->K, p0 > 0, s);
    }
    p->launches += 3;
  }
  if (e != cudaSuccess) return cuda_fail(e, "adjoint launch");
  if (p->precision == TT_PRECISION_F32 && !p->pair_threads && p->inplace_adjoint && !p->slab)
    p->partials_valid = false;  // the outside partials overwrote the post-order tiles
  const size_t kss = size_t(p->K) * p->S * p->S;
  if (grad_matrices) {
    e = cudaMemcpyAsync(grad_matrices, p->d_G, size_t(p->batch) * p->B * kss * sizeof(double),
                        cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return cuda_fail(e, "dlnL/dP copy");
  }
  if (grad_frequencies) {
    e = cudaMemcpyAsync(grad_frequencies, p->d_rootgrad, size_t(p->batch) * p->S * sizeof(double),
                        cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return cuda_fail(e, "dlnL/dpi copy");
  }
  if (grad_weights) {
    e = cudaMemcpyAsync(grad_weights, p->d_rootgrad + size_t(p->batch) * p->S,
                        size_t(p->batch) * p->K * sizeof(double), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return cuda_fail(e, "dlnL/dc copy");
  }
  p->grads_valid = true;
  return TT_OK;
}

int tt_transition_matrices_gradient(tt_plan *p, const double *lam, const double *U, const double *W,
                                    const double *bl, const double *rates, double *dlam, double *dU,
                                    double *dW, double *dbl, double *drates, void *stream) {
  if (!p || !lam || !U || !W || !bl || !rates) return fail(TT_ERR_INVALID_ARGUMENT, "NULL argument");
  if (!p->grads_valid) return fail(TT_ERR_NOT_READY, "tt_gradient has not been called");
  int rc = check_device(p);
  if (rc) return rc;
  if (p->wide)
    return tt::wide_matrices_gradient(p, lam, U, W, bl, rates, dlam, dU, dW, dbl, drates,
                                      static_cast<cudaStream_t>(stream));
  cudaError_t e = tt::launch_pmatrix_backward(p->d_G, lam, U, W, bl, rates, p->S, p->B, p->K, p->batch,
                                              dlam, dU, dW, dbl, drates, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "transition-matrix gradient launch");
  p->launches += 1;
  return TT_OK;
}

int tt_rate_matrix_gradient(tt_plan *p, const double *lam, const double *U, const double *W, const double *bl,
                            const double *rates, double *dQ, double *dbl, double *drates, void *stream) {
  if (!p || !lam || !U || !W || !bl || !rates) return fail(TT_ERR_INVALID_ARGUMENT, "NULL argument");
  if (!p->grads_valid) return fail(TT_ERR_NOT_READY, "tt_gradient has not been called");
  int rc = check_device(p);
  if (rc) return rc;
  return tt::rate_matrix_gradient(p, lam, U, W, bl, rates, dQ, dbl, drates, static_cast<cudaStream_t>(stream));
}

int tt_plan_device_status(tt_plan *p, void *stream, int32_t *status, int32_t reset) {
  if (!p || !status) return fail(TT_ERR_INVALID_ARGUMENT, "NULL argument");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int v = 0;
  cudaError_t e = cudaMemcpyAsync(&v, p->d_status, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "status read");
  *status = v;
  if (reset) {
    e = cudaMemsetAsync(p->d_status, 0, sizeof(int), s);
    if (e != cudaSuccess) return cuda_fail(e, "status reset");
  }
  return TT_OK;
}

int tt_schedule(int32_t tip_count, const int32_t *postorder, int32_t *steps, int32_t *slot_counts) {
  if (!postorder || !steps || !slot_counts) return fail(TT_ERR_INVALID_ARGUMENT, "NULL argument");
  if (tip_count < 2) return fail(TT_ERR_INVALID_ARGUMENT, "a tree needs at least 2 tips");
  tt_plan tmp;
  tmp.T = tip_count;
  tmp.I = tip_count - 1;
  tmp.B = 2 * tip_count - 2;
  const int rc = build_schedule(&tmp, postorder);
  if (rc != TT_OK) return rc;
  std::memcpy(steps, tmp.steps.data(), tmp.steps.size() * sizeof(int));
  slot_counts[0] = tmp.slots_fwd;
  slot_counts[1] = tmp.slots_bwd;
  return TT_OK;
}

int tt_plan_set_option(tt_plan *p, int32_t option, int32_t value) {
  if (!p) return fail(TT_ERR_INVALID_ARGUMENT, "NULL plan");
  switch (option) {
    case TT_OPT_FWD_STAGES:
    case TT_OPT_BWD_STAGES: {
      if (p->wide || p->precision != TT_PRECISION_F32)
        return fail(TT_ERR_UNSUPPORTED, "ring depths apply to FP32 4-state plans");
      if (value < 2 || value > 8) return fail(TT_ERR_INVALID_ARGUMENT, "ring depth must be in [2, 8]");
      const bool bwd = option == TT_OPT_BWD_STAGES;
      int smem_max = 0;
      cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->device);
      const int sl = bwd ? p->slots_bwd : p->slots_fwd;
      if (std::max({tt::tl_smem_bytes(p->K, 256, sl, bwd, value), tt::tq_smem_bytes(p->K, 256, sl, bwd, value),
                    bwd ? size_t(0) : tt::tl_ws_smem_bytes(p->K, 256, p->slots_ws, value),
                    bwd ? std::max(tt::ta_smem_bytes(p->K, 256, value), tt::tp_smem_bytes(p->K, 256, value))
                        : size_t(0)}) > size_t(smem_max))
        return fail(TT_ERR_UNSUPPORTED, "ring does not fit in shared memory");
      (bwd ? p->nstage_b : p->nstage_f) = value;
      return TT_OK;
    }
    case TT_OPT_TENSOR_CORES:
      return tt::wide_set_tensor_cores(p, value != 0);
    case TT_OPT_TENSOR_CORE_ADJOINT:
      return tt::wide_set_tensor_core_adjoint(p, value != 0);
    case TT_OPT_PRODUCER_WARP:
      if (value && (p->wide || p->precision != TT_PRECISION_F32))
        return fail(TT_ERR_UNSUPPORTED, "the producer-warp post-order serves FP32 4-state plans");
      if (value && p->nstage_f > 8) return fail(TT_ERR_UNSUPPORTED, "the producer-warp post-order takes <= 8 stages");
      if (p->producer_warp != (value != 0)) p->partials_valid = false;
      p->producer_warp = value != 0;
      return TT_OK;
    case TT_OPT_PAIR_THREADS:
      if (value && (p->wide || p->precision != TT_PRECISION_F32 || !tt::pair_threads_supported(p->K)))
        return fail(TT_ERR_UNSUPPORTED, "pair-thread kernels serve FP32 4-state plans with 1-4 or 7-8 categories");
      if (p->pair_threads != (value != 0)) p->partials_valid = false;  // another partial layout
      p->pair_threads = value != 0;
      return TT_OK;
    case TT_OPT_INPLACE_ADJOINT:
      if (value && (p->wide || p->precision != TT_PRECISION_F32))
        return fail(TT_ERR_UNSUPPORTED, "the in-place adjoint serves FP32 4-state plans");
      if (p->inplace_adjoint != (value != 0)) p->partials_valid = false;
      p->inplace_adjoint = value != 0;
      return TT_OK;
    case TT_OPT_PAIR_ADJOINT:
      if (value && (p->wide || p->precision != TT_PRECISION_F32 || !tt::pair_adjoint_supported(p->K)))
        return fail(TT_ERR_UNSUPPORTED, "the pair-thread in-place adjoint serves FP32 4-state plans with 1-4 or 7-8 "
                                        "categories");
      p->pair_adjoint = value != 0;  // same partial layout: stored partials stay valid
      return TT_OK;
    case TT_OPT_SLAB_PATTERNS: {
      if (value < 0) return fail(TT_ERR_INVALID_ARGUMENT, "the slab size must be >= 0 (0 = all patterns)");
      const int slab = slab_round(value, p->N);
      auto alloc = [p](int n) { return p->wide ? tt::wide_alloc_slab(p, n) : alloc_grad_buffers(p, n); };
      if (slab == p->slab && (p->wide ? tt::wide_has_buffers(p) : p->d_partials != nullptr)) return TT_OK;
      const int old = p->slab;
      const int rc = alloc(slab);
      if (rc) {
        const std::string msg = g_last_error;
        alloc(old);  // keep the previous buffers when they can be had again
        return fail(rc, msg);
      }
      return TT_OK;
    }
    case TT_OPT_ACTIVE_SAMPLES:
      if (value < 0 || value > p->batch)
        return fail(TT_ERR_INVALID_ARGUMENT, "the active sample count must be in [0, batch] (0 = all)");
      if (plan_run_samples(p) != (value ? value : p->batch)) p->partials_valid = false;
      p->active = value;
      return TT_OK;
    default:
      return fail(TT_ERR_INVALID_ARGUMENT, "unknown option");
  }
}

int tt_plan_get_option(const tt_plan *p, int32_t option, int32_t *value) {
  if (!p || !value) return fail(TT_ERR_INVALID_ARGUMENT, "NULL argument");
  switch (option) {
    case TT_OPT_FWD_STAGES: *value = p->nstage_f; return TT_OK;
    case TT_OPT_BWD_STAGES: *value = p->nstage_b; return TT_OK;
    case TT_OPT_TENSOR_CORES: *value = tt::wide_tensor_cores(p) ? 1 : 0; return TT_OK;
    case TT_OPT_TENSOR_CORE_ADJOINT: *value = tt::wide_tensor_core_adjoint(p) ? 1 : 0; return TT_OK;
    case TT_OPT_PAIR_THREADS: *value = p->pair_threads ? 1 : 0; return TT_OK;
    case TT_OPT_PRODUCER_WARP: *value = p->producer_warp ? 1 : 0; return TT_OK;
    case TT_OPT_INPLACE_ADJOINT: *value = p->inplace_adjoint ? 1 : 0; return TT_OK;
    case TT_OPT_SLAB_PATTERNS: *value = p->slab; return TT_OK;
    case TT_OPT_PAIR_ADJOINT: *value = p->pair_adjoint ? 1 : 0; return TT_OK;
    case TT_OPT_ACTIVE_SAMPLES: *value = p->active; return TT_OK;
    default: return fail(TT_ERR_INVALID_ARGUMENT, "unknown option");
  }
}

int tt_plan_selftest_timeout(tt_plan *p, uint64_t limit_ns, void *stream) {
  if (!p) return fail(TT_ERR_INVALID_ARGUMENT, "NULL plan");
  if (limit_ns < 1 || limit_ns > 10000000000ull) return fail(TT_ERR_INVALID_ARGUMENT, "limit_ns must be in [1, 1e10]");
  int rc = check_device(p);
  if (rc) return rc;
  cudaError_t e = tt::launch_wait_selftest(p->d_status, limit_ns, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "self-test launch");
  p->launches += 1;
  return TT_OK;
}

int tt_plan_launch_count(const tt_plan *p, int64_t *count) {
  if (!p || !count) return fail(TT_ERR_INVALID_ARGUMENT, "NULL argument");
  *count = p->launches;
  return TT_OK;
}

}  // extern "C"
