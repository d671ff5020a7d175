// Internal plan state shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "tt_launch.h"

namespace tt {
struct WideState;  // state of the wide-state (S != 4) path, tt_wide.cu
}

struct tt_plan {
  int device = 0;
  int T = 0, I = 0, B = 0, S = 0, K = 0, N = 0, batch = 0, precision = 0;
  int C = 0, slots_fwd = 0, slots_bwd = 0;
  int slots_ws = 0;  // stack slots of the producer-warp post-order (register carry to the parent)
  int tile_f = 0, tile_b = 0, ntiles_f = 0, ntiles_b = 0, code_stride = 0;
  int nstage_f = tt::kStages, nstage_b = tt::kStages;
  size_t elem = 0;  // bytes per partial value
  bool pair_threads = false;  // FP32 4-state: one thread per (pattern, category pair)
  bool producer_warp = true;  // FP32 4-state post-order with a producer warp
  bool inplace_adjoint = true;  // FP32 4-state adjoint storing outside partials over the post-order tiles
  bool pair_adjoint = false;    // ... with one thread per (pattern, category pair) (tp_backward_kernel)
  bool tips_set = false, pmat_set = false, partials_valid = false, grads_valid = false;
  // patterns whose post-order partials are held at once (0 = all).  When
  // nonzero, tt_gradient recomputes the post-order one pattern slab at a
  // time into buffers of that size (wide plans also run tt_log_likelihood
  // slab by slab).
  int slab = 0;
  int last_rescale = 1;  // rescale flag of the last post-order (repeated by the slab recompute)
  int active = 0;        // samples the pruning passes run over (0 = all)
  long long launches = 0;
  std::vector<int> steps;       // host copy of the schedule (I x 12)
  std::vector<int> steps_ws;    // records of the producer-warp post-order (I x 12)
  std::vector<int> branch_pos;  // B
  // device buffers
  int4 *d_steps = nullptr;
  int4 *d_steps_rev = nullptr;
  int4 *d_steps_ws = nullptr;
  int *d_branch_pos = nullptr;
  uint8_t *d_codes = nullptr;
  void *d_table = nullptr;
  double *d_weights = nullptr;
  void *d_pmat = nullptr;
  void *d_partials = nullptr;
  double *d_tile_lnl = nullptr;
  void *d_gpart = nullptr;
  void *d_rootpart = nullptr;
  double *d_G = nullptr;
  double *d_rootgrad = nullptr;
  int *d_status = nullptr;
  double *d_qpart = nullptr;  // rate-matrix gradient partials and the finishing step's Z (first use)
  int qpart_chunks = 0;       // chunk slots of d_qpart
  size_t bytes = 0;
  size_t grad_bytes = 0;  // of `bytes`: the stored partials and per-tile gradient blocks
  tt::WideState *wide = nullptr;  // non-NULL for S != 4 plans
};

// Samples the pruning passes and their reductions run over (TT_OPT_ACTIVE_SAMPLES).
inline int plan_run_samples(const tt_plan *p) { return p->active > 0 && p->active < p->batch ? p->active : p->batch; }

namespace tt {
// Wide-state path (tt_wide.cu): same contracts as the C entry points.
int wide_create(tt_plan *p);  // everything but the pattern-sized buffers
// bytes of the pattern-sized buffers for passes over n patterns
size_t wide_pattern_bytes(const tt_plan *p, int n);
// (re)allocate the pattern-sized buffers for slabs of `slab` patterns (0 = all)
int wide_alloc_slab(tt_plan *p, int slab);
bool wide_has_buffers(const tt_plan *p);
void wide_destroy(tt_plan *p);
int wide_set_tips(tt_plan *p, const uint8_t *codes, const double *code_table, int code_count,
                  const double *weights);
int wide_update_matrices(tt_plan *p, const double *lam, const double *U, const double *W, const double *bl,
                         const double *rates, cudaStream_t s);
int wide_set_matrices(tt_plan *p, const double *matrices, cudaStream_t s);
int wide_log_likelihood(tt_plan *p, const double *props, const double *freqs, int rescale, bool keep,
                        double *lnl, double *site_lnl, cudaStream_t s);
int wide_gradient(tt_plan *p, const double *props, const double *freqs, double *grad_matrices,
                  double *grad_frequencies, double *grad_weights, cudaStream_t s);
int wide_matrices_gradient(tt_plan *p, const double *lam, const double *U, const double *W, const double *bl,
                           const double *rates, double *dlam, double *dU, double *dW, double *dbl,
                           double *drates, cudaStream_t s);
int wide_set_tensor_cores(tt_plan *p, bool on);
int wide_set_tensor_core_adjoint(tt_plan *p, bool on);
bool wide_tensor_core_adjoint(const tt_plan *p);
// dlnL/dQ, branch lengths and category rates from the plan's dlnL/dP (tt_qgrad.cu)
int rate_matrix_gradient(tt_plan *p, const double *lam, const double *U, const double *W, const double *bl,
                         const double *rates, double *dQ, double *dbl, double *drates, cudaStream_t s);
bool wide_tensor_cores(const tt_plan *p);
}  // namespace tt
