/*
 * torchtree_gb300 — C ABI of the GB300 tree-likelihood engine.
 *
 * Felsenstein pruning log-likelihood and its gradient for a batch of
 * samples that share one tree topology and one compressed alignment.
 * All entry points take plain pointers and sizes; device pointers are
 * CUDA global-memory addresses on the current device, `stream` is a
 * cudaStream_t (NULL = legacy default stream).  Every call returns a
 * tt_status (0 = success); tt_last_error() gives a message for the calling
 * thread's most recent failure.
 *
 * Index conventions (torchtree/evolution/tree_model.py:37-53):
 *   tips 0..T-1 in taxa order, internal nodes T..2T-2, root = 2T-2;
 *   the branch above node i carries index i, so there are B = 2T-2 branches.
 * Layouts (row-major, batch outermost):
 *   eigenvalues [b][S], eigenvectors U [b][S][S], inverse W [b][S][S],
 *   branch_lengths [b][B], category_rates [b][K], category_weights [b][K],
 *   frequencies [b][S], transition matrices [b][B][K][S][S] (P[i][j] =
 *   P(j at child | i at parent), the reference's `mats`).
 */
#ifndef TORCHTREE_GB300_H
#define TORCHTREE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  TT_OK = 0,
  TT_ERR_INVALID_ARGUMENT = 1,
  TT_ERR_UNSUPPORTED = 2,
  TT_ERR_OUT_OF_MEMORY = 3,
  TT_ERR_CUDA = 4,
  TT_ERR_DEVICE_TIMEOUT = 5, /* a bounded device-side wait gave up */
  TT_ERR_NOT_READY = 6       /* a required earlier call was not made */
} tt_status;

enum { TT_PRECISION_F32 = 0, TT_PRECISION_F64 = 1 };

typedef struct tt_plan tt_plan;

/* Library version string. */
const char *tt_version(void);

/* Message of the calling thread's last failed call ("" if none). */
const char *tt_last_error(void);

/*
 * Create a plan for one topology.  Replaces the per-call set-up that
 * TreeLikelihoodModel.__init__ / _call do in Python
 * (torchtree/evolution/tree_likelihood.py:283-311, 313-356).
 *   postorder: host int32 [T-1][3] of (node, left, right) triples in a
 *              valid post-order (tree_model.py:187-195); the last triple is
 *              the root.
 *   precision: TT_PRECISION_F32 (partials in FP32 with rescaling; log
 *              scalers and the pattern sum in FP64) or TT_PRECISION_F64.
 * Allocates all device workspace on the current device.
 */
int tt_plan_create(tt_plan **plan, int32_t tip_count, const int32_t *postorder,
                   int32_t state_count, int32_t category_count,
                   int32_t pattern_count, int32_t batch, int32_t precision);

/* Release a plan and its device memory (NULL is accepted).  The reference
 * frees its tensors with the TreeLikelihoodModel object: no explicit
 * counterpart. */
int tt_plan_destroy(tt_plan *plan);

/* Device bytes held by the plan (no reference counterpart; admission by
 * memory footprint uses it). */
int tt_plan_workspace_bytes(const tt_plan *plan, size_t *bytes);

/*
 * Upload the compressed alignment (site_pattern.py:100-151): per tip and
 * pattern a uint8 code indexing `code_table`, the distinct tip partial
 * vectors.  A tip-state alignment (compute_tips_states) uses the table
 * [one-hot rows 0..S-1, all-ones row S]; a partial-vector alignment
 * (compute_tips_partials) uses its distinct columns.
 *   codes:      host uint8 [T][N], every value < code_count
 *   code_table: host double [code_count][S], code_count <= 256
 *   weights:    host double [N] (the reference's int64 pattern counts)
 */
int tt_plan_set_tips(tt_plan *plan, const uint8_t *codes,
                     const double *code_table, int32_t code_count,
                     const double *weights);

/*
 * Transition matrices from an eigen system, all branches x categories x
 * samples in one launch (substitution_model/abstract.py:57-76):
 *   P[b][i][k] = U[b] diag(exp(lambda[b] * t[b][i] * r[b][k])) W[b]
 * computed in FP64 and stored at the plan's precision.
 */
int tt_update_transition_matrices(tt_plan *plan, const double *eigenvalues,
                                  const double *eigenvectors,
                                  const double *inverse_eigenvectors,
                                  const double *branch_lengths,
                                  const double *category_rates, void *stream);

/*
 * Transition matrices given directly (the reference's `mats` argument,
 * tree_likelihood.py:40-75): device double [b][B][K][S][S].
 */
int tt_set_transition_matrices(tt_plan *plan, const double *matrices,
                               void *stream);

/*
 * Log-likelihood per sample (tree_likelihood.py:40-75 without rescaling,
 * 186-221 with rescaling):
 *   lnL[b] = sum_n w_n log( sum_k c[b][k] sum_i pi[b][i] L_root[b][k][i][n] )
 * rescale != 0 rescales every internal partial by a power of two and
 * accumulates the exponents exactly; rescale == 0 runs unscaled.
 * keep_partials != 0 stores the internal partials for tt_gradient.
 *   log_likelihood:      device double [b]
 *   site_log_likelihood: device double [b][N] or NULL
 */
int tt_log_likelihood(tt_plan *plan, const double *category_weights,
                      const double *frequencies, int32_t rescale,
                      int32_t keep_partials, double *log_likelihood,
                      double *site_log_likelihood, void *stream);

/*
 * Gradient of sum_b lnL[b] after tt_log_likelihood(keep_partials=1),
 * by a pre-order adjoint pass (replaces autograd through
 * tree_likelihood.py:186-221):
 *   grad_matrices:          device double [b][B][K][S][S] or NULL
 *   grad_frequencies:       device double [b][S] or NULL
 *   grad_category_weights:  device double [b][K] or NULL
 * The gradient with respect to P is always kept inside the plan for
 * tt_transition_matrices_gradient.  FP32 plans (unless
 * TT_OPT_INPLACE_ADJOINT is 0) and plans with S != 4 consume the stored
 * partials: a second tt_gradient needs a new tt_log_likelihood with
 * keep_partials=1 (TT_ERR_NOT_READY otherwise).  Plans with pattern slabs
 * (TT_OPT_SLAB_PATTERNS) recompute the post-order here, one slab at a time,
 * and need no new tt_log_likelihood.
 */
int tt_gradient(tt_plan *plan, const double *category_weights,
                const double *frequencies, double *grad_matrices,
                double *grad_frequencies, double *grad_category_weights,
                void *stream);

/*
 * Chain the plan's dlnL/dP (from tt_gradient) through
 * P = U diag(exp(lambda t r)) W (abstract.py:67-76).  Outputs (device
 * double, any may be NULL): grad_eigenvalues [b][S], grad_eigenvectors
 * [b][S][S], grad_inverse_eigenvectors [b][S][S], grad_branch_lengths
 * [b][B], grad_category_rates [b][K].
 */
int tt_transition_matrices_gradient(
    tt_plan *plan, const double *eigenvalues, const double *eigenvectors,
    const double *inverse_eigenvectors, const double *branch_lengths,
    const double *category_rates, double *grad_eigenvalues,
    double *grad_eigenvectors, double *grad_inverse_eigenvectors,
    double *grad_branch_lengths, double *grad_category_rates, void *stream);

/*
 * Chain the plan's dlnL/dP (from tt_gradient) to the rate matrix itself:
 * with Q = U diag(lambda) W and P = exp(Q t r), dlnL/dQ = W^T X U^T where
 * X = sum over branches and categories of F(t r) .* (U^T G W^T) and
 * F_mn = (e^(lambda_m t r) - e^(lambda_n t r)) / (lambda_m - lambda_n)
 * (t r e^(lambda_m t r) when equal) -- the derivative of the matrix
 * exponential in its eigenbasis.  This replaces autograd through
 * abstract.py:57-79 including the eigendecomposition, so callers chain
 * dlnL/dQ straight into the rate-matrix parameters (no eigenvector
 * derivatives).  Outputs (device double, any may be NULL):
 * grad_rate_matrix [b][S][S], grad_branch_lengths [b][B],
 * grad_category_rates [b][K].
 */
int tt_rate_matrix_gradient(tt_plan *plan, const double *eigenvalues,
                            const double *eigenvectors,
                            const double *inverse_eigenvectors,
                            const double *branch_lengths,
                            const double *category_rates,
                            double *grad_rate_matrix,
                            double *grad_branch_lengths,
                            double *grad_category_rates, void *stream);

/*
 * Device status word: TT_OK, or TT_ERR_DEVICE_TIMEOUT when a kernel's
 * bounded wait gave up since the last reset.  Synchronises the stream.  No
 * reference counterpart: the reference has no device waits and reports
 * numeric trouble in-band (a -inf lnL, tree_likelihood.py:378-388).
 */
int tt_plan_device_status(tt_plan *plan, void *stream, int32_t *status,
                          int32_t reset);

/*
 * Host-only: the execution schedule a plan would use (no device needed):
 * the post-order of update_traversals (tree_model.py:187-195) as the
 * kernels' step records.
 *   steps: int32 [T-1][12] per step (node, left, right, forward slot of
 *          left / right / output, adjoint slot of input / left / right,
 *          the in-place adjoint's flags: carry or store each internal child
 *          and whether this node's outside partial was stored, the reversed
 *          index of the step that stored it, 1 unused), -1 where a slot does
 *          not apply;
 *   slot_counts: int32 [2] shared-memory slots of the forward and adjoint.
 * Validates `postorder` exactly as tt_plan_create does.
 */
int tt_schedule(int32_t tip_count, const int32_t *postorder, int32_t *steps,
                int32_t *slot_counts);

/*
 * tt_log_likelihood / tt_gradient of several plans in one call.  No
 * counterpart in the reference (it evaluates one model per call); it serves a
 * server that batches the work of many data sets.  Plans on the default FP32
 * 4-state kernels (producer-warp post-order, in-place adjoint, whole
 * alignment resident) with one category-pair count are merged into one
 * post-order launch and one adjoint launch over all their tiles (up to 16
 * plans per launch); every other plan runs its own calls.  Each plan's
 * results are the ones its own calls give, bit for bit.
 *   plans[count], category_weights[count], frequencies[count] (device, per
 *   plan as for tt_log_likelihood), log_likelihood[count] (device);
 *   grad_frequencies / grad_weights: NULL or arrays of `count` device
 *   pointers (entries may be NULL).  A plan may appear once per call.
 */
int tt_plans_log_likelihood(int32_t count, tt_plan *const *plans,
                            const double *const *category_weights,
                            const double *const *frequencies, int32_t rescale,
                            int32_t keep_partials, double *const *log_likelihood,
                            void *stream);
int tt_plans_gradient(int32_t count, tt_plan *const *plans,
                      const double *const *category_weights,
                      const double *const *frequencies,
                      double *const *grad_frequencies,
                      double *const *grad_weights, void *stream);

/*
 * Eigen system of reversible rate matrices on the device, FP64.  Replaces
 * the eigendecomposition inside SymmetricSubstitutionModel.p_t
 * (torchtree/evolution/substitution_model/abstract.py:57-79: Q normalised,
 * symmetrised with Pi^1/2, eigh).
 *   q: device double [b][S][S], normalised rate matrices (rows sum to 0,
 *      reversible with respect to `frequencies`); only the lower triangle of
 *      Pi^1/2 Q Pi^-1/2 is read, as eigh does;
 *   frequencies: device double [b][S];
 *   eigenvalues [b][S] (ascending), u [b][S][S], w [b][S][S] with
 *   Q = U diag(eigenvalues) W and W = U^-1 (device);
 *   status: device int32, set to TT_ERR_UNSUPPORTED if a matrix did not
 *   converge (never cleared here).
 * 1 <= S <= 64.  FP32 Jacobi, two FP64 Newton-Schulz steps on its
 * eigenvectors, FP64 Jacobi on the rotated matrix; 7 launches on `stream`,
 * no workspace.
 */
int tt_reversible_eigen(int32_t batch, int32_t state_count, const double *q,
                        const double *frequencies, double *eigenvalues,
                        double *u, double *w, int32_t *status, void *stream);

/*
 * Transition matrices of general (not necessarily reversible) rate
 * matrices: P[b][br][k] = exp(Q_b * branch_lengths[b][br] *
 * category_rates[b][k]), FP64, every matrix in one launch (scaling and
 * squaring with the [13/13] Pade approximant).  Replaces
 * NonSymmetricSubstitutionModel.p_t (torchtree/evolution/substitution_model/
 * abstract.py:86-94: torch.matrix_exp of the normalised Q times t).
 *   q [b][S][S] (normalised), branch_lengths [b][B], category_rates [b][K],
 *   matrices [b][B][K][S][S]; all device; S <= 64.  The result goes to a
 *   plan through tt_set_transition_matrices.
 */
int tt_transition_matrices_expm(int32_t batch, int32_t state_count,
                                int32_t branch_count, int32_t category_count,
                                const double *q, const double *branch_lengths,
                                const double *category_rates, double *matrices,
                                void *stream);

/*
 * Adjoint of tt_transition_matrices_expm (autograd through torch.matrix_exp
 * in the reference, abstract.py:86-94): for G = dlnL/dP [b][B][K][S][S] (tt_gradient's
 * grad_matrices), grad_q_parts[b][br][k] = tau L(tau Q^T, G) (the Frechet
 * derivative, tau = t r) and grad_times[b][br][k] = tr(G^T Q P); dlnL/dQ is
 * the sum of the parts over branches and categories, dlnL/dt_br =
 * sum_k r_k grad_times, dlnL/dr_k = sum_br t_br grad_times.  S <= 32.
 */
int tt_transition_matrices_expm_adjoint(int32_t batch, int32_t state_count,
                                        int32_t branch_count, int32_t category_count,
                                        const double *q, const double *branch_lengths,
                                        const double *category_rates,
                                        const double *grad_matrices,
                                        double *grad_q_parts, double *grad_times,
                                        void *stream);

/*
 * Quantiles of the Gamma(shape, rate 1) distribution at (2k+1)/(2K),
 * k = 0..K-1, and their derivative with respect to the shape (FP64,
 * analytic).  The discretised Gamma site model's rates are x_k / mean(x)
 * (the quantile construction of site_model.py:173-195; torchtree itself
 * ships no Gamma model).  shape [b], x [b][K], dx_dshape [b][K].
 * tt_gamma_quantiles takes device pointers and writes NaN where the shape is
 * not finite and positive; tt_gamma_quantiles_host takes host pointers and
 * returns TT_ERR_INVALID_ARGUMENT instead.
 */
int tt_gamma_quantiles(int32_t batch, int32_t category_count, const double *shape,
                       double *x, double *dx_dshape, void *stream);
int tt_gamma_quantiles_host(int32_t batch, int32_t category_count,
                            const double *shape, double *x, double *dx_dshape);

/*
 * FP64 log-likelihood that allocates no device memory.  No counterpart in
 * the reference: it exists for callers that cannot call cudaMalloc (an
 * application whose own memory manager owns every device byte, or a host
 * that hands a plug-in device buffers but no right to allocate), for whom
 * tt_plan_create is closed.  Same result as tt_set_transition_matrices +
 * tt_log_likelihood on a TT_PRECISION_F64 plan.
 *   postorder: host int32 [T-1][3]; 2 <= T <= 1024; state_count 4;
 *   codes device uint8 [T][N] (< code_count), code_table device double
 *   [code_count][4], weights device double [N], matrices device double
 *   [b][B][K][4][4], category_weights device [b][K], frequencies device
 *   [b][4], log_likelihood device double [b].
 * Scratch lives in one 8 MiB static device array held by every GPU that
 * loads the library; a problem needing more is rejected with
 * TT_ERR_INVALID_ARGUMENT.  Every call looks the array's address up in the
 * current context (the first call on a device loads the module).  A stream
 * that is being captured is refused (TT_ERR_UNSUPPORTED): the schedule is
 * copied from pageable host memory.  The call synchronises `stream` before
 * it returns and reads the kernel's status word back; a bounded wait that
 * gave up returns TT_ERR_DEVICE_TIMEOUT.  A tip code >= code_count gives a
 * NaN log-likelihood for the samples it touches.  Calls share the array:
 * calls that overlap on the GPU race and must be serialised by the caller.
 */
int tt_log_likelihood_static(int32_t tip_count, const int32_t *postorder,
                             int32_t state_count, int32_t category_count,
                             int32_t pattern_count, int32_t batch,
                             const uint8_t *codes, const double *code_table,
                             int32_t code_count, const double *weights,
                             const double *matrices,
                             const double *category_weights,
                             const double *frequencies, int32_t rescale,
                             double *log_likelihood, void *stream);

/*
 * Site-pattern compression on the host (site_pattern.py:69-97): the distinct
 * columns of `matrix` (uint8 [rows][sites], row-major; one row per taxon, or
 * per taxon and codon position) in lexicographic order of the column read
 * from row 0 down -- the reference's sorted(Counter(zip(*sequences))) -- and
 * their counts.  Outputs: *n_patterns; first_site [sites] (a site holding
 * pattern p, its first occurrence); counts [sites]; site_pattern [sites] or
 * NULL (the pattern of every site).  No device memory is touched.
 */
int tt_compress_columns(const uint8_t *matrix, int64_t rows, int64_t sites,
                        int64_t *n_patterns, int64_t *first_site,
                        int64_t *counts, int64_t *site_pattern);

/*
 * Time-tree operations (no reference kernels; the reference evaluates them
 * with torch ops and autograd):
 *   tt_time_tree_create: topology (postorder as for tt_plan_create) and the
 *     tips' sampling times (host double [T]); lower bounds of internal nodes
 *     are the largest sampling time below them (tree_height_transform.py:38-60).
 *   tt_ratio_transform: GeneralNodeHeightTransform._call and
 *     log_abs_det_jacobian (tree_height_transform.py:62-99): ratios [b][T-1]
 *     (internal nodes T..2T-3 by index - T, root height last) -> internal
 *     heights [b][T-1], branch lengths [b][2T-2] (h[parent] - h[child],
 *     tree_model.py:23-40; may be NULL), log|J| [b].  Device pointers.
 *   tt_ratio_transform_backward: dlnL/dratios [b][T-1] from dlnL/dheights,
 *     dlnL/dbranch_lengths, dlnL/dlog|J| (any of the three may be NULL).
 *     Both transform calls take T <= 9,600 (a sample's rows in shared memory).
 *   tt_constant_coalescent: ConstantCoalescent.log_prob
 *     (coalescent.py:112-134) for internal heights [b][T-1] and theta [b]:
 *     log_prob [b], gradients [b][T-1] and [b] (may be NULL); T <= 4,096.
 */
typedef struct tt_time_tree tt_time_tree;
int tt_time_tree_create(tt_time_tree **tree, int32_t tip_count,
                        const int32_t *postorder, const double *sampling_times);
int tt_time_tree_destroy(tt_time_tree *tree);
int tt_ratio_transform(tt_time_tree *tree, int32_t batch, const double *ratios,
                       double *heights, double *branch_lengths,
                       double *log_det_jacobian, void *stream);
int tt_ratio_transform_backward(tt_time_tree *tree, int32_t batch,
                                const double *ratios, const double *heights,
                                const double *grad_heights,
                                const double *grad_branch_lengths,
                                const double *grad_log_det, double *grad_ratios,
                                void *stream);
int tt_constant_coalescent(tt_time_tree *tree, int32_t batch,
                           const double *heights, const double *theta,
                           double *log_prob, double *grad_heights,
                           double *grad_theta, void *stream);

/*
 * Self-test of the device-side failure path (no reference counterpart): one
 * kernel waits, with the bounded wait every staged kernel uses, on a barrier
 * that nothing completes, gives up after limit_ns (1 .. 1e10) and records
 * TT_ERR_DEVICE_TIMEOUT in the plan's status word, which
 * tt_plan_device_status then reports.  The context and the plan stay usable.
 */
int tt_plan_selftest_timeout(tt_plan *plan, uint64_t limit_ns, void *stream);

/* Number of kernel launches the plan issued since creation (no reference
 * counterpart). */
int tt_plan_launch_count(const tt_plan *plan, int64_t *count);

/*
 * Options of a plan (no reference counterpart: the reference has no kernels
 * to shape and keeps autograd's whole graph).  Kernel shapes, for
 * autotuning, leave results unchanged; the pattern-slab size changes only
 * the grouping of FP64 sums.
 *   TT_OPT_FWD_STAGES / TT_OPT_BWD_STAGES: staging-ring depth of the FP32
 *     4-state post-order / adjoint kernels (2..8; rejected when the ring
 *     does not fit in shared memory);
 *   TT_OPT_TENSOR_CORES: 1 = FP32 codon post-order on the tensor cores,
 *     0 = CUDA-core kernel;
 *   TT_OPT_TENSOR_CORE_ADJOINT: 1 = FP32 codon adjoint on the tensor cores
 *     (the default; holds split copies of the transition matrices, 32 KB per
 *     sample, branch and category), 0 = CUDA-core kernel;
 *   TT_OPT_PAIR_THREADS: FP32 4-state kernels with one thread per (pattern,
 *     category pair) (1) or per pattern (0, the default);
 *   TT_OPT_PRODUCER_WARP: FP32 4-state post-order with a warp that only
 *     issues the staging copies (1, the default) or with the copies issued
 *     by the first compute thread and a block barrier per step (0);
 *   TT_OPT_INPLACE_ADJOINT: FP32 4-state adjoint that writes the outside
 *     partials over the stored post-order tiles (1, the default: a second
 *     tt_gradient then needs a new tt_log_likelihood with keep_partials=1)
 *     or keeps them in a shared-memory stack (0);
 *   TT_OPT_PAIR_ADJOINT: that in-place adjoint with the category pairs of a
 *     pattern on adjacent threads (1) or all in one thread (0); K in 1-4 or
 *     7-8; either reads the same stored partials;
 *   TT_OPT_SLAB_PATTERNS: how many patterns' post-order partials are held
 *     at once (rounded up to a multiple of 512; 0 = all, the default when
 *     they fit).  With a slab size set, tt_gradient recomputes the post-order
 *     one slab at a time before each slab's adjoint, and a second
 *     tt_gradient for the same matrices needs no new tt_log_likelihood.
 *     4-state plans: tt_log_likelihood stores nothing (one extra post-order
 *     pass per gradient).  20/61-state plans: tt_log_likelihood also runs
 *     slab by slab and leaves the last slab's partials for the gradient.
 *     tt_plan_create picks a slab size itself when the whole alignment's
 *     partials and per-tile gradient blocks would take more than 7/8 of the
 *     free device memory.  Setting it reallocates those buffers and drops
 *     any kept partials.  Results equal the unslabbed ones up to the order
 *     of the FP64 sums over slabs.
 *   TT_OPT_ACTIVE_SAMPLES: run the post-order, the adjoint and their
 *     reductions (tt_log_likelihood, tt_gradient and the tt_plans_* calls)
 *     over samples 0 .. n-1 only (1 <= n <= batch; 0 = all, the default).  Transition matrices and the rate-matrix chain still
 *     cover every sample; the log-likelihoods and gradients of samples >= n
 *     are left unspecified.  The results of samples < n equal those of a
 *     call over all samples.  A change of n drops any kept partials.
 * tt_plan_get_option reads the value in use.
 */
enum {
  TT_OPT_FWD_STAGES = 1,
  TT_OPT_BWD_STAGES = 2,
  TT_OPT_TENSOR_CORES = 3,
  TT_OPT_PAIR_THREADS = 4,
  TT_OPT_PRODUCER_WARP = 5,
  TT_OPT_INPLACE_ADJOINT = 6,
  TT_OPT_SLAB_PATTERNS = 7,
  TT_OPT_PAIR_ADJOINT = 8,
  TT_OPT_TENSOR_CORE_ADJOINT = 9,
  TT_OPT_ACTIVE_SAMPLES = 10
};
int tt_plan_set_option(tt_plan *plan, int32_t option, int32_t value);
int tt_plan_get_option(const tt_plan *plan, int32_t option, int32_t *value);

#ifdef __cplusplus
}
#endif

#endif /* TORCHTREE_GB300_H */
