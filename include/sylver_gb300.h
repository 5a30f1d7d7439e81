/*
 * sylver_gb300: GB300-native numeric factorize + solve for sparse symmetric
 * systems (multifrontal Cholesky and threshold-pivoted LDL^T), exported with
 * the reference SyLVER C-ABI so that existing callers relink unchanged.
 *
 * Indexing, ownership and error conventions are the reference's:
 *   - ptr/row are 1-based lower-triangle CSC (ptr is long, row is int);
 *   - akeep/fkeep are opaque handles allocated by the library and released by
 *     spldlt_free_akeep/spldlt_free_fkeep;
 *   - errors come back in inform->flag (<0 error, >0 warning, 0 success);
 *   - factorize and solve are synchronous.
 * Factors live in GPU memory owned by fkeep.  There is no CPU fallback: when
 * no CUDA device is usable, factorize returns SYLVER_ERROR_CUDA_UNKNOWN (-51).
 */
#ifndef SYLVER_GB300_H
#define SYLVER_GB300_H

#include <stdbool.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Reference: include/sylver/sylver.h:19-37 (same layout). */
typedef struct {
  int flag;
  int matrix_dup;
  int matrix_missing_diag;
  int matrix_outrange;
  int matrix_rank;
  int maxdepth;
  int maxfront;
  int num_delay;
  long num_factor;
  long num_flops;
  int num_neg;
  int num_sup;
  int num_two;
  int stat;
  int cuda_error;
  int cublas_error;
  char unused[80];
} sylver_inform_t;

/* Reference: include/sylver/sylver.h:39-71 (same layout). */
typedef struct {
  int array_base;
  int print_level;
  int unit_diagnostics;
  int unit_error;
  int unit_warning;
  int ordering;
  int nemin;
  bool prune_tree;
  long min_gpu_work;
  int scaling;
  int pivot_method;
  double small;
  double u;
  long small_subtree_threshold;
  int nb;
  int cpu_topology;
  bool action;
  bool use_gpu;
  double gpu_perf_coeff;
  int failed_pivot_method;
  int scheduler;
} sylver_options_t;

/* Error / warning flags: src/sylver_datatypes_mod.F90:14-45. */
enum {
  SYLVER_SUCCESS = 0,
  SYLVER_ERROR_CALL_SEQUENCE = -1,
  SYLVER_ERROR_A_N_OOR = -2,
  SYLVER_ERROR_A_PTR = -3,
  SYLVER_ERROR_A_ALL_OOR = -4,
  SYLVER_ERROR_SINGULAR = -5,
  SYLVER_ERROR_NOT_POS_DEF = -6,
  SYLVER_ERROR_PTR_ROW = -7,
  SYLVER_ERROR_ORDER = -8,
  SYLVER_ERROR_VAL = -9,
  SYLVER_ERROR_X_SIZE = -10,
  SYLVER_ERROR_JOB_OOR = -11,
  SYLVER_ERROR_NOT_LLT = -13,
  SYLVER_ERROR_NOT_LDLT = -14,
  SYLVER_ERROR_NO_SAVED_SCALING = -15,
  SYLVER_ERROR_ALLOCATION = -50,
  SYLVER_ERROR_CUDA_UNKNOWN = -51,
  SYLVER_ERROR_CUBLAS_UNKNOWN = -52,
  SYLVER_ERROR_UNIMPLEMENTED = -98,
  SYLVER_ERROR_UNKNOWN = -99,
  SYLVER_WARNING_IDX_OOR = 1,
  SYLVER_WARNING_DUP_IDX = 2,
  SYLVER_WARNING_DUP_AND_OOR = 3,
  SYLVER_WARNING_MISSING_DIAGONAL = 4,
  SYLVER_WARNING_MISS_DIAG_OORDUP = 5,
  SYLVER_WARNING_ANAL_SINGULAR = 6,
  SYLVER_WARNING_FACT_SINGULAR = 7,
  SYLVER_WARNING_MATCH_ORD_NO_SCALE = 8,
  /* No reference counterpart: iterative refinement (FP32 factors, or FP64
   * with ir_max_iter > 0) stopped at ir_max_iter corrections with the scaled
   * backward error still above ir_tol; x holds the last iterate and
   * sylver_gb300_solve_stats the error reached. */
  SYLVER_GB300_WARNING_IR_NOT_CONVERGED = 9
};

/* Solve job values: src/sylver_datatypes_mod.F90:46-51. */
enum {
  SYLVER_SOLVE_JOB_ALL = 0,
  SYLVER_SOLVE_JOB_FWD = 1,
  SYLVER_SOLVE_JOB_DIAG = 2,
  SYLVER_SOLVE_JOB_BWD = 3,
  SYLVER_SOLVE_JOB_DIAG_BWD = 4
};

/* ---- public C-ABI (replaces src/interfaces/C/sylver_ciface.F90) ---------- */

/* Replaces sylver_c_init (sylver_ciface.F90:354-364): selects device 0 and
 * creates the library's stream.  ncpu/ngpu are accepted and recorded. */
void sylver_init(int ncpu, int ngpu);
/* Replaces sylver_c_finalize (sylver_ciface.F90:367-375). */
void sylver_finalize(void);
/* Replaces sylver_c_default_options (sylver_ciface.F90:304-351). */
void sylver_default_options(sylver_options_t* options);
/* Replaces spldlt_c_analyse (sylver_ciface.F90:374-467).  options->ordering
 * 0 takes `order` (order[i] = 1-based pivot position of variable i); any
 * other value runs the library's nested dissection. */
void spldlt_analyse(int n, int* order, long const* ptr, int const* row, double const* val,
                    void** akeep, bool check, sylver_options_t const* options,
                    sylver_inform_t* inform);
/* Replaces spldlt_c_factorize (sylver_ciface.F90:530-631), FP64 factors.
 * With options->scaling <= 0 and a non-null `scale` (length n, user order)
 * the factorization is of S A S, S = diag(scale)
 * (src/spldlt_factorize_mod.F90:727-733); spldlt_solve then applies S on the
 * way in for jobs 0 and 1 and on the way out for jobs 0, 3 and 4, as the
 * reference's solve does (src/spldlt_factorize_mod.F90:945-1050), so that job
 * 0 solves A x = b.  Refinement (FP32 factors) uses the residual of A. */
void spldlt_factorize(bool posdef, long const* ptr, int const* row, double const* val,
                      double* scale, void* akeep, void** fkeep,
                      sylver_options_t const* options, sylver_inform_t* inform);
/* Replaces spldlt_c_solve (sylver_ciface.F90:634-711).  x is ldx x nrhs,
 * column-major, overwritten by the solution.  When fkeep holds FP32 factors
 * (spldlt_factorize_mixed) job 0 runs FP64 iterative refinement. */
void spldlt_solve(int job, int nrhs, double* x, int ldx, void* akeep, void* fkeep,
                  sylver_options_t const* options, sylver_inform_t* inform);
/* Replace spldlt_c_free_akeep / spldlt_c_free_fkeep (sylver_ciface.F90:714-826). */
void spldlt_free_akeep(void** akeep);
void spldlt_free_fkeep(void** fkeep);

/* ---- internal C-ABI #2 (replaces src/SymbolicTree.cxx, src/NumericTree*.cxx) */

/* Interoperable options/inform: src/sylver_ciface.hxx:39-87. */
typedef struct {
  int print_level;
  bool action;
  double small;
  double u;
  double multiplier;
  long small_subtree_threshold;
  int nb;
  int pivot_method;
  int failed_pivot_method;
  int cpu_topology;
} sylver_options_c;

typedef struct {
  int flag;
  int num_delay;
  int num_neg;
  int num_two;
  int num_zero;
  int maxfront;
  int not_first_pass;
  int not_second_pass;
} sylver_inform_c;

/* Replaces spldlt_create_symbolic_tree (src/SymbolicTree.cxx:110-137).  The
 * arrays are copied; nsubtrees/subtrees/small/contrib_dest/exec_loc are
 * accepted for signature compatibility (no CPU subtrees exist here). */
void* spldlt_create_symbolic_tree(void* akeep, int n, int nnodes, int const* sptr,
                                  int const* sparent, long const* rptr, int const* rlist,
                                  long const* nptr, long const* nlist, int nsubtrees,
                                  int const* subtrees, int const* small,
                                  int const* contrib_dest, int const* exec_loc);
void spldlt_destroy_symbolic_tree(void* symbolic_tree);

/* Replace spldlt_create_numeric_tree_dbl (src/NumericTree.cxx:27-45) and
 * spldlt_create_numeric_tree_posdef_dbl (src/NumericTreePosdef.cxx:19-35),
 * same argument order as the Fortran bind(C) interfaces
 * (src/spldlt_factorize_mod.F90:72-83).  aval is host memory (values in the
 * order nlist refers to).  scaling (null: none) is indexed by the tree's
 * variables (the rlist values, 1-based there): entry (r, c) of a front is
 * initialised to scaling[r] * a * scaling[c] as init_a_block does
 * (src/kernels/assemble.hxx:162-180).  The tree solves then work on the
 * scaled system; applying the scaling to x around them is the caller's job,
 * as in the reference's Fortran solve (src/spldlt_factorize_mod.F90:945-1050). */
void* spldlt_create_numeric_tree_dbl(bool posdef, void* fkeep, void* symbolic_tree,
                                     double* aval, const double* scaling,
                                     void** child_contrib, sylver_options_c* options,
                                     sylver_inform_c* inform);
void* spldlt_create_numeric_tree_posdef_dbl(void* fkeep, void* symbolic_tree, double* aval,
                                            const double* scaling, void** child_contrib,
                                            sylver_options_c* options, sylver_inform_c* inform);
void spldlt_destroy_numeric_tree_dbl(bool posdef, void* tree);
void spldlt_destroy_numeric_tree_posdef_dbl(void* tree);

/* Replace spldlt_tree_solve_{fwd,bwd,diag,diag_bwd}_dbl
 * (src/NumericTree.cxx:56-136) and the _posdef_ fwd/bwd
 * (src/NumericTreePosdef.cxx:46-83).  x is host memory, indexed in pivot
 * order as the reference's tree solves expect; returns a reference flag. */
int spldlt_tree_solve_fwd_dbl(bool posdef, void const* tree, int nrhs, double* x, int ldx);
int spldlt_tree_solve_bwd_dbl(bool posdef, void const* tree, int nrhs, double* x, int ldx);
int spldlt_tree_solve_diag_dbl(bool posdef, void const* tree, int nrhs, double* x, int ldx);
int spldlt_tree_solve_diag_bwd_dbl(bool posdef, void const* tree, int nrhs, double* x, int ldx);
int spldlt_tree_solve_fwd_posdef_dbl(void const* tree, int nrhs, double* x, int ldx);
int spldlt_tree_solve_bwd_posdef_dbl(void const* tree, int nrhs, double* x, int ldx);

/* ---- GB300 extensions (no reference counterpart) ------------------------- */

/* Factor precision selector for spldlt_factorize_mixed. */
enum { SYLVER_GB300_FP64 = 0, SYLVER_GB300_FP32 = 1 };

/* Same contract as spldlt_factorize; `precision` chooses FP64 factors or FP32
 * factors (FP32 arithmetic, FP64 pivot tests).  FP32 factors make
 * spldlt_solve refine in FP64 until the scaled backward error is <= ir_tol
 * (or ir_max_iter iterations). */
void spldlt_factorize_mixed(bool posdef, long const* ptr, int const* row, double const* val,
                            double* scale, void* akeep, void** fkeep,
                            sylver_options_t const* options, sylver_inform_t* inform,
                            int precision, double ir_tol, int ir_max_iter);

/* Device-resident variants: val_dev / x_dev are CUDA device pointers (same
 * layouts as the host calls).  Used when inputs already live in HBM. */
void spldlt_factorize_device(bool posdef, double const* val_dev, void* akeep, void** fkeep,
                             sylver_options_t const* options, sylver_inform_t* inform,
                             int precision, double ir_tol, int ir_max_iter);
void spldlt_solve_device(int job, int nrhs, double* x_dev, int ldx, void* akeep, void* fkeep,
                         sylver_options_t const* options, sylver_inform_t* inform);

/* Refinement statistics of the last solve on fkeep: iterations taken and the
 * final max-over-RHS scaled backward error.  Returns 0, or -1 for a null fkeep. */
int sylver_gb300_solve_stats(void const* fkeep, int* ir_iters, double* bwd_err);

/* Scaled backward error after each solve of the last refinement on fkeep
 * (first entry: after the initial solve); returns the number written
 * (at most max_entries), or -1 for a null fkeep. */
int sylver_gb300_solve_history(void const* fkeep, double* bwd_err, int max_entries);

/* Symbolic arrays of an analysis (1-based, reference layout).  Pass null for
 * any array not wanted; sizes: sptr/rptr/nptr nnodes+1, sparent nnodes,
 * rlist rptr[nnodes]-1, nlist 2*(nptr[nnodes]-1), perm n (1-based position). */
int sylver_gb300_akeep_sizes(void const* akeep, int* n, int* nnodes, long* rlist_len,
                             long* nlist_len);
int sylver_gb300_akeep_arrays(void const* akeep, int* sptr, int* sparent, long* rptr,
                              int* rlist, long* nptr, long* nlist, int* perm);

/* Scaling saved by a matching-based analysis (options.ordering = 2), user
 * order, n entries; returns n, or 0 when the analysis saved none.  No
 * reference counterpart (the reference keeps it in akeep%scaling). */
int sylver_gb300_akeep_scaling(void const* akeep, double* scale);

/* Pivot-order D^-1 of an LDL^T factorization (2 entries per pivot, the
 * reference's storage: 1x1 [d, 0], 2x2 [a, b, Inf, c]) and the pivot-order
 * permutation applied by delays; for tests.  Returns number of pivots. */
int sylver_gb300_fkeep_diag(void const* fkeep, double* d, int* piv_order);

/* Per-front sizes of an LDL^T factorization in front (postorder) order:
 * rows m (with delayed rows), fully-summed columns n (own plus delayed in)
 * and columns eliminated; any pointer may be null.  D^-1 and the pivot order
 * of sylver_gb300_fkeep_diag come front by front in this order, nelim
 * entries each.  Returns the number of fronts (0 for a Cholesky factor).
 * No reference counterpart; for tests. */
int sylver_gb300_fkeep_fronts(void const* fkeep, int* m, int* n, int* nelim);

/* Bytes of the factor storage in the factor precision: the front arena
 * (every front's block), or for an LDL^T factorization whose front blocks
 * would not fit in device memory the compact store of the fronts' factor
 * columns; with dst non-null and cap at least that size the storage is
 * copied there (host memory).  Returns the size, or -1 for a null fkeep.
 * No reference counterpart; for tests (bitwise reproducibility of the
 * factors). */
long sylver_gb300_fkeep_factor_bytes(void const* fkeep, void* dst, long cap);

/* The CUDA stream (cudaStream_t) all library work is issued on; callers that
 * time with CUDA events record them on this stream. */
void* sylver_gb300_stream(void);

/* Re-run the factorization held by fkeep with one CUDA event pair around
 * every launch (no graph) and accumulate per kernel kind:
 * 0 memset, 1 init-A, 2 extend-add (or the one-pass assembly that replaces all
 * three, kinds 0 and 1 then empty), 3 small fronts, 4 panel triangular solve,
 * 5 SIMT tile update, 6 diagonal-block Cholesky, 7 solve inverses, 8 tensor-core
 * panel split, 9 tensor-core update, 10 blocked diagonal block, 11 blocked panel
 * (Cholesky factorizations only).  ms[k] = total milliseconds, launches[k] =
 * count, flops[k] = algorithmic flops (update kernels: lower-triangle tile work).
 * Arrays hold 12 entries.  Returns 0 or a reference flag. */
int sylver_gb300_profile_factor(void* fkeep, double const* val_dev, double* ms, long* launches,
                                double* flops);

/* Re-run the Cholesky factorization held by fkeep launch by launch with CUDA
 * events (no graph) and add each launch's time to its level of the assembly
 * tree (leaves are level 0): level_ms[l] for l < number of levels (set-up
 * and the solve inverses are not counted).  Returns the number of levels, or
 * a reference flag (-10 when max_levels is too small).  The learned
 * scheduler trains on these per-level timings.  No reference counterpart. */
int sylver_gb300_profile_levels(void* fkeep, double const* val_dev, double* level_ms,
                                int max_levels);

/* Time one forward + backward sweep of the Cholesky factor held by fkeep for
 * nrhs (1..32) right-hand sides (zeros, in an internal buffer), launch by
 * launch with CUDA events and no graph, accumulated per kernel kind:
 * 0 small fronts forward, 1 small fronts backward (pivot rows), 2 + k for the
 * other launches (k: 0/1 gather forward/backward, 2/3 scatter forward/
 * backward, 4 diagonal block forward, 5 rows below forward, 6 rows below
 * backward, 7 diagonal block backward, 8 contribution rows backward, 9
 * contribution rows forward, 11/12 a level's block steps as one dataflow
 * launch forward/backward).  Arrays hold 16 entries.  Returns 0, or -98 for
 * an LDL^T factor or nrhs outside 1..32.  No reference counterpart. */
int sylver_gb300_profile_solve(void* fkeep, int nrhs, double* ms, long* launches);

/* Diagnostic: run the tensor-core (tcgen05, 3xBF16) contribution-block
 * update on a synthetic rows x k panel and report max|C - C_ref| / max|C_ref|
 * against an FP64 host product.  Returns 0 or a reference flag. */
int sylver_gb300_tc_selfcheck(int rows, int k, double* max_rel_err);

/* Diagnostic: the bounded wait of the dataflow solve sweep on a synthetic
 * one-task sweep.  starve != 0: the task waits on a counter nothing sets, so
 * the wait must give up (ST_TIMEOUT, 32, in *status) and the launch finish;
 * starve == 0: the counter is set first and *status must be 0.  *seconds:
 * the launch's wall time.  Faults and hangs nothing; changes no device
 * setting.  Returns 0 or a reference flag.  No reference counterpart. */
int sylver_gb300_dataflow_selftest(int starve, unsigned* status, double* seconds);

/* Diagnostic: the device's FP64 fused multiply-add rate in TFLOP/s, from one
 * timed launch of independent fma chains on every SM (CUDA events, after a
 * warm-up launch); the denominator of the FP64 path's roofline.  Changes no
 * device setting.  No reference counterpart. */
int sylver_gb300_fp64_fma_rate(double* tflops);

/* Counters of the last factorization on fkeep (kernel launches, levels). */
int sylver_gb300_fkeep_counters(void const* fkeep, long* kernel_launches, int* nlevels,
                                double* factor_ms);

/* No counterpart in the reference.  Allocation-free forward solve L y = b of
 * an existing factorization `tree` (an fkeep, or a tree from
 * spldlt_create_numeric_tree_dbl) with FP64 factors, for callers that cannot
 * let a library allocate device memory: applications whose own pool
 * allocator owns the device memory budget, or code that must not risk the
 * device-wide synchronisation of cudaMalloc/cudaFree.  x_dev is device
 * memory, ldx x nrhs, indexed in pivot order like spldlt_tree_solve_fwd_dbl;
 * `stream` is a cudaStream_t (null: the library stream); the call returns
 * after the solve completes.  Its only scratch is a fixed 16 MiB __device__
 * array in the library image: a level needing more than 2,097,152 doubles
 * (sum of the level's front rows x min(nrhs, 32)) returns
 * SYLVER_ERROR_X_SIZE.  The first call on a device looks up that array's
 * address.  The call waits for its stream before returning, so it is not
 * for use while that stream is being captured.  All calls share the array,
 * so calls that overlap on the GPU race.  Returns a reference flag. */
int spldlt_tree_solve_fwd_noalloc_dbl(bool posdef, void const* tree, int nrhs, double* x_dev,
                                      int ldx, void* stream);

/* ---- schedule (kernel-path choices; no reference counterpart) ------------ */

/* Kernel paths of the level schedule.  They select which kernels process a
 * front, never the arithmetic.  0 keeps the built-in default. */
typedef struct {
  int small_front_rows;  /* Cholesky: fronts with at most this many rows are factorised whole
                            by one CTA (capped at 96 FP64 / 128 FP32; default 96) */
  int tc_min_cb_rows;    /* FP32 Cholesky: contribution blocks with at least this many rows
                            use the tensor-core update (default 64; negative: never) */
  int solve_large_cols;  /* fronts with at least this many eliminated columns use the blocked
                            multi-CTA solve (default 96) */
  int ldlt_tpp_cols;     /* LDL^T: fronts with at most this many fully-summed columns skip the
                            a-posteriori block steps and use threshold partial pivoting only
                            (default 0: none) */
  int fs_panel_cols;     /* FP32 Cholesky: width of the outer panels in which the fully-summed
                            columns of large fronts are eliminated, a multiple of 64 up to 256
                            (default 64); the trailing fully-summed update after each panel
                            runs on the tensor cores.  Negative: 64-column steps with SIMT
                            updates throughout */
  int fs_panel_group;    /* FP32 Cholesky: outer panels per trailing fully-summed update, 1 to 8
                            (default 4).  Within a group each panel but the last updates only
                            the group's remaining columns; the columns past the group get one
                            tensor-core update with K = group x panel width */
  int front_memory;      /* front storage economy: 0 when needed (all front blocks would take
                            more than half of the device memory), 1 always, negative never.
                            Cholesky: contribution blocks given back to later fronts once the
                            parent's level has assembled them (each level zeroed just before it);
                            LDL^T: each level's factor columns copied to a compact store and
                            whole blocks given back (LDL^T always gives contribution blocks
                            back) */
  int solve_dataflow;    /* solves with FP32 factors: the block steps of a level's large fronts
                            as one launch of persistent CTAs that hand each step to the next
                            through counters, or one launch per block step.  0 (default):
                            dataflow for Cholesky, per-step launches for LDL^T (measured faster
                            there); positive: dataflow for both; negative: never */
} sylver_gb300_schedule_t;

/* Set the schedule used by factorizations planned afterwards (a new fkeep);
 * null restores the defaults.  Process-wide, not thread-safe. */
void sylver_gb300_set_schedule(sylver_gb300_schedule_t const* schedule);
void sylver_gb300_get_schedule(sylver_gb300_schedule_t* schedule);

/* ---- learned scheduler network (no reference counterpart) ---------------- */

/* MLP nin -> nhidden -> nhidden -> 1 (ReLU) on the GPU, FP32, used to
 * predict the log factorization time of a schedule from matrix features.
 * Parameters (flat): W1 (nhidden x nin), b1, W2 (nhidden x nhidden), b2,
 * W3 (1 x nhidden), b3.  Inputs are row-major batch x nin (host memory). */
void* sylver_gb300_mlp_create(int nin, int nhidden, unsigned seed);
void sylver_gb300_mlp_free(void* mlp);
long sylver_gb300_mlp_num_params(void const* mlp);
int sylver_gb300_mlp_set_params(void* mlp, float const* params);
int sylver_gb300_mlp_get_params(void const* mlp, float* params);
int sylver_gb300_mlp_forward(void* mlp, float const* x, int batch, float* y);
/* Mean-squared-error loss and its gradient (np entries) for one batch. */
int sylver_gb300_mlp_loss_grad(void* mlp, float const* x, float const* y, int batch,
                               float* loss, float* grad);
/* Full-batch Adam training for `epochs` steps; loss after the last step. */
int sylver_gb300_mlp_train(void* mlp, float const* x, float const* y, int batch, int epochs,
                           float lr, float* final_loss);

#ifdef __cplusplus
}
#endif
#endif /* SYLVER_GB300_H */
