/*
 * nasoq_gb300.h -- C ABI of the GB300 supernodal LDL^T (Bunch-Kaufman)
 * factorization, supernodal solves and GMRES refinement.
 *
 * Plain pointers and sizes only.  Host buffers stay owned by the caller;
 * device memory is owned by the plan.  Every function returns an int status
 * (NQG_OK == 0; negative values are errors, positive values are warnings),
 * mirroring the int returns of the reference API instead of exceptions.
 *
 * The C++ drop-in classes nasoq::SolverSettings and nasoq::Nasoq
 * (include/nasoq/QP/linear_solver_wrapper.h, include/nasoq/nasoq.h) are
 * implemented on top of these entry points.
 */
#ifndef NASOQ_GB300_H
#define NASOQ_GB300_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define NQG_OK 0
#define NQG_WARN_ZERO_PIVOT 1     /* factor finished; a pivot block was exactly singular */
#define NQG_WARN_NONFINITE 2      /* factor finished; a non-finite value appeared */
#define NQG_ERR_ARG (-1)          /* invalid argument */
#define NQG_ERR_CUDA (-2)         /* a CUDA call failed (no device, out of memory, ...) */
#define NQG_ERR_SYMBOLIC (-3)     /* ordering / supernode analysis failed */
#define NQG_ERR_STATE (-4)        /* call out of order (e.g. solve before factor) */
#define NQG_ERR_TIMEOUT (-5)      /* a bounded device-side wait gave up */
#define NQG_ERR_SIZE (-6)         /* problem exceeds a fixed capacity */

#define NQG_FP64 0                /* factor stored and computed in FP64 */
#define NQG_FP32 1                /* factor in FP32, refinement residuals in FP64 */

typedef struct nqg_settings {
  int precision;        /* NQG_FP64 or NQG_FP32 */
  int req_ref_iter;     /* GMRES restarts (reference SolverSettings::req_ref_iter) */
  int max_inner_iter;   /* GMRES inner steps (reference max_inner_iter) */
  double tol_abs;       /* GMRES absolute tolerance (reference tol_abs) */
  double tol_rel;       /* GMRES relative tolerance (reference tol_rel) */
  double reg_diag;      /* diagonal perturbation (reference reg_diag) */
  /* 1: |a_jj| < reg_diag -> a_jj = reg_diag, the refinement sees 0 there
   *    (reference find_perturbation / set_diags);
   * 0: a_jj += reg_diag on columns [0, perturb_plus_cols), a_jj -= reg_diag
   *    on the others, the refinement sees the unperturbed matrix (reference
   *    apply_perturbation / remove_perturbation / add_perturbation). */
  int regularization;
  int n_relax[3];       /* supernode relaxation (reference n_relax) */
  double z_relax[3];    /* supernode relaxation (reference z_relax) */
  /* FP32 factor only: diagonal entries smaller than this in magnitude are
   * replaced by +-reg_diag_fp32 (sign kept, 0 -> +) in the matrix that is
   * factored, bounding the element growth of block-restricted pivoting to
   * what FP32 can carry; the refinement still works on the reference's
   * matrix.  <= 0 selects 3e-5 * max|a_ij|. */
  double reg_diag_fp32;
  /* FP32 factor only: arithmetic of the triangular solves applied inside the
   * refinement.  NQG_FP64 (default) widens the factor entries and keeps the
   * solve vectors in FP64; NQG_FP32 runs the solves in FP32 (faster, and
   * enough when the refined residual still meets the tolerance; on
   * ill-conditioned systems it can stall the refinement earlier). */
  int solve_precision;
  /* regularization 0: number of leading columns perturbed by +reg_diag (the
   * reference's A->ncol: the Hessian block of a QP); < 0: every column. */
  int perturb_plus_cols;
} nqg_settings;

/* Reference defaults (src/QP/linear_solver_wrapper.cpp:205-244). */
void nqg_default_settings(nqg_settings *s);

/* Human-readable text of a status code. */
const char *nqg_status_str(int status);

/* ---- symbolic analysis (host only, no GPU needed) ----------------------- */
typedef struct nqg_symbolic nqg_symbolic;

typedef struct nqg_symbolic_info {
  int n, nsuper, max_sup_wid, max_col;
  int64_t ssize;        /* length of the row-list array */
  int64_t xsize;        /* number of factor values */
  double metis_seconds, total_seconds;
} nqg_symbolic_info;

/* Replaces symbolic_analysis_lin_solve (src/symbolic/symbolic_phase.cpp:167)
 * as called by SolverSettings::symbolic_analysis
 * (src/QP/linear_solver_wrapper.cpp:396-536): METIS ordering, etree,
 * column counts, weighted postorder, relaxed supernodes, supernodal row
 * structure.  A is lower-stored CSC (sorted, diagonal first).  extra_cols
 * (nullable, n ints) flags columns kept as single-column supernodes. */
int nqg_symbolic_create(int n, const int *Ap, const int *Ai, const int *extra_cols, const int n_relax[3],
                        const double z_relax[3], nqg_symbolic **out);
int nqg_symbolic_get_info(const nqg_symbolic *sym, nqg_symbolic_info *info);
/* Copies the arrays out (any pointer may be NULL).  Sizes: perm, iperm,
 * parent, colcount, col2sup, extra_cols: n; super: nsuper+1; sparent: nsuper;
 * lpi: nsuper+1 (row-list start per supernode); ls: ssize; colp: n+1 (value
 * offset per column, reference L->p). */
int nqg_symbolic_export(const nqg_symbolic *sym, int *perm, int *iperm, int *parent, int *colcount, int *super,
                        int *sparent, int *col2sup, int64_t *lpi, int *ls, int64_t *colp, int *extra_cols);
void nqg_symbolic_destroy(nqg_symbolic *sym);

/* ---- numeric plan (GPU) -------------------------------------------------- */
typedef struct nqg_plan nqg_plan;

typedef struct nqg_timings {
  double factor_ms, solve_ms, refine_ms;  /* last call, device time */
  int num_ref_iter;                        /* Arnoldi steps of the last refinement */
  int num_pivot_supernodes;                /* supernodes whose columns BK permuted */
  int num_2x2;                             /* 2x2 pivot blocks in the factor */
  double last_residual;                    /* preconditioned residual norm at exit */
} nqg_timings;

/* Symbolic analysis + device upload of the matrix (replaces
 * SolverSettings::symbolic_analysis, src/QP/linear_solver_wrapper.cpp:396).
 * A: lower CSC, n columns, values Ax; the perturbation rule of the settings
 * is applied to a private copy.  Allocates all device memory of the plan. */
int nqg_plan_create(int n, const int *Ap, const int *Ai, const double *Ax, const int *extra_cols,
                    const nqg_settings *settings, nqg_plan **out);
int nqg_plan_destroy(nqg_plan *plan);
/* Work on the given CUDA stream (cudaStream_t passed as void*; NULL = the
 * plan's own stream). */
int nqg_set_stream(nqg_plan *plan, void *stream);
/* Polls before a cross-CTA wait of this plan gives up (grid barriers and
 * pivot exchanges of the multi-CTA factorization, flag waits of the block
 * triangular solves); polls <= 0 restores the default (2^26).  A wait that
 * gives up makes the call return NQG_ERR_TIMEOUT; the plan stays usable.
 * The shared-memory barrier waits of the tensor-core kernels keep their
 * fixed bound.  Synchronizes the plan's stream. */
int nqg_set_wait_limit(nqg_plan *plan, long long polls);
int nqg_get_symbolic(const nqg_plan *plan, const nqg_symbolic **sym);

/* Replace all matrix values (same pattern as at creation); host buffer.
 * The perturbation rule is re-applied. */
int nqg_set_values(nqg_plan *plan, const double *Ax);
/* Overwrite `count` entries of the CSC value array (indices into Ax) in both
 * the factorization and the refinement copies of the matrix (the edit that
 * SolverSettings::add_del_matrix_qp applies to A_ord,
 * src/QP/linear_solver_wrapper.cpp:1020-1137). */
int nqg_edit_values(nqg_plan *plan, int count, const int64_t *idx, const double *vals);

/* Full numeric factorization (replaces ldl_left_sn_02_v2,
 * src/ldl/Serial_blocked_ldl_02_2.cpp:18-183, and the reorder_matrix that
 * follows it, src/QP/linear_solver_wrapper.cpp:1432-1460). */
int nqg_factor(nqg_plan *plan);
/* Partial refactorization of `count` supernodes, which must be closed under
 * "ancestor of a listed supernode" as the SoMod marking produces (replaces
 * update_ldl_left_sn_02_v2, src/ldl/Serial_update_ldl.cpp:18-277). */
int nqg_refactor(nqg_plan *plan, int count, const int *snodes);

/* Visibility masks for the masked solve of the QP mode (reference
 * visible_sn / extra_cols as passed to
 * solve_phase_ldl_blocked_parallel_permuted_update, src/linear_solver/
 * solve_phase.cpp:133-161).  NULL = everything visible. */
int nqg_set_visibility(nqg_plan *plan, const uint8_t *visible_sn, const uint8_t *hidden_col);

/* Solve K x = rhs with host buffers: permute, supernodal forward / diagonal /
 * backward solve, then GMRES refinement on the unperturbed matrix, unpermute
 * (replaces SolverSettings::solve_only, src/QP/linear_solver_wrapper.cpp:
 * 1300-1404, with pmgmres_ldlt_auto(_update), src/gmres/mgmres.cpp:1015-1421). */
int nqg_solve(nqg_plan *plan, const double *rhs, double *x);
/* Same with device buffers (n doubles each, may alias).  Both return
 * NQG_ERR_TIMEOUT when a wait of the block solves gave up (x is then not a
 * solution). */
int nqg_solve_device(nqg_plan *plan, const double *d_rhs, double *d_x);
/* Refinement only (reference SolverSettings::iterative_ref_only,
 * src/QP/linear_solver_wrapper.cpp:1406-1430): GMRES on K x = rhs,
 * preconditioned by the current factor, started from x = rhs; host buffers. */
int nqg_refine_only(nqg_plan *plan, const double *rhs, double *x);
/* Only the LDL^T solve of an ordered vector in place on the device
 * (reference solve_phase_ldl_blocked_parallel, src/linear_solver/
 * solve_phase.cpp:88-111). */
int nqg_ldlt_solve_ordered_device(nqg_plan *plan, double *d_x_ord);
/* y = K x in the original ordering with the unperturbed matrix, device
 * buffers (reference spmv_csc_sym_one_int, src/matrixVector/spmv_CSC.cpp:26). */
int nqg_spmv_device(nqg_plan *plan, const double *d_x, double *d_y);

int nqg_get_timings(const nqg_plan *plan, nqg_timings *t);
/* Copies the current factor to host buffers (any may be NULL): values
 * (xsize doubles), d (2n: diagonal, then 2x2 sub-diagonals), perm (n, the
 * combined fill-reducing + pivoting permutation), ls (ssize, row lists after
 * pivoting). */
int nqg_get_factor(const nqg_plan *plan, double *values, double *d, int *perm, int *ls);
/* Device error word of the last factor/solve (bit flags, 0 = clean). */
int nqg_get_device_status(const nqg_plan *plan, int *status_bits);

/* ---- measurement ----------------------------------------------------------
 * Kernel classes timed with CUDA events on the plan's stream when profiling
 * is on; alg_flops / alg_bytes are the algorithmic work of the launches
 * (useful multiply-adds x 2, and bytes of factor values that must be read). */
#define NQG_K_UPDATE 0          /* Schur updates between supernodes */
#define NQG_K_WIDE_PANEL 1      /* wide supernode: BK panel without pivot search */
#define NQG_K_WIDE_TRAILING 2   /* wide supernode: trailing update */
#define NQG_K_BK 3              /* narrow supernodes: BK + panel */
#define NQG_K_SOLVE 4           /* forward / backward supernodal solves */
#define NQG_K_SPMV 5            /* refinement residual SpMV */
#define NQG_K_OTHER 6           /* assembly, row renaming, vector kernels */
#define NQG_K_WIDE_PIVOT 7      /* wide supernode: BK panel with pivot search */
#define NQG_K_PACK 8            /* split-BF16 / split-TF32 operand packing of the tcgen05 updates */
#define NQG_K_CLASSES 9
typedef struct nqg_kernel_stats {
  long long launches;
  double total_ms;
  double alg_flops;
  double alg_bytes;
} nqg_kernel_stats;
int nqg_set_profiling(nqg_plan *plan, int on);
/* Accumulated since profiling was switched on (synchronizes the stream). */
int nqg_get_kernel_stats(nqg_plan *plan, int kernel_class, nqg_kernel_stats *stats);
/* Number of kernels this plan launched since creation. */
int nqg_get_launch_count(const nqg_plan *plan, long long *count);

/* ---- allocation-free dense factorization --------------------------------
 * No counterpart in the reference.  For callers that must not allocate GPU
 * memory once they are running (for example a real-time controller that
 * reserved its memory at start-up, or a host application whose device memory
 * is owned by another framework's allocator): Bunch-Kaufman LDL^T of one
 * dense nrow x w panel in caller device memory -- the w x w symmetric
 * diagonal block (lower triangle used) on top of nrow - w rows below it, the
 * same computation the factorization applies to each wide supernode.  On
 * return d_A holds L (unit diagonal, 2x2 sub-diagonals zeroed, the rows below
 * solved as L21), d_D the diagonal then the 2x2 sub-diagonals (2w doubles),
 * d_perm the pivot order (w ints, d_perm[m] = original column at position m).
 * Requires lda == nrow and nrow <= 8192 (else NQG_ERR_SIZE).  It calls no
 * cudaMalloc/cudaFree: its scratch is one fixed ~4.4 MB device array that
 * every GPU loading this library holds until the process exits, shared by
 * all calls, so calls whose GPU work overlaps (e.g. on two streams) race.
 * Every call looks up that array's device address (cudaGetSymbolAddress,
 * which allocates nothing), so a device reset between calls is safe.  Work
 * runs on `stream` (NULL = default stream); the call is synchronous: it waits
 * for that work and reads the status word back before it returns. */
int nqg_dense_ldlt_noalloc(int nrow, int w, double *d_A, int lda, double *d_D, int *d_perm, void *stream);

/* ---- QP solve (dual active-set NASOQ over the GPU LBL) ------------------- */
typedef struct nqg_qp_settings {
  int variant;          /* 0 Fixed, 1 AUTO, 2 Tuned, 3 PREDET (reference nasoq_mode) */
  double eps_abs;       /* KKT tolerance (reference Nasoq::eps_abs) */
  double diag_perturb;  /* KKT regularization (reference diag_perturb) */
  double stop_tol;      /* refinement tolerance (reference stop_tol) */
  int max_iter;         /* refinement iterations (reference max_iter) */
  int max_iter_nas;     /* active-set iteration cap (reference max_iter_nas) */
  int precision;        /* NQG_FP64 or NQG_FP32 factorization */
  /* > 0: rounds of Ruiz equilibration of H, A, B, q, a, b before the solve,
   * undone on the data and the solution after it (reference Nasoq::scaling,
   * src/nasoq.cpp:662-703); 0: none.  Single-problem solver only: the
   * batched solver rejects a nonzero value. */
  int scaling;
} nqg_qp_settings;

typedef struct nqg_qp_result {
  int status;           /* reference nasoq_status: 1 Optimal, 2 Inaccurate, 3 NotConverged, 0 Infeasible */
  int num_iter, active_size;
  double objective, primal_obj, dual_obj;
  double lag_res, cons_sat_norm, non_negativity_infn, complementarity_infn;
  double total_seconds, factor_seconds;
} nqg_qp_result;

/* Defaults of the reference Nasoq object (src/nasoq.cpp:163-182). */
void nqg_qp_default_settings(nqg_qp_settings *s);
/* min 1/2 x'Hx + q'x  s.t.  A x = a,  B x <= b.  H: n-by-n lower CSC (diagonal
 * first); A: meq-by-n CSC; B: mineq-by-n CSC (A/B pointers may be NULL when
 * their row count is 0).  Outputs x (n), y (meq equality duals), z (mineq
 * inequality duals), active_set (mineq ints, first result->active_size used).
 * Replaces Nasoq(...) + Nasoq::solve() (src/nasoq.cpp:95-160, 656-710).
 * With warm-start arrays (x0, z0, y0 and a list of n_as active constraints,
 * all non-NULL) it replaces symbolic_QP + set_warm_start + numeric_QP
 * (src/nasoq.cpp:413-436, 741-762). */
int nqg_qp_solve(int n, const int *Hp, const int *Hi, const double *Hx, const double *q, int meq, const int *Ap,
                 const int *Ai, const double *Ax, const double *a, int mineq, const int *Bp, const int *Bi,
                 const double *Bx, const double *b, const nqg_qp_settings *settings, const double *x0,
                 const double *z0, const double *y0, int n_as, const int *as0, double *x, double *y, double *z,
                 int *active_set, nqg_qp_result *result);

/* ---- batched QP solve ------------------------------------------------------
 * Many small QPs (min 1/2 x'Hx + q'x  s.t.  Ax = a, Bx <= b) solved together
 * on the GPU by the reference's dual active-set method (Nasoq::solve,
 * src/nasoq.cpp:656-710, with numeric_QP :478-610): one CTA of a persistent
 * kernel runs one problem's whole active-set iteration -- partial
 * refactorizations, masked solves, refinement, step lengths and active-set
 * edits -- on the device, with no host round trip per iteration.  Problems
 * are grouped by sparsity pattern; each pattern gets one symbolic analysis
 * (the reference's ordering and supernodes).  The reference has no working
 * batch path (its numeric_QP_batch, src/nasoq.cpp:1540, is unfinished); per
 * problem the semantics are those of nqg_qp_solve. */
typedef struct nqg_batch nqg_batch;

typedef struct nqg_batch_settings {
  nqg_qp_settings qp;   /* variant (Fixed, AUTO or PREDET), eps_abs, ...; qp.precision: NQG_FP64 or NQG_FP32
                           factorization and triangular solves (FP64 refinement either way) */
  int refine;           /* 0: the reference's GMRES schedule (restarts x steps from the variant);
                           1: adaptive flexible GMRES to refine_tol */
  double refine_tol;    /* refine == 1: stop once ||b - Kx||_2 <= refine_tol * ||b||_2 */
  int threads;          /* CTA size, a multiple of 32 up to 256 (0: 128) */
  int use_graph;        /* 1: the queue resets and the kernels are replayed from a captured CUDA graph */
  int stage;            /* 1: a problem's factor and row lists stay in shared memory when they fit
                           (problems grouped into shared-memory tiers, one launch per tier) */
  int share_factor;     /* 1 (default): problems with identical matrices (same H, A, C values, e.g. a
                           parametric family whose q / b / d change) share the factorization with every
                           inequality hidden, computed once at finalize; each solve starts from a copy
                           and refactors only the paths of its active rows.  0: every solve factors its
                           own KKT matrix from scratch. */
} nqg_batch_settings;

typedef struct nqg_batch_stats {
  int status, num_iter, active_size, flags;  /* flags: NQG_WARN_* bits of the device status */
  int refine_steps, solves, warm_dropped, pad;  /* Krylov steps, KKT solves, warm-start rows dropped */
  double objective, lag_res, cons_sat_norm, non_negativity_infn, complementarity_infn;
} nqg_batch_stats;

typedef struct nqg_batch_info {
  int nprob, npatterns, grid, threads, blocks_per_sm;
  int warp_factor;      /* 1: small supernodes factored a warp each, level by level */
  int64_t smem_bytes, slot_bytes;
  double last_ms;       /* device time of the last nqg_batch_solve */
} nqg_batch_info;

/* Defaults: the reference's Nasoq defaults with eps_abs = 1e-8, FP64, the
 * reference's refinement schedule, CUDA graph on. */
void nqg_batch_default_settings(nqg_batch_settings *s);
int nqg_batch_create(const nqg_batch_settings *s, nqg_batch **out);
/* Adds one QP (same arrays as nqg_qp_solve); returns its index (>= 0). */
int nqg_batch_add(nqg_batch *b, int n, const int *Hp, const int *Hi, const double *Hx, const double *q, int meq,
                  const int *Ap, const int *Ai, const double *Ax, const double *a, int mineq, const int *Bp,
                  const int *Bi, const double *Bx, const double *bineq);
/* Groups by pattern, analyses each pattern, uploads; no problem can be added afterwards. */
int nqg_batch_finalize(nqg_batch *b);
/* New q / a / b of every problem, concatenated in problem order (NULL: unchanged). */
int nqg_batch_set_vectors(nqg_batch *b, const double *q_all, const double *a_all, const double *b_all);
/* The same, enqueued on the batch's stream without waiting: ordered before
 * the next solve on that stream.  Arrays in page-locked memory are copied
 * asynchronously and must stay unchanged until the stream has passed the
 * copies (e.g. until the next nqg_batch_get_all); pageable arrays are staged
 * before the call returns. */
int nqg_batch_set_vectors_async(nqg_batch *b, const double *q_all, const double *a_all, const double *b_all);
/* Proposed active set of problem i for the next solve (n_as < 0: cold start).
 * The solve factors the KKT system with these constraints active, drops the
 * ones whose multipliers come out negative (up to three rounds, then a cold
 * start), and continues the active-set iteration from there (the role of the
 * reference's set_warm_start, src/nasoq.cpp:413-436). */
int nqg_batch_set_warm_start(nqg_batch *b, int i, int n_as, const int *as);
/* Warm-start sets of every problem from device-resident scores (row i, ld
 * floats apart: one score per inequality of problem i, e.g. the logits of an
 * nqg_mlp): each problem proposes its constraints scoring above `threshold`,
 * skipping one parallel to a constraint already proposed (the two sides of a
 * box); a problem without proposal starts cold.  Enqueued on the batch's
 * stream. */
int nqg_batch_warm_start_from_scores(nqg_batch *b, const float *d_scores, int ld, float threshold);
/* Every problem back to a cold start. */
int nqg_batch_clear_warm_starts(nqg_batch *b);
/* Solves every problem; returns when done. */
int nqg_batch_solve(nqg_batch *b);
/* Enqueues the solve on the batch's stream (nqg_batch_get_stream) and returns. */
int nqg_batch_solve_async(nqg_batch *b);
int nqg_batch_get(nqg_batch *b, int i, double *x, double *y, double *z, int *active_set, nqg_qp_result *res);
int nqg_batch_get_all(nqg_batch *b, double *x_all, double *y_all, double *z_all, nqg_batch_stats *stats);
int nqg_batch_get_info(const nqg_batch *b, nqg_batch_info *info);
int nqg_batch_get_stream(const nqg_batch *b, void **stream);
/* Per-phase SM-cycle counters of the solves (summed over problems), for
 * profiling: on = 1 enables them for the next solves.  get_profile copies up
 * to n counters and resets them: [0] total, [1] set-up and first solve,
 * [2] partial refactorizations, [3] triangular-solve applications, [4] SpMVs,
 * [5] refinement (solves included), [6] entering-constraint selection,
 * [7] steps and edits, [8] supernodes factored, [9] active-set iterations,
 * and inside [3]: [10] forward sweeps of wide levels, [11] of narrow levels,
 * [12] diagonal solves, [13] backward sweeps, [14] gathers and scatters;
 * inside [1]: [15] the factorizations of the set-up rounds (a shared
 * factorization's copy and the active rows' refactorization included);
 * every supernode factorization split into [16] assembly, [17] descendant
 * updates, [18] Bunch-Kaufman, [19] rows below, [20] inverse of the
 * diagonal block, [21] stores; [22] pivot renaming after a factorization. */
int nqg_batch_set_profiling(nqg_batch *b, int on);
int nqg_batch_get_profile(nqg_batch *b, unsigned long long *counters, int n);
const char *nqg_batch_last_error(const nqg_batch *b);
int nqg_batch_destroy(nqg_batch *b);

/* ---- active-set model (learned warm start) ----------------------------------
 * No counterpart in the reference (its warm-start entry, Nasoq::set_warm_start,
 * src/nasoq.cpp:413-436, takes a given set).  A multilayer perceptron theta ->
 * one logit per inequality of a parametric QP family (ReLU hidden layers,
 * BF16 weights with FP32 master copies, FP32 accumulation), trained on the
 * GPU by its own forward / backward kernels with Adam on a weighted sigmoid
 * cross-entropy; its logits feed nqg_batch_warm_start_from_scores.
 * sizes[0] inputs, sizes[1 .. nsizes-2] hidden widths, sizes[nsizes-1]
 * outputs; weights row-major (out x in), layer after layer. */
typedef struct nqg_mlp nqg_mlp;
int nqg_mlp_create(int nsizes, const int *sizes, unsigned long long seed, nqg_mlp **out);
int nqg_mlp_num_params(const nqg_mlp *m, long *n_weights, long *n_biases);
int nqg_mlp_set_weights(nqg_mlp *m, const float *w_all, const float *b_all);
int nqg_mlp_get_weights(nqg_mlp *m, float *w_all, float *b_all);
int nqg_mlp_forward(nqg_mlp *m, int rows, const float *x, float *logits);
/* Device buffers, enqueued on `stream` (NULL: the model's own stream, and the
 * call waits).  The model's activation buffers serve every call: forwards of
 * one model on different streams must not overlap (use one model per stream). */
int nqg_mlp_forward_device(nqg_mlp *m, int rows, const float *d_x, float *d_logits, void *stream);
int nqg_mlp_loss_grad(nqg_mlp *m, int rows, const float *x, const float *y, float pos_weight, double *loss,
                      float *gw_all, float *gb_all);
int nqg_mlp_set_data(nqg_mlp *m, int n, const float *x, const float *y);
int nqg_mlp_train(nqg_mlp *m, int epochs, int batch, float lr, float pos_weight, unsigned long long seed,
                  double *epoch_loss);
const char *nqg_mlp_last_error(const nqg_mlp *m);
int nqg_mlp_destroy(nqg_mlp *m);

/* ---- SMP QP files (reference smp-format) -------------------------------- */
/* A QP read from an SMP file (reference SMP::load, smp-format/smp_format.h:
 * 174-233) and converted to  min 1/2 x'Hx + q'x  s.t.  A x = b, C x <= d
 * (QPFormatConverter::smp_to_ie, smp-format/mp_format_converter.h:681-712):
 * rows l <= c'x <= u become c'x <= u and/or -c'x <= -l, infinite sides
 * (|bound| = 1e20) dropped, in row order (find_inequalities_by_bounds,
 * :264-433).  H is lower-stored with a zero diagonal in empty columns.
 * Host only; no GPU needed. */
typedef struct nqg_qp_data nqg_qp_data;
/* Returns NQG_OK, or NQG_ERR_ARG for an unreadable or invalid file; *out is
 * set either way (nqg_qp_data_error explains a failure) and must be freed
 * with nqg_qp_data_destroy. */
int nqg_smp_load(const char *path, nqg_qp_data **out);
const char *nqg_qp_data_error(const nqg_qp_data *qp);
/* n, equality rows, inequality rows; nnz[3] = entries of H, A, C. */
int nqg_qp_data_sizes(const nqg_qp_data *qp, int *n, int *meq, int *mineq, int64_t *nnz);
/* CSC arrays (H lower, A meq x n, C mineq x n) and vectors; any may be NULL. */
int nqg_qp_data_export(const nqg_qp_data *qp, int *Hp, int *Hi, double *Hx, double *q, int *Ap, int *Ai, double *Ax,
                       double *b, int *Cp, int *Ci, double *Cx, double *d);
/* The constant objective term, the stated optimum and the stated solution
 * (counts 0 when the file holds none); any pointer may be NULL. */
int nqg_qp_data_extras(const nqg_qp_data *qp, double *fixed, double *optimal_obj, int *n_primals, double *primals,
                       int *n_duals, double *duals);
const char *nqg_qp_data_description(const nqg_qp_data *qp);
int nqg_qp_data_destroy(nqg_qp_data *qp);

#ifdef __cplusplus
}
#endif
#endif
