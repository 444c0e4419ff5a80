// Device layout of the batched QP solver (batch.cu): many small QPs solved by
// NASOQ's dual active-set method (reference src/nasoq.cpp:478-610) in one
// persistent kernel, one CTA per QP, with no host round trip per iteration.
//
// Problems are grouped by sparsity pattern.  Each distinct pattern of the
// super-KKT matrix [H A^T C^T; A 0 0; C 0 0] (reference
// SolverSettings::build_super_matrix, src/QP/linear_solver_wrapper.cpp:246)
// gets one host symbolic analysis (the same ordering and supernodes as the
// reference) and one set of integer work lists; every problem of the pattern
// only brings its values.  All integer arrays of all patterns live in one
// pool and are addressed by the offsets below.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace nqg {

constexpr int BATCH_MR_CAP = 10;  // largest number of Krylov steps per restart
constexpr int BATCH_PROFILE_COUNTERS = 24;

struct BPat {
  int n, meq, mineq, N, base;  // N = n + meq + mineq; base = n + meq (first constraint column)
  int ns, nlev, xsize, ssize, nnzK, nnzR, max_w, max_nr;
  // int-pool offsets
  int o_super;     // ns+1   first (ordered) column of each supernode
  int o_sparent;   // ns     supernodal elimination tree (-1 at roots)
  int o_col2sup;   // N      ordered column -> supernode
  int o_lpi;       // ns+1   start of each supernode's row list
  int o_lpx;       // ns+1   start of each supernode's values (column-major nrow x w)
  int o_ls0;       // ssize  row lists of the analysis (ordered indices, sorted)
  int o_perm0;     // N      fill-reducing order: perm0[c] = original column at position c
  int o_lvl_ptr;   // nlev+1 supernodes grouped by tree level (leaves first)
  int o_lvl_sn;    // ns
  int o_lev;       // ns     tree level of each supernode
  int o_pair_ptr;  // ns+1   descendants of every supernode (elimination-tree reach): descendants
  int o_pair_mid;  // ns     that never hide first, then the constraint columns (from pair_mid[s])
  int o_pair_d, o_pair_lb, o_pair_ub;  // per pair: descendant, first / last row of it inside the target
  int o_Rp, o_Rj, o_Rq;  // full symmetric CSR of K (original numbering); Rq = index of the lower-CSC value
  int o_ent;       // nnzK   per lower-CSC value: constraint k of an entry in constraint row k (>= 0),
                   //        -2-col for the diagonal of column col, -1 otherwise
  int o_bt_ptr, o_bt_var, o_bt_q;  // per constraint: its variables and the lower-CSC value index of each entry
  int o_bt_rpos;   // per constraint entry: its position in the CSR row of its variable
  int o_sn_con;    // ns     constraint whose (single) column a supernode holds, -1 otherwise
  int o_con_sn;    // mineq  supernode of each constraint column
  int o_eq_ptr, o_eq_var, o_eq_q;  // per equality row: its variables and value indices
  int o_snrec;     // 8 ints per supernode: c0, w, nrow, value offset, row-list offset, pair start, pair_mid, pair end
  int o_prec;      // 4 ints per pair: descendant, lb, ub, descendant's row-list offset
  int o_con_ptr, o_con_tgt;  // per constraint: (target supernode, bit) of every pair whose descendant is its column
  int o_sn_big;    // ns bytes (packed in ints): 1 where a warp solves the supernode (w > 4 or nrow * w > 64)
  int cmask_ok;    // every supernode has at most 64 constraint-column descendants (bit masks apply)
};

// One QP of the batch: where its values are, its derived settings, and where
// its results go.
struct BProb {
  int pat;
  int outer, inner;          // refinement restarts x inner steps
  int max_iter_nas;
  int ws_n;                  // warm start: size of the proposed active set (-1: cold start)
  int base;                  // group of problems with identical K (shared cold factorization), -1: none
  int64_t o_kv;              // nnzK values of K (original, every constraint entry present)
  int64_t o_pert;            // N bytes: diagonal replaced by the regularization
  int64_t o_q, o_b, o_d;     // n, meq, mineq
  int64_t o_x, o_y, o_z;     // n, meq, mineq (results; warm start in)
  int64_t o_as;              // mineq ints: final active set (insertion order); warm-start set in
  double reg, zero_thresh, eps_abs, tol_abs, tol_rel;
  double reg32;              // FP32 factor: sign-keeping floor of its diagonal (3e-5 max |k_ij|)
};

// Results of one QP (reference Nasoq fields of the same names).
struct BResult {
  int status;        // nasoq_status: 1 Optimal, 2 Inaccurate, 3 NotConverged, 0 Infeasible
  int num_iter, active_size, flags;  // flags: device status bits (zero pivot, non-finite)
  int refine_steps, solves, warm_dropped, pad;
  double objective, primal_obj, dual_obj;
  double lag_res, cons_sat_norm, non_negativity_infn, complementarity_infn;
};

// Per-CTA scratch: one problem at a time, sized for the largest pattern.
struct BSlot {
  int64_t o_L, o_D, o_ls, o_perm, o_iperm, o_lperm, o_mark, o_piv, o_alist, o_vlist, o_mlist;
  int64_t o_Fv, o_Rv;  // factorization / refinement values of K in CSR order (inactive rows zeroed)
  int64_t o_cmask;     // per supernode: bit mask of its active constraint-column descendants
  int64_t o_rhs, o_sol, o_r, o_w, o_V, o_Z, o_tmp;
  int64_t bytes;
};

struct BArgs {
  const BPat *pats;
  const BProb *probs;
  const int *ipool;
  const double *dpool;       // problem values and vectors (BProb offsets)
  double *dout;              // problem results (x, y, z)
  int *iout;                 // active sets
  BResult *res;
  const int *order;          // queue order of the problems
  int *head;                 // work-queue counter (reset before every launch)
  int nprob;
  unsigned char *slots;      // per-CTA scratch
  BSlot slot;                // layout of one slot
  int refine;                // 0: reference GMRES schedule, 1: adaptive flexible GMRES
  double refine_tol;         // adaptive: relative residual target
  int mr_max;                // capacity of the Krylov arrays
  int N_max, w_max, nr_max, ns_max, mi_max, nlev_max;  // shared-memory sizing
  unsigned long long *prof;  // per-phase SM cycles summed over CTAs, or null
  int stage_bytes;           // shared memory for the factor and row lists of problems that fit
  int warp_factor;           // level-parallel factorization, a warp per supernode of <= 32 x 32
  // Problems with identical matrix values (same pattern, values,
  // regularization) share the factorization with every inequality hidden: a
  // launch with mode = 1 computes it once per group into `bases` (one slot
  // layout each, for problem base_rep[g]); mode = 0 starts every member from
  // a copy of it and refactors only the paths of its warm-start rows.
  unsigned char *bases;
  const int *base_rep;
  int nbase;
  int mode;
};

size_t batch_smem_bytes(const BArgs &a, size_t tsize);
int batch_ws_from_scores(int nprob, BProb *probs, const BPat *pats, const int *ipool, const double *dpool, int *iout,
                         const float *scores, int ld, float thr, cudaStream_t st);
int batch_ws_clear(int nprob, BProb *probs, cudaStream_t st);
// Copies stacked q / b / d (offsets per problem in voff[3 i + 0..2], -1: not
// given) from a staging buffer into the value pool.
int batch_scatter_vectors(int nprob, const BProb *probs, const BPat *pats, const int64_t *voff, const double *stage,
                          double *dpool, cudaStream_t st);
template <class T> int batch_prepare(int threads, size_t smem_attr, size_t smem, int *blocks_per_sm);
template <class T> int launch_batch(const BArgs &a, int grid, int threads, size_t smem, cudaStream_t st);

}  // namespace nqg
