// Drop-in nasoq::SolverSettings: the LBL solver object of the reference
// (include/nasoq/QP/linear_solver_wrapper.h:53-306) with the same public
// fields and methods.  symbolic_analysis() runs the host analysis and creates
// a GPU plan (include/nasoq_gb300.h); numerical_factorization(),
// update_factorization() and solve_only() run on the GPU.
#ifndef NASOQ_GB300_LINEAR_SOLVER_WRAPPER_H
#define NASOQ_GB300_LINEAR_SOLVER_WRAPPER_H

#include <chrono>
#include <vector>

#include "nasoq/common/def.h"

struct nqg_plan;

namespace nasoq {

enum solve_type { FULL = 0, REFACTOR = 1, UPDATE = 2, SOLVE = 3 };

struct profiling_solver_info {
  std::chrono::time_point<std::chrono::system_clock> start, end;
  std::chrono::duration<double> elapsed_seconds;
  double fact_time, analysis_time, solve_time, iter_time, ordering_time;
  double update_time;
  double piv_reord;
  double *timing_chol;
  profiling_solver_info(int nt);
  profiling_solver_info(int nt, double ft, double at, double st, double it, double ot, double ut, double pr);
  ~profiling_solver_info();
  std::chrono::time_point<std::chrono::system_clock> tic();
  std::chrono::time_point<std::chrono::system_clock> toc();
  double elapsed_time(std::chrono::time_point<std::chrono::system_clock> beg,
                      std::chrono::time_point<std::chrono::system_clock> lst);
  void print_profiling();
};

struct perturbed_value {
  double per_value;
  int col_idx;
};

struct SolverSettings {
  int solver_mode;  // 0: plain solve, 1: QP mode with row/column edits
  BCSC *L;
  double *valL, *d_val, *x, *rhs;
  CSC *A, *SM;
  CSC *AorSM;
  CSC *A_ord, *AT_ord;
  CSC *B, *BT;
  CSC *C, *CT;
  size_t dim1;
  size_t base;
  int *perm_piv, *pinv;
  int a_consistent;
  int ldl_variant, ldl_update_variant;
  double *sm_rhs, *sm_solution;
  int *l_pb, *l_pe, *l_i;
  double *l_x;
  int is_super, simplicial_alloc;
  size_t ws_int_size;
  size_t ws_dbl_size;
  int n_level, n_par;
  int *level_ptr, *level_set, *par_ptr, *par_set;
  int n_level_s, n_par_s;
  int *level_ptr_s, *par_ptr_s, *par_set_s;
  int *s_level_ptr, *s_level_set;
  int s_level_no;
  int *prune_ptr, *prune_set;
  int *extra_cols;
  int n_relax[3];
  double z_relax[3];
  int max_sup_wid, max_col, status = 0;
  int ordering_type;
  int *atree, *etree, *etree_mod;
  int *visible_cnt;
  int *child_ptr, *child_no, *num_child;
  int *child_sn_ptr, *child_sn_no, *num_sn_child;
  std::vector<std::vector<int>> children_vec;
  std::vector<int> detached_nodes;
  int col_del, to_del;
  double reg_diag;
  int num_pivot;
  int max_iter, max_inner_iter;
  int num_ref_iter;
  int req_ref_iter;
  double tol_abs, tol_rel;
  std::vector<perturbed_value> perturbed_diags;
  int regularization;
  int cost_param, level_param, final_seq_node;
  int chunk, num_thread, thread_thresh;
  profiling_solver_info *psi;
  std::vector<int> modified_sns;
  bool *marked, *visible_sn;
  double *ws;
  double *ws_zeroed;
  int *ws_int;
  double *extra_rhs;
  int remove_trans;
  double A_l1, x_l1, rhs_l1, res_l1;
  double bwd_err;

  // ---- GPU-specific (not in the reference header)
  int gpu_precision;          // 0: FP64 factor (default), 1: FP32 factor and solves + FP64 flexible GMRES
  nqg_plan *plan;             // device plan, created by symbolic_analysis()
  std::vector<std::vector<long long>> const_val_idx;  // QP mode: SM value index of every entry of each constraint
  int last_gpu_status;        // status of the last C-ABI call
  bool own_simplicial;        // l_pb / l_pe / l_i allocated by convert_supernode_to_simplicial()

  SolverSettings(CSC *Amat, double *rhs_in);
  SolverSettings(CSC *Amat, double *rhs_in, CSC *Bmat);
  SolverSettings(CSC *Amat, double *rhs_in, CSC *Bmat, double *b);
  SolverSettings(CSC *Amat, double *rhs_in, CSC *Bmat, CSC *BTmat);
  SolverSettings(CSC *Amat, double *rhs_in, CSC *Bmat, CSC *BTmat, CSC *Cmat, CSC *CTmat);
  ~SolverSettings();

  void default_setting();
  int build_super_matrix();
  void find_perturbation(double tol);
  // +tol on the diagonals of the first A->ncol columns of AorSM, -tol on the
  // rest (host values; the plan applies the same rule when regularization != 1)
  void apply_perturbation(double tol);
  // the same on the host ordered copy A_ord (the plan factors the perturbed
  // matrix and refines with the unperturbed one by itself)
  void add_perturbation(double tol);
  void remove_perturbation(double tol);
  int symbolic_analysis();
  void reset_symbolic_factor();
  // level sets of the supernodal tree (s_level_*) when num_thread > thread_thresh
  void architecture_related_params();
  // host workspaces ws / ws_int / ws_zeroed, with the reference's sizes
  void allocate_workspace();
  int numerical_factorization();
  int delete_node_tree_simple(int k);
  int add_node_tree_simple(int k);
  void bfs_tree(int cur_sn);
  // column-tree variants (etree_mod / child_ptr / child_no, built on first use)
  int delete_node_tree(int k);
  int add_node_tree(int k);
  int add_del_matrix_qp(int add_del, std::vector<int> add_drp_const);
  int update_somod(std::vector<int> add_drp_const, const int n_rhs, const double *new_rhs);
  int downdate_somod(std::vector<int> add_drp_const, int n_rhs);
  int update_factorization();
  // placeholders with the reference's return values (1, 1, NULL, 1, NULL)
  int edit_matrix();
  int edit_rhs();
  double *edit_solve_rhs();
  int edit_update_factorization(int add_del, std::vector<int> add_drp_const);
  double *update_solve();
  double *solve_only();
  double *solve_only(const int n_rhs, double *rhs_in);
  // refinement alone, started from x = rhs (x returned)
  double *iterative_ref_only();
  // brings L->Perm / L->IPerm and A_ord up to the permutation of the last
  // factorization (the GPU folds the pivots into it while factoring)
  void reorder_matrix();
  void compute_norms();
  double backward_error();
  // column pointers / row indices of the factor in simplicial form (l_pb, l_pe, l_i)
  void convert_supernode_to_simplicial();
  void copy_lsuper_to_l();
  void set_diags(double d);
  // downloads the factor; 1 when every value is finite and the permutation is one
  int check_ldlt_factor();
  // Copies the GPU factor into valL / d_val and the current permutation into
  // L->Perm / L->IPerm (host buffers owned by this object).
  int download_factor();
};

}  // namespace nasoq
#endif
