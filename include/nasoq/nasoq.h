// Drop-in nasoq::Nasoq: the dual active-set QP solver of the reference
// (include/nasoq/nasoq.h:26-493) for
//     min 1/2 x'Hx + q'x   s.t.   A x = a,  B x <= b
// with the same constructors, settings fields, solve() entry points and
// result fields.  Every KKT factorization, partial refactorization and solve
// of the active-set loop runs on the GPU through nasoq::SolverSettings.
#ifndef NASOQ_GB300_NASOQ_H
#define NASOQ_GB300_NASOQ_H

#include <chrono>
#include <string>
#include <vector>

#include "nasoq/QP/linear_solver_wrapper.h"
#include "nasoq/QP/qp_utils.h"
#include "nasoq/common/def.h"

namespace nasoq {

struct QPSettings {
  double eps;
  double eps_primal, eps_dual, eps_slack, eps_nn;
  double diag_perturb;
  int batch_size;
  double eps_rel;
  int scaling;
  double zero_thresh;
  int inner_iter_ref;
  int outer_iter_ref;
  int max_iter;
  double stop_tol;
  int max_iter_nas;
  std::string nasoq_variant;
  QPSettings();
};

enum nasoq_mode { Fixed = 0, AUTO, Tuned, PREDET };

enum nasoq_status { Optimal = 1, Inaccurate = 2, NotConverged = 3, Infeasible = 0, NotFinished = 4 };

struct nasoq_config {
  int inner_iter, outer_iter;
  double pert_diag, stop_tol;
  nasoq_config(int a, int b, double c, double d);
};

struct qp_info {
  std::chrono::time_point<std::chrono::system_clock> tot_st, tot_end;
  std::chrono::time_point<std::chrono::system_clock> fct_st, fct_end;
  std::chrono::time_point<std::chrono::system_clock> ini_st, ini_end;
  bool sw;
  std::chrono::duration<double> elapsed_seconds;
  double tot;
  double factt, init;
  int num_update, num_downdate, num_refactor, num_solve;
  qp_info();
  std::chrono::time_point<std::chrono::system_clock> tic();
  std::chrono::time_point<std::chrono::system_clock> toc();
  double elapsed_time(std::chrono::time_point<std::chrono::system_clock> beg,
                      std::chrono::time_point<std::chrono::system_clock> lst);
  void print();
};

struct Nasoq {
  std::string sol_name;
  int hessian_size, eq_const_size, ineq_const_size;
  CSC *H, *HT, *A, *AT, *B, *BT;
  double *q, *a, *b;
  int n_active;
  double diag_perturb, zero_thresh, eps_abs, eps_rel;
  double primal_obj, dual_obj, objective;
  double non_negativity_infn, complementarity_infn;
  int inner_iter_ref, outer_iter_ref, max_iter;
  double stop_tol;
  int *eTree;
  int *col2const, *const2col;
  CSC *sKKT, *sKKTt;
  double *sKKTrhs;
  int *etree;
  int *pinv;
  int *col2sup;
  size_t skkt_col;
  int scaling;              // > 0: Ruiz equilibration steps; < 0: single scalar scaling
  double *D, *E, *F, *Dinv, *Einv, *Finv;
  double c, cinv;
  double *rec_length;
  double *dual_vars, *dual_vars_eq;
  double *primal_vars;
  double *kkt_solution, *lagrange_mult, *lagrange_mult_eq, *descent;
  std::vector<int> active_set;
  int *as0;
  int is_converged;
  int num_iter, max_iter_nas;
  int used_constraints, num_active;
  int *used_const;
  int auto_reg_en;
  int warm_start;
  int batch_size;
  double *workspace;
  double qp_scalar, inv_qp_scalar;
  nasoq_mode variant;
  nasoq_status ret_val;
  SolverSettings *ss;
  qp_info *qi;
  double *dual_FB_a, *dual_FB_b, *dual_FB;
  double *primal_FB_a, *primal_FB_b, *primal_FB;
  double lag_res, cons_sat_norm;
  // GPU-specific (not in the reference header): 0 FP64 factor, 1 FP32 factor
  int gpu_precision;

  Nasoq(size_t H_size, int *Hp, int *Hi, double *Hx, double *q_in, size_t B_row, size_t B_col, int *Bp, int *Bi,
        double *Bx, double *b_ineq);
  Nasoq(size_t H_size, int *Hp, int *Hi, double *Hx, double *q_in, size_t A_size1, size_t A_size2, int *Ap, int *Ai,
        double *Ax, double *a_eq, size_t B_size1, size_t B_size2, int *Bp, int *Bi, double *Bx, double *b_ineq);
  ~Nasoq();

  void default_setting();
  int symbolic_QP();
  void reset_symbolic_info();
  void auto_perturbation(size_t total_nnz, double H_norm2, size_t dim, double &reg_diag, int &outer_iter_ref,
                         int &inner_iter_ref);
  void auto_perturbation2(size_t dim, size_t total_nnz, double H_norm2, double range, int n_ineq, double ineq_ratio,
                          double acc_thresh, double &reg_diag, int &outer_iter_ref, int &inner_iter_ref,
                          double &tol);
  void determine_iterations(size_t total_nnz, double acc_thresh, int &outer_iter_ref, int &inner_iter_ref);
  void allocate_workspace();
  int set_warm_start(double *x0_in, double *dual_in, const std::vector<int> &actve_set, double *dual_in_eq = nullptr);
  int set_warm_start_primal(double *x0_in);
  int initialize_x();
  int numeric_QP();
  void update_dual(double step);
  void update_primal(double step);
  int update_active_set(int add_drop, int c_no);
  int solve();
  nasoq_status check_solve_status(int st);
  void detect_solver_name();
  int solve(double *primal_in, double *dual_in, const std::vector<int> &as);
  int solve(double *primal_in);
  int primal_feasibility(int &nxt_add);
  // number of negative multipliers among the first num_active
  int dual_feasibility();
  double dual_step_length(int &nxt_drop);
  double primal_step_length(int nxt_active);
  int update_rhs(int nxt_active);
  // the KKT system of the current active set assembled and solved afresh
  int solve_kkt_from_scratch();
  int solve_kkt(solve_type s_type);
  void edit_kkt(int add_del, int nxt_col);
  double compute_primal_obj();
  // x'Px for an upper-stored P (-1 if P holds an entry below the diagonal)
  double quad_form(const CSC *P, const double *x);
  double compute_dual_obj();
  double complementarity_norm();
  double compute_objective();
  double lagrangian_residual_norm();
  double constraint_sat_norm();
  // Fischer-Burmeister residual norms of the dual and primal complementarity
  double dual_FB_norm();
  double primal_FB_norm();
  double non_negativity_norm();
  void print(int vb_level = 0);
  // <p_name>_primal.txt, _dual.txt and _info.txt (iterations, objectives, time)
  void export_to_file(std::string p_name, std::string vec_head = "");
  void print_log();
  void print_qp_range(int verbose = 0);
  // scalar scaling (scaling < 0) and Ruiz equilibration (scaling > 0) of the
  // problem data, and their inverses on the data and the solution
  int scale_data_2();
  int unscale_data_2();
  int unscale_solution_2();
  int scale_data();
  int unscale_data();
  int unscale_solution();
  // the batched-addition variant of the active-set loop
  int numeric_QP_batch();
  int edit_kkt_batch(int add_del, std::vector<idx_val> nxt_list);
  double primal_step_length_batch(const std::vector<idx_val> &nxt_list);
  int primal_feasibility_batch(std::vector<idx_val> &pair_list);
  int dual_feasibility_inner(int &most_neg);
  int update_active_set_batch(int add_drop, const std::vector<idx_val> nxt_lst);
};

}  // namespace nasoq
#endif
