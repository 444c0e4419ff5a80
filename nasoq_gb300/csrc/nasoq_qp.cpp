// nasoq::Nasoq: the dual active-set QP loop (reference src/nasoq.cpp) over
// nasoq::SolverSettings.  The loop keeps the reference's decisions: the most
// violated inequality enters (primal_feasibility, :787-840), the primal and
// dual step lengths pick between a full step that activates it and a dual step
// that drops the constraint with the smallest ratio (:478-610); every KKT
// change is a SoMod row/column edit followed by a partial refactorization and
// a masked solve on the GPU.
#include "nasoq/nasoq.h"

#include <algorithm>
#include <cmath>
#include <fstream>
#include <iostream>
#include <limits>

#include "nasoq_gb300.h"
#include "qp_rules.hpp"

namespace nasoq {

QPSettings::QPSettings() {
  eps = eps_rel = std::pow(10, -3);
  eps_primal = eps_dual = eps_slack = eps_nn = eps;
  diag_perturb = zero_thresh = std::pow(10, -9);
  max_iter_nas = 4000;
  batch_size = 1;
  scaling = 0;
  inner_iter_ref = 0;
  outer_iter_ref = 0;
  max_iter = 0;
  stop_tol = 1e-15;
  nasoq_variant = "Fixed";
}

nasoq_config::nasoq_config(int a_, int b_, double c_, double d_) : inner_iter(a_), outer_iter(b_), pert_diag(c_),
                                                                   stop_tol(d_) {}

qp_info::qp_info() : sw(true), tot(0), factt(0), init(0), num_update(0), num_downdate(0), num_refactor(0),
                     num_solve(0) {}
std::chrono::time_point<std::chrono::system_clock> qp_info::tic() { return std::chrono::system_clock::now(); }
std::chrono::time_point<std::chrono::system_clock> qp_info::toc() { return std::chrono::system_clock::now(); }
double qp_info::elapsed_time(std::chrono::time_point<std::chrono::system_clock> beg,
                             std::chrono::time_point<std::chrono::system_clock> lst) {
  elapsed_seconds = lst - beg;
  return elapsed_seconds.count();
}
void qp_info::print() { std::cout << tot << "," << factt << ","; }

// ---- small host kernels of the KKT checks --------------------------------
static CSC *transpose_into(const CSC *M, CSC *T) {
  // T = M^T (values kept, rows sorted), M is nrow x ncol
  T->nrow = M->ncol;
  T->ncol = M->nrow;
  size_t nnz = M->ncol ? (size_t)M->p[M->ncol] : 0;
  T->nzmax = nnz;
  T->p = new int[T->ncol + 1]();
  T->i = new int[std::max<size_t>(nnz, 1)];
  T->x = new double[std::max<size_t>(nnz, 1)];
  for (size_t q = 0; q < nnz; ++q) T->p[M->i[q] + 1]++;
  for (size_t r = 0; r < T->ncol; ++r) T->p[r + 1] += T->p[r];
  std::vector<int> pos(T->p, T->p + T->ncol);
  for (size_t j = 0; j < M->ncol; ++j)
    for (int q = M->p[j]; q < M->p[j + 1]; ++q) {
      int t = pos[M->i[q]]++;
      T->i[t] = (int)j;
      T->x[t] = M->x[q];
    }
  T->stype = 0;
  T->packed = TRUE;
  T->sorted = TRUE;
  return T;
}

// y = M x for an m-by-n CSC (reference spmv_csc_small, src/matrixVector/spmv_CSC.cpp:453)
static void spmv_small(size_t m, size_t n, const int *Mp, const int *Mi, const double *Mx, const double *x, double *y) {
  std::fill(y, y + m, 0.0);
  if (!Mp || !x) return;
  for (size_t j = 0; j < n; ++j)
    for (int q = Mp[j]; q < Mp[j + 1]; ++q) y[Mi[q]] += Mx[q] * x[j];
}

// y = H x, H lower-stored symmetric (reference spmv_csc_sym_one_int)
static void spmv_sym_lower(size_t n, const int *Hp, const int *Hi, const double *Hx, const double *x, double *y) {
  std::fill(y, y + n, 0.0);
  for (size_t j = 0; j < n; ++j) {
    double yj = 0.0;
    const double xj = x[j];
    for (int q = Hp[j]; q < Hp[j + 1]; ++q) {
      int i = Hi[q];
      if (i == (int)j) {
        y[i] += Hx[q] * xj;
      } else if (i > (int)j) {
        y[i] += Hx[q] * xj;
        yj += Hx[q] * x[i];
      }
    }
    y[j] += yj;
  }
}

static double inf_norm(size_t n, const double *v) {
  double m = 0;
  for (size_t i = 0; i < n; ++i) {
    double s = std::abs(v[i]);
    if ((!std::isfinite(s) || s > m) && std::isfinite(m)) m = s;
  }
  return m;
}

static double frob_lower(const CSC *H) { return nqg::qp_frob_lower((int)H->ncol, H->p, H->i, H->x); }

// ---- construction ---------------------------------------------------------
Nasoq::Nasoq(size_t H_size, int *Hp, int *Hi, double *Hx, double *q_in, size_t B_row, size_t B_col, int *Bp, int *Bi,
             double *Bx, double *b_ineq) {
  H = new CSC;
  H->nzmax = Hp[H_size];
  H->ncol = H->nrow = H_size;
  H->stype = -1;
  H->p = Hp;
  H->i = Hi;
  H->x = Hx;
  hessian_size = (int)H_size;
  HT = nullptr;
  q = q_in;
  A = new CSC;
  A->stype = 1;
  AT = new CSC;
  a = nullptr;
  eq_const_size = 0;
  B = new CSC;
  B->ncol = B_col;
  B->nrow = B_row;
  B->stype = 0;
  B->p = Bp;
  B->i = Bi;
  B->x = Bx;
  B->nzmax = B_row > 0 ? Bp[B_col] : 0;
  BT = new CSC;
  b = b_ineq;
  ineq_const_size = (int)B_row;
  workspace = new double[B->nrow + 4 * H->ncol + 1];
  primal_vars = new double[std::max<size_t>(H->ncol, 1)]();
  dual_vars = new double[std::max<size_t>(B->nrow, 1)]();
  dual_vars_eq = nullptr;
  used_const = new int[std::max<size_t>(B->nrow, 1)]();
  num_active = 0;
  num_iter = 0;
  warm_start = 0;
  n_active = 0;
  qi = new qp_info;
  ss = nullptr;
  sKKT = nullptr;
  sKKTrhs = kkt_solution = lagrange_mult = lagrange_mult_eq = descent = nullptr;
  primal_obj = dual_obj = objective = 0;
  non_negativity_infn = complementarity_infn = lag_res = cons_sat_norm = 0;
  is_converged = 0;
  used_constraints = 0;
  ret_val = NotConverged;
  gpu_precision = 0;
  eTree = col2const = const2col = etree = pinv = col2sup = as0 = nullptr;
  sKKTt = nullptr;
  D = E = F = Dinv = Einv = Finv = rec_length = nullptr;
  c = cinv = 1.0;
  qp_scalar = inv_qp_scalar = 1.0;
  dual_FB_a = dual_FB_b = dual_FB = primal_FB_a = primal_FB_b = primal_FB = nullptr;
  default_setting();
}

Nasoq::Nasoq(size_t H_size, int *Hp, int *Hi, double *Hx, double *q_in, size_t A_size1, size_t A_size2, int *Ap,
             int *Ai, double *Ax, double *a_eq, size_t B_size1, size_t B_size2, int *Bp, int *Bi, double *Bx,
             double *b_ineq)
    : Nasoq(H_size, Hp, Hi, Hx, q_in, B_size1, B_size2, Bp, Bi, Bx, b_ineq) {
  A->ncol = A_size2;
  A->nrow = A_size1;
  A->stype = 1;
  A->p = Ap;
  A->i = Ai;
  A->x = Ax;
  a = a_eq;
  if (A->nrow > 0) {
    A->nzmax = Ap[H_size];
    dual_vars_eq = new double[A->nrow]();
  }
  eq_const_size = (int)A->ncol;
}

Nasoq::~Nasoq() {
  for (double *v : {D, E, F, Dinv, Einv, Finv}) delete[] v;
  delete[] workspace;
  delete[] primal_vars;
  delete[] dual_vars_eq;
  delete[] dual_vars;
  delete[] used_const;
  delete ss;
  delete qi;
  for (CSC *T : {BT, AT}) {
    if (!T) continue;
    delete[] T->p;
    delete[] T->i;
    delete[] T->x;
    delete T;
  }
  delete H;
  delete A;
  delete B;
}

void Nasoq::default_setting() {
  // reference :163-182
  max_iter_nas = 4000;
  diag_perturb = 1e-9;
  zero_thresh = diag_perturb;
  eps_abs = 1e-3;
  eps_rel = eps_abs;
  warm_start = 0;
  batch_size = 1;
  scaling = 0;
  inner_iter_ref = 0;
  outer_iter_ref = 0;
  max_iter = 0;
  stop_tol = 1e-15;
  auto_reg_en = 0;
  variant = Fixed;
  sol_name = "NASOQ-Fixed";
}

void Nasoq::auto_perturbation2(size_t dim, size_t total_nnz, double H_norm2, double range, int n_ineq,
                               double ineq_ratio, double acc_thresh, double &reg, int &outer, int &inner,
                               double &tol) {
  nqg::qp_auto_perturbation2(dim, total_nnz, H_norm2, range, n_ineq, ineq_ratio, acc_thresh, reg, outer, inner, tol);
}

void Nasoq::determine_iterations(size_t total_nnz, double acc_thresh, int &outer, int &inner) {
  nqg::qp_determine_iterations(total_nnz, acc_thresh, outer, inner);
}

void Nasoq::reset_symbolic_info() {}  // an empty routine in the reference too (:280-281)

void Nasoq::auto_perturbation(size_t total_nnz, double H_norm2, size_t dim, double &reg, int &outer, int &inner) {
  // the reference's first tuning table (:283-312): small problems refine
  // 2x2 with 1e-11 (1e-7 when ||H||_F < 1); large ones pick by ||H||_F
  if (total_nnz < 3e4 || dim < 4100) {
    reg = H_norm2 < 1 ? 1e-7 : 1e-11;
    outer = inner = 2;
    return;
  }
  if (H_norm2 < 1) {
    reg = 1e-7;
    outer = inner = 1;
  } else if (H_norm2 < 1e3) {
    reg = 1e-11;
    outer = inner = 9;
  } else if (H_norm2 < 5e5) {
    reg = 1e-8;
    outer = inner = 0;
  } else {
    reg = 1e-11;
    outer = inner = 1;
  }
}

void Nasoq::allocate_workspace() {
  // the reference sizes its scratch here without allocating it (:400-411);
  // `workspace` (B rows + 4 n doubles) is allocated by the constructor
}

int Nasoq::symbolic_QP() {
  transpose_into(B, BT);
  std::vector<double> rhs0(std::max(hessian_size, 1), 0.0);
  if (A->nrow > 0) {
    transpose_into(A, AT);
    ss = new SolverSettings(H, rhs0.data(), B, BT, A, AT);
  } else {
    ss = new SolverSettings(H, rhs0.data(), B, BT);
  }
  ss->ldl_variant = 2;
  ss->ldl_update_variant = 2;
  ss->solver_mode = 1;
  ss->req_ref_iter = max_iter;
  ss->max_inner_iter = max_iter;
  const size_t total_nnz = H->nzmax + B->nzmax;
  if (auto_reg_en == 2) {
    double H_norm2 = frob_lower(H);
    auto_perturbation2(H->ncol, total_nnz, H_norm2, 0.0, (int)B->nrow, B->nrow / double(H->ncol), eps_abs,
                       diag_perturb, outer_iter_ref, inner_iter_ref, stop_tol);
  } else if (auto_reg_en == 1) {
    determine_iterations(total_nnz, eps_abs, outer_iter_ref, inner_iter_ref);
    stop_tol = 1e-15;
    double H_norm2 = frob_lower(H);
    diag_perturb = H_norm2 < 1 ? std::pow(10, -7) : std::pow(10, -9);
  } else {
    outer_iter_ref = inner_iter_ref = max_iter;
  }
  // An FP32 factorization is only the preconditioner of the FP64 refinement:
  // without enough refinement its solutions carry FP32 rounding into every
  // active-set decision (on degenerate problems enough to make the loop
  // cycle).  Its refinement therefore runs up to 4 restarts of 10 steps and
  // stops once the preconditioned residual is below 1e-10, absolute and
  // relative to the first one.
  ss->tol_abs = ss->tol_rel = stop_tol;
  if (gpu_precision) {
    outer_iter_ref = std::max(outer_iter_ref, 4);
    inner_iter_ref = std::max(inner_iter_ref, 10);
    ss->tol_abs = ss->tol_rel = std::max(stop_tol, 1e-10);
  }
  ss->req_ref_iter = outer_iter_ref;
  ss->max_inner_iter = inner_iter_ref;
  ss->reg_diag = diag_perturb;
  ss->gpu_precision = gpu_precision;
  zero_thresh = diag_perturb;
  if (!ss->symbolic_analysis()) return -1;
  skkt_col = ss->SM->ncol;
  sKKTrhs = ss->rhs;
  kkt_solution = ss->x;
  descent = kkt_solution;
  lagrange_mult_eq = kkt_solution + H->ncol;
  lagrange_mult = kkt_solution + H->ncol + A->nrow;
  sKKT = ss->A_ord;
  return 0;
}

int Nasoq::set_warm_start(double *x0_in, double *dual_in, const std::vector<int> &actve_set, double *dual_in_eq) {
  for (size_t i = 0; i < H->ncol; ++i) primal_vars[i] = x0_in[i];
  if (dual_in_eq)
    for (size_t l = 0; l < A->nrow; ++l) dual_vars_eq[l] = dual_in_eq[l];
  for (size_t j = 0; j < B->nrow; ++j) dual_vars[j] = dual_in[j];
  n_active = 0;
  for (int c_no : actve_set) {
    active_set.push_back(c_no);
    edit_kkt(1, c_no);
    n_active++;
    used_const[c_no] = 1;
  }
  warm_start = 1;
  return warm_start;
}

int Nasoq::set_warm_start_primal(double *x0_in) {
  for (size_t i = 0; i < H->ncol; ++i) primal_vars[i] = x0_in[i];
  n_active = 0;
  warm_start = 1;
  return warm_start;
}

int Nasoq::initialize_x() {
  for (size_t i = 0; i < H->ncol; ++i) sKKTrhs[i] = -q[i];
  for (size_t i = H->ncol, j = 0; i < H->ncol + A->nrow; ++i, ++j) sKKTrhs[i] = a[j];
  for (size_t i = H->ncol + A->nrow; i < skkt_col; ++i) sKKTrhs[i] = 0.0;
  ss->ldl_update_variant = 2;
  solve_kkt(UPDATE);  // unconstrained solution
  for (size_t i = 0; i < H->ncol; ++i) primal_vars[i] = kkt_solution[i];
  for (size_t i = 0, j = H->ncol; i < A->nrow; ++i, ++j) dual_vars_eq[i] = kkt_solution[j];
  return 1;
}

int Nasoq::numeric_QP() {
  int nxt_active = -1, nxt_drop = -1, to_add = 1, num_violated = 0;
  double prime_step, dual_step, step;
  solve_type typ_nxt_solve = warm_start ? REFACTOR : SOLVE;
  while (true) {
    if (num_iter > max_iter_nas) {
      is_converged = 0;
      return is_converged;
    }
    if (to_add == 1) {
      num_violated = primal_feasibility(nxt_active);
      if (num_violated == 0) {
        is_converged = 1;
        return is_converged;
      } else if (nxt_active == -1) {
        is_converged = 0;
        return is_converged;
      }
      update_rhs(nxt_active);
    }
    solve_kkt(typ_nxt_solve);
    prime_step = primal_step_length(nxt_active);
    dual_step = dual_step_length(nxt_drop);
    step = prime_step > dual_step ? dual_step : prime_step;
    if (step == std::numeric_limits<double>::max()) {
      is_converged = 0;
      return is_converged;
    } else if (prime_step == std::numeric_limits<double>::max() && step == dual_step) {  // dual step
      update_dual(step);
      dual_vars[nxt_active] = dual_vars[nxt_active] + step;
      to_add = 0;
      edit_kkt(to_add, nxt_drop);
      typ_nxt_solve = UPDATE;
      update_active_set(to_add, nxt_drop);
    } else {  // full step
      update_primal(step);
      update_dual(step);
      dual_vars[nxt_active] = dual_vars[nxt_active] + step;
      if (step == prime_step) {
        to_add = 1;
        edit_kkt(to_add, nxt_active);
        typ_nxt_solve = UPDATE;
        update_active_set(to_add, nxt_active);
      } else if (step == dual_step) {
        to_add = 0;
        edit_kkt(to_add, nxt_drop);
        typ_nxt_solve = UPDATE;
        update_active_set(to_add, nxt_drop);
      }
    }
    num_iter++;
  }
}

void Nasoq::update_dual(double step) {
  for (size_t i = 0; i < A->nrow; ++i) dual_vars_eq[i] -= step * lagrange_mult_eq[i];
  for (int c : active_set) dual_vars[c] -= step * lagrange_mult[c];
}

void Nasoq::update_primal(double step) {
  for (int i = 0; i < hessian_size; ++i) primal_vars[i] = primal_vars[i] - step * descent[i];
}

int Nasoq::update_active_set(int add_drop, int c_no) {
  if (add_drop) {
    n_active++;
    active_set.push_back(c_no);
    used_const[c_no] = 1;
    return 1;
  }
  n_active--;
  auto it = std::find(active_set.begin(), active_set.end(), c_no);
  if (active_set.empty()) return 0;
  if ((active_set.size() == 1 && active_set[0] == c_no) || (it != active_set.end() && active_set.size() > 1)) {
    active_set.erase(it);
    used_const[c_no] = 0;
    return 1;
  }
  return 0;
}

int Nasoq::solve() {
  ret_val = NotConverged;
  warm_start = 0;
  qi->tot_st = qi->tic();
  int status = 0;
  if (scaling > 0) scale_data();
  if (scaling < 0) scale_data_2();
  if (variant == Tuned) {
    if (symbolic_QP() < 0) return ret_val = Infeasible;
    for (int i = 0; i < 4; i++) {
      initialize_x();
      status = numeric_QP();
    }
  } else {
    auto_reg_en = variant == AUTO ? 2 : (variant == Fixed ? 1 : 0);
    if (symbolic_QP() < 0) return ret_val = Infeasible;
    initialize_x();
    status = numeric_QP();
  }
  if (scaling > 0) {
    unscale_data();
    unscale_solution();
  }
  if (scaling < 0) {
    unscale_data_2();
    unscale_solution_2();
  }
  qi->tot_end = qi->toc();
  qi->tot = qi->elapsed_time(qi->tot_st, qi->tot_end);
  compute_objective();
  ret_val = check_solve_status(status);
  detect_solver_name();
  return ret_val;
}

nasoq_status Nasoq::check_solve_status(int st) {
  if (st == 0) return Infeasible;
  constraint_sat_norm();
  lagrangian_residual_norm();
  complementarity_norm();
  non_negativity_norm();
  if (lag_res <= eps_abs && cons_sat_norm <= eps_abs && non_negativity_infn <= eps_abs) ret_val = Optimal;
  else if (cons_sat_norm <= eps_abs) ret_val = Inaccurate;
  else ret_val = NotConverged;
  return ret_val;
}

void Nasoq::detect_solver_name() {
  if (variant == Fixed) sol_name = "NASOQ-Fixed";
  else if (variant == AUTO) sol_name = "NASOQ-AUTO";
  else if (variant == Tuned) sol_name = "NASOQ-TUNED";
  else sol_name = "NASOQ";
}

int Nasoq::solve(double *primal_in, double *dual_in, const std::vector<int> &as) {
  warm_start = 1;
  qi->tot_st = qi->tic();
  if (scaling > 0) scale_data();
  int rv = symbolic_QP();
  if (rv < 0) return rv;
  set_warm_start(primal_in, dual_in, as);
  rv = numeric_QP();
  if (scaling > 0) {
    unscale_data();
    unscale_solution();
  }
  qi->tot_end = qi->toc();
  qi->tot = qi->elapsed_time(qi->tot_st, qi->tot_end);
  compute_objective();
  constraint_sat_norm();
  lagrangian_residual_norm();
  return rv;
}

int Nasoq::solve(double *primal_in) {
  warm_start = 1;
  qi->tot_st = qi->tic();
  if (scaling > 0) scale_data();
  int rv = symbolic_QP();
  if (rv < 0) return rv;
  set_warm_start_primal(primal_in);
  rv = numeric_QP();
  if (scaling > 0) {
    unscale_data();
    unscale_solution();
  }
  qi->tot_end = qi->toc();
  qi->tot = qi->elapsed_time(qi->tot_st, qi->tot_end);
  compute_objective();
  constraint_sat_norm();
  lagrangian_residual_norm();
  return rv;
}

int Nasoq::primal_feasibility(int &nxt_add) {
  // most violated inequality beyond eps_abs (reference :787-840)
  nxt_add = -1;
  int violated_no = 0;
  if (B->nrow == 0) return violated_no;
  double *tmp = workspace;
  spmv_small(B->nrow, B->ncol, B->p, B->i, B->x, primal_vars, tmp);
  const double tol = eps_abs;
  double max_violated = tol;
  for (size_t i = 0; i < B->nrow; ++i) {
    tmp[i] -= b[i];
    if (tmp[i] > tol) violated_no++;
    if (tmp[i] > max_violated) {
      nxt_add = (int)i;
      max_violated = tmp[i];
    }
  }
  return violated_no;
}

int Nasoq::dual_feasibility() {
  int neg = 0;
  for (int i = 0; i < num_active; ++i)
    if (dual_vars[i] < 0) neg++;
  return neg;
}

double Nasoq::dual_step_length(int &nxt_drop) {
  double step = std::numeric_limits<double>::max();
  for (size_t i = 0; i < B->nrow; ++i) {
    if (lagrange_mult[i] > 0 && used_const[i]) {
      double tmp = dual_vars[i] / lagrange_mult[i];
      if (tmp < step) {
        step = tmp;
        nxt_drop = (int)i;
      }
    }
  }
  return step;
}

double Nasoq::primal_step_length(int nxt_active) {
  double step = std::numeric_limits<double>::max(), bdotx = 0, ddotb = 0;
  for (int i = BT->p[nxt_active]; i < BT->p[nxt_active + 1]; ++i) {
    bdotx += BT->x[i] * primal_vars[BT->i[i]];
    ddotb += BT->x[i] * descent[BT->i[i]];
  }
  if (ddotb < zero_thresh) return step;
  return -(b[nxt_active] - bdotx) / ddotb;
}

int Nasoq::update_rhs(int nxt_active) {
  if (nxt_active < 0 || nxt_active >= (int)B->nrow) return 0;
  std::fill_n(sKKTrhs, skkt_col, 0.0);
  for (int i = BT->p[nxt_active]; i < BT->p[nxt_active + 1]; ++i) sKKTrhs[BT->i[i]] = BT->x[i];
  return 1;
}

int Nasoq::solve_kkt_from_scratch() {
  // [H A' B_S'; A 0 0; B_S 0 0] of the active set S as one lower CSC, the
  // rhs entries of its rows, solved by a plain-mode solver (reference :890-919)
  const int n = (int)H->ncol, me = (int)A->nrow, ns = (int)active_set.size(), N = n + me + ns;
  for (int i = 0; i < me; ++i) lagrange_mult_eq[i] = 0;
  for (size_t i = 0; i < B->nrow; ++i) lagrange_mult[i] = 0;
  std::vector<int> slot(B->nrow, -1);
  for (int t = 0; t < ns; ++t) slot[active_set[t]] = t;
  std::vector<std::vector<std::pair<int, double>>> cols(N);
  for (int j = 0; j < n; ++j) {
    for (int q = H->p[j]; q < H->p[j + 1]; ++q)
      if (H->i[q] >= j) cols[j].push_back({H->i[q], H->x[q]});
    if (me > 0)
      for (int q = A->p[j]; q < A->p[j + 1]; ++q) cols[j].push_back({n + A->i[q], A->x[q]});
    for (int q = B->p[j]; q < B->p[j + 1]; ++q)
      if (slot[B->i[q]] >= 0) cols[j].push_back({n + me + slot[B->i[q]], B->x[q]});
    std::sort(cols[j].begin(), cols[j].end());
  }
  for (int k = n; k < N; ++k) cols[k].push_back({k, 0.0});
  std::vector<int> Kp(N + 1, 0), Ki;
  std::vector<double> Kx, rhs(N);
  for (int j = 0; j < N; ++j) {
    for (auto &e : cols[j]) {
      Ki.push_back(e.first);
      Kx.push_back(e.second);
    }
    Kp[j + 1] = (int)Ki.size();
  }
  for (int i = 0; i < n + me; ++i) rhs[i] = sKKTrhs[i];
  for (int t = 0; t < ns; ++t) rhs[n + me + t] = sKKTrhs[n + me + active_set[t]];
  CSC K;
  K.nrow = K.ncol = N;
  K.nzmax = Kx.size();
  K.p = Kp.data();
  K.i = Ki.data();
  K.x = Kx.data();
  K.stype = -1;
  SolverSettings lin(&K, rhs.data());
  lin.req_ref_iter = outer_iter_ref;
  lin.max_inner_iter = inner_iter_ref;
  lin.tol_abs = lin.tol_rel = stop_tol;
  lin.reg_diag = diag_perturb;
  lin.gpu_precision = gpu_precision;
  if (!lin.symbolic_analysis() || lin.numerical_factorization() < 0) return 0;
  const double *sol = lin.solve_only();
  for (int i = 0; i < n; ++i) descent[i] = sol[i];
  for (int i = 0; i < me; ++i) lagrange_mult_eq[i] = sol[n + i];
  for (int t = 0; t < ns; ++t) lagrange_mult[active_set[t]] = sol[n + me + t];
  delete[] lin.x;
  return 1;
}

int Nasoq::solve_kkt(solve_type s_type) {
  qi->fct_st = qi->tic();
  if (s_type == SOLVE) {
    ss->solve_only();
  } else if (s_type == UPDATE) {
    ss->update_factorization();
    ss->solve_only();
  } else {
    ss->numerical_factorization();
    ss->solve_only();
  }
  qi->fct_end = qi->toc();
  qi->factt += qi->elapsed_time(qi->fct_st, qi->fct_end);
  return 0;
}

void Nasoq::edit_kkt(int add_del, int nxt_col) {
  std::vector<int> sn_list(1, nxt_col);
  ss->add_del_matrix_qp(add_del, sn_list);
}

double Nasoq::compute_primal_obj() {
  std::vector<double> tmp(H->ncol);
  spmv_sym_lower(H->ncol, H->p, H->i, H->x, primal_vars, tmp.data());
  double quad = 0, lin = 0;
  for (size_t i = 0; i < H->ncol; ++i) quad += tmp[i] * primal_vars[i];
  for (size_t i = 0; i < H->ncol; ++i) lin += q[i] * primal_vars[i];
  primal_obj = 0.5 * quad + lin;
  return primal_obj;
}

double Nasoq::quad_form(const CSC *P, const double *x) {
  double v = 0.0;
  for (size_t j = 0; j < P->ncol; ++j)
    for (int q = P->p[j]; q < P->p[j + 1]; ++q) {
      const int i = P->i[q];
      if (i == (int)j) v += 0.5 * P->x[q] * x[i] * x[i];
      else if (i < (int)j) v += P->x[q] * x[i] * x[j];
      else return -1;
    }
  return v;
}

double Nasoq::compute_dual_obj() {
  double *tmp = workspace;
  spmv_small(B->nrow, B->ncol, B->p, B->i, B->x, primal_vars, tmp);
  dual_obj = 0;
  for (size_t i = 0; i < B->nrow; ++i) dual_obj += (tmp[i] - b[i]) * dual_vars[i];
  return dual_obj;
}

double Nasoq::complementarity_norm() {
  double *tmp = workspace;
  spmv_small(B->nrow, B->ncol, B->p, B->i, B->x, primal_vars, tmp);
  for (size_t i = 0; i < B->nrow; ++i) tmp[i] = dual_vars[i] * (tmp[i] - b[i]);
  complementarity_infn = inf_norm(B->nrow, tmp);
  return complementarity_infn;
}

double Nasoq::compute_objective() {
  objective = compute_primal_obj() + compute_dual_obj();
  return objective;
}

double Nasoq::lagrangian_residual_norm() {
  const size_t n = H->ncol;
  double *Hx = workspace, *eqd = workspace + n, *bd = workspace + 2 * n, *res = workspace + 3 * n;
  spmv_sym_lower(n, H->p, H->i, H->x, primal_vars, Hx);
  if (A->nrow > 0) spmv_small(AT->nrow, AT->ncol, AT->p, AT->i, AT->x, dual_vars_eq, eqd);
  else std::fill(eqd, eqd + n, 0.0);
  if (B->nrow > 0) spmv_small(BT->nrow, BT->ncol, BT->p, BT->i, BT->x, dual_vars, bd);
  else std::fill(bd, bd + n, 0.0);
  for (size_t i = 0; i < n; ++i) res[i] = Hx[i] + q[i] + bd[i] + eqd[i];
  lag_res = inf_norm(n, res);
  return lag_res;
}

double Nasoq::constraint_sat_norm() {
  double *tmp = workspace;
  spmv_small(B->nrow, B->ncol, B->p, B->i, B->x, primal_vars, tmp);
  for (size_t i = 0; i < B->nrow; ++i) {
    double diff = tmp[i] - b[i];
    tmp[i] = diff < 0.0 ? 0.0 : diff;
  }
  cons_sat_norm = inf_norm(B->nrow, tmp);
  if (A->nrow > 0) {
    spmv_small(A->nrow, A->ncol, A->p, A->i, A->x, primal_vars, tmp);
    for (size_t i = 0; i < A->nrow; ++i) tmp[i] = tmp[i] - a[i];
    cons_sat_norm = std::max(cons_sat_norm, inf_norm(A->nrow, tmp));
  }
  return cons_sat_norm;
}

// a + b - sqrt(a^2 + b^2): zero exactly when a >= 0, b >= 0 and a b = 0
static void fischer_burmeister(size_t m, const double *a, const double *b, double *f) {
  for (size_t i = 0; i < m; ++i) f[i] = a[i] + b[i] - std::sqrt(a[i] * a[i] + b[i] * b[i]);
}

double Nasoq::dual_FB_norm() {
  // the dual complementarity at z with x(z) = H^{-1} (B' z), H^{-1} q through
  // a plain-mode solver on H (reference :1108-1160)
  const size_t n = H->ncol, m = B->nrow;
  std::vector<double> Bz(n), t1(m), t2(m), fa(m), fb(m), f(m);
  spmv_small(BT->nrow, BT->ncol, BT->p, BT->i, BT->x, dual_vars, Bz.data());
  SolverSettings hs(H, Bz.data());
  hs.gpu_precision = gpu_precision;
  hs.symbolic_analysis();
  hs.numerical_factorization();
  double *hx = hs.solve_only();
  spmv_small(m, B->ncol, B->p, B->i, B->x, hx, t1.data());
  for (size_t j = 0; j < n; ++j) hs.rhs[j] = q[j];
  hx = hs.solve_only();
  spmv_small(m, B->ncol, B->p, B->i, B->x, hx, t2.data());
  for (size_t i = 0; i < m; ++i) {
    fa[i] = dual_vars[i];
    fb[i] = t1[i] + t2[i] + b[i];
  }
  fischer_burmeister(m, fa.data(), fb.data(), f.data());
  delete[] hs.x;
  return inf_norm(m, f.data());
}

double Nasoq::primal_FB_norm() {
  const size_t m = B->nrow;
  std::vector<double> bx(m), fa(m), fb(m), f(m);
  spmv_small(m, B->ncol, B->p, B->i, B->x, primal_vars, bx.data());
  for (size_t i = 0; i < m; ++i) {
    fa[i] = dual_vars[i];
    fb[i] = b[i] - bx[i];
  }
  fischer_burmeister(m, fa.data(), fb.data(), f.data());
  return inf_norm(m, f.data());
}

double Nasoq::non_negativity_norm() {
  double *tmp = workspace;
  for (size_t i = 0; i < B->nrow; ++i) tmp[i] = dual_vars[i] > 0.0 ? 0 : dual_vars[i];
  non_negativity_infn = inf_norm(B->nrow, tmp);
  return non_negativity_infn;
}

void Nasoq::print(int) {
  if (is_converged) std::cout << "\nConverged in " << num_iter << " .";
  std::cout << "\n objective is (primal, dual, total):" << primal_obj << ", " << dual_obj << ", " << objective
            << "\n";
}

// the header, then one value per line at 30 significant digits
static void write_values(const std::string &path, size_t n, const double *v, const std::string &head) {
  if (n == 0) return;
  std::ofstream f(path);
  f.precision(30);
  f << head;
  for (size_t i = 0; i < n; ++i) {
    f << v[i];
    if (i + 1 < n) f << "\n";
  }
}

void Nasoq::export_to_file(std::string p_name, std::string vec_head) {
  write_values(p_name + "_primal.txt", H->ncol, primal_vars, vec_head);
  write_values(p_name + "_dual.txt", B->nrow, dual_vars, "");
  const double info[5] = {(double)num_iter, primal_obj, dual_obj, objective, qi->tot};
  write_values(p_name + "_info.txt", 5, info, "");
}

// largest |v|, smallest |v| above 0 among entries that are not a new maximum,
// mean and variance of |v| (the reference's max_min_vector rule)
static void abs_range(size_t n, const double *v, double &mx, double &mn, double &avg, double &var) {
  mx = -std::numeric_limits<double>::max();
  mn = std::numeric_limits<double>::max();
  avg = var = 0;
  for (size_t i = 0; i < n; ++i) {
    const double t = std::abs(v[i]);
    if (t > mx) mx = t;
    else if (t < mn && t > 0) mn = t;
    avg += t / n;
  }
  for (size_t i = 0; i < n; ++i) {
    const double t = std::abs(v[i]) - avg;
    var += t * t / n;
  }
}

void Nasoq::print_qp_range(int verbose) {
  // data arrays bound both ends of the range, solution arrays only the top
  struct Item {
    size_t n;
    const double *v;
    bool both;
  };
  const Item items[] = {{H->nzmax, H->x, true},           {H->ncol, q, true},
                        {H->ncol, primal_vars, false},    {A->nzmax, A->x, true},
                        {A->nrow, a, true},               {A->nrow, dual_vars_eq, false},
                        {B->nzmax, B->x, true},           {B->nrow, b, true},
                        {B->nrow, dual_vars, false}};
  double max_max = -std::numeric_limits<double>::max(), min_min = std::numeric_limits<double>::max();
  for (const Item &it : items) {
    double mx = 0, mn = 0, avg = 0, var = 0;
    if (it.v) abs_range(it.n, it.v, mx, mn, avg, var);
    else abs_range(0, nullptr, mx, mn, avg, var);
    if (verbose) std::cout << mx << "," << mn << "," << avg << "," << var << ",";
    if (it.both) min_min = std::min(min_min, mn);
    max_max = std::max(max_max, mx);
  }
  std::cout << min_min << "," << max_max << "," << max_max / min_min << ",";
}

void Nasoq::print_log() {
  std::cout << eps_abs << "," << outer_iter_ref << "," << inner_iter_ref << ",";
  std::cout << stop_tol << "," << diag_perturb << "," << ret_val << "," << num_iter << ",";
  std::cout << qi->tot << "," << active_set.size() << "," << cons_sat_norm << ",";
  std::cout << lag_res << "," << primal_obj << "," << dual_obj << "," << objective << ",";
  std::cout << non_negativity_infn << "," << complementarity_infn << ",";
}

// ---- scaling -----------------------------------------------------------------
// diag(row) M diag(col), the row factor applied first (the products are
// rounded in the reference's order)
static void scale_rows_cols(CSC *M, const double *row, const double *col) {
  if (!M || !M->p) return;
  for (size_t j = 0; j < M->ncol; ++j)
    for (int q = M->p[j]; q < M->p[j + 1]; ++q) {
      if (row) M->x[q] *= row[M->i[q]];
      if (col) M->x[q] *= col[j];
    }
}

static void scale_all(CSC *M, double s) {
  if (!M || !M->p) return;
  for (int q = 0; q < M->p[M->ncol]; ++q) M->x[q] *= s;
}

// column infinity norms of a lower- or upper-stored symmetric matrix
static void sym_col_norms(const CSC *M, double *e) {
  std::fill(e, e + M->ncol, 0.0);
  for (size_t j = 0; j < M->ncol; ++j)
    for (int q = M->p[j]; q < M->p[j + 1]; ++q) {
      const int i = M->i[q];
      const double v = std::abs(M->x[q]);
      e[j] = std::max(e[j], v);
      if (i != (int)j) e[i] = std::max(e[i], v);
    }
}

// a norm below 1e-4 counts as 1 (no scaling), one above 1e4 is capped there
static double clamp_norm(double v) { return v < 1e-4 ? 1.0 : (v > 1e4 ? 1e4 : v); }

int Nasoq::scale_data_2() {
  // a single scalar on the data (reference :1319-1332, where the scalar is
  // fixed at 1)
  inv_qp_scalar = 1.0;
  qp_scalar = 1.0 / inv_qp_scalar;
  scale_all(H, qp_scalar * qp_scalar);
  for (size_t i = 0; i < H->ncol; ++i) q[i] *= qp_scalar;
  scale_all(A, qp_scalar);
  scale_all(B, qp_scalar);
  return 1;
}

int Nasoq::unscale_data_2() {
  scale_all(H, inv_qp_scalar * inv_qp_scalar);
  for (size_t i = 0; i < H->ncol; ++i) q[i] *= inv_qp_scalar;
  scale_all(A, inv_qp_scalar);
  scale_all(AT, inv_qp_scalar);
  scale_all(B, inv_qp_scalar);
  scale_all(BT, inv_qp_scalar);
  return 1;
}

int Nasoq::unscale_solution_2() {
  for (size_t i = 0; i < H->ncol; ++i) primal_vars[i] *= qp_scalar;
  return 1;
}

int Nasoq::scale_data() {
  // Modified Ruiz equilibration of the KKT matrix [H A' B'; A 0 0; B 0 0]
  // with S = diag(D, E, F), plus the cost scaling c, `scaling` rounds
  // (reference :1352-1483, the OSQP data scaling): each round divides every
  // row and column by the square root of its infinity norm, then scales H
  // and q by 1 / max(mean column norm of H, |q|_inf).
  const size_t n = H->ncol, me = A->nrow, m = B->nrow;
  auto fresh = [](double *&v, size_t k) {
    delete[] v;
    v = new double[std::max<size_t>(k, 1)];
    std::fill(v, v + std::max<size_t>(k, 1), 1.0);
  };
  fresh(D, n), fresh(E, me), fresh(F, m), fresh(Dinv, n), fresh(Einv, me), fresh(Finv, m);
  c = 1.0;
  std::vector<double> dt(n), dc(n), et(me), ft(m);
  for (int r = 0; r < scaling; ++r) {
    sym_col_norms(H, dt.data());
    for (const CSC *M : {(const CSC *)A, (const CSC *)B}) {
      if (!M->p) continue;
      for (size_t j = 0; j < M->ncol; ++j) {
        double mx = 0;
        for (int q2 = M->p[j]; q2 < M->p[j + 1]; ++q2) mx = std::max(mx, std::abs(M->x[q2]));
        dt[j] = std::max(dt[j], mx);
      }
    }
    std::fill(et.begin(), et.end(), 0.0);
    std::fill(ft.begin(), ft.end(), 0.0);
    if (A->p)
      for (size_t j = 0; j < A->ncol; ++j)
        for (int q2 = A->p[j]; q2 < A->p[j + 1]; ++q2) et[A->i[q2]] = std::max(et[A->i[q2]], std::abs(A->x[q2]));
    if (B->p)
      for (size_t j = 0; j < B->ncol; ++j)
        for (int q2 = B->p[j]; q2 < B->p[j + 1]; ++q2) ft[B->i[q2]] = std::max(ft[B->i[q2]], std::abs(B->x[q2]));
    for (double &v : dt) v = 1.0 / std::sqrt(clamp_norm(v));
    for (double &v : et) v = 1.0 / std::sqrt(clamp_norm(v));
    for (double &v : ft) v = 1.0 / std::sqrt(clamp_norm(v));
    scale_rows_cols(H, dt.data(), dt.data());
    scale_rows_cols(A, et.data(), dt.data());
    scale_rows_cols(B, ft.data(), dt.data());
    for (size_t i = 0; i < n; ++i) {
      q[i] *= dt[i];
      D[i] *= dt[i];
    }
    for (size_t i = 0; i < me; ++i) E[i] *= et[i];
    for (size_t i = 0; i < m; ++i) F[i] *= ft[i];
    // cost scaling
    sym_col_norms(H, dc.data());
    double mean = 0;
    for (double v : dc) mean += v;
    mean /= (double)n;
    const double qn = clamp_norm(inf_norm(n, q));
    const double ct = 1.0 / clamp_norm(std::max(mean, qn));
    scale_all(H, ct);
    for (size_t i = 0; i < n; ++i) q[i] *= ct;
    c *= ct;
  }
  cinv = 1.0 / c;
  for (size_t i = 0; i < n; ++i) Dinv[i] = 1.0 / D[i];
  for (size_t i = 0; i < me; ++i) Einv[i] = 1.0 / E[i];
  for (size_t i = 0; i < m; ++i) Finv[i] = 1.0 / F[i];
  for (size_t i = 0; i < me; ++i) a[i] *= E[i];
  for (size_t i = 0; i < m; ++i) b[i] *= F[i];
  return 0;
}

int Nasoq::unscale_data() {
  scale_all(H, cinv);
  scale_rows_cols(H, Dinv, Dinv);
  for (size_t i = 0; i < H->ncol; ++i) {
    q[i] *= cinv;
    q[i] *= Dinv[i];
  }
  if (A->nrow > 0) {
    scale_rows_cols(A, Einv, Dinv);
    scale_rows_cols(AT, Dinv, Einv);
    for (size_t i = 0; i < A->nrow; ++i) a[i] *= Einv[i];
  }
  scale_rows_cols(B, Finv, Dinv);
  scale_rows_cols(BT, Dinv, Finv);
  for (size_t i = 0; i < B->nrow; ++i) b[i] *= Finv[i];
  return 0;
}

int Nasoq::unscale_solution() {
  for (size_t i = 0; i < H->ncol; ++i) primal_vars[i] *= D[i];
  for (size_t i = 0; i < A->nrow; ++i) {
    dual_vars_eq[i] *= E[i];
    dual_vars_eq[i] *= cinv;
  }
  for (size_t i = 0; i < B->nrow; ++i) {
    dual_vars[i] *= F[i];
    dual_vars[i] *= cinv;
  }
  return 0;
}

// ---- the batched-addition variant (reference :1540-1735) -----------------------
idx_val::idx_val() : val(0.0), idx(-1) {}
idx_val::idx_val(int i, double v) : val(v), idx(i) {}
bool CMP(idx_val x, idx_val y) { return x.val < y.val; }
int remove_from_list(std::vector<idx_val> &list_const, int c_no) {
  for (size_t i = 0; i < list_const.size(); ++i)
    if (list_const[i].idx == c_no) {
      list_const.erase(list_const.begin() + i);
      return 1;
    }
  return 0;
}

int Nasoq::numeric_QP_batch() {
  // every violated row enters at once (all but the most violated through a
  // row edit); rows whose multiplier turns negative leave again before the
  // step; then the usual primal / dual step on the most violated row
  int nxt_active = -1, nxt_drop = -1, to_add = 1;
  std::vector<idx_val> nxt_list;
  solve_type typ = SOLVE;
  while (true) {
    if (num_iter > max_iter_nas) return is_converged = 0;
    if (to_add == 1) {
      const int nviol = primal_feasibility_batch(nxt_list);
      if (nviol == 0) {
        compute_objective();
        return is_converged = 1;
      }
      if (nxt_list.empty()) return is_converged = 0;
      edit_kkt_batch(to_add, nxt_list);
      nxt_active = nxt_list.back().idx;
      update_rhs(nxt_active);
      typ = UPDATE;
      to_add = 0;
    }
    while (!to_add) {
      int neg = -1;
      solve_kkt(typ);
      if (dual_feasibility_inner(neg) == 0) break;
      edit_kkt(to_add, neg);
      typ = UPDATE;
      remove_from_list(nxt_list, neg);
    }
    update_active_set_batch(0, nxt_list);
    const double prime_step = primal_step_length_batch(nxt_list);
    const double dual_step = dual_step_length(nxt_drop);
    const double step = prime_step > dual_step ? dual_step : prime_step;
    if (step == std::numeric_limits<double>::max()) return is_converged = 0;
    if (prime_step == std::numeric_limits<double>::max() && step == dual_step) {
      to_add = 0;
      edit_kkt(to_add, nxt_drop);
      typ = UPDATE;
      update_active_set(to_add, nxt_drop);
    } else {
      update_primal(step);
      update_dual(step);
      dual_vars[nxt_active] += step;
      if (step == prime_step) {
        to_add = 1;
        edit_kkt(to_add, nxt_active);
        update_active_set(to_add, nxt_active);
      } else if (step == dual_step) {
        to_add = 0;
        edit_kkt(to_add, nxt_drop);
        typ = UPDATE;
        update_active_set(to_add, nxt_drop);
      }
    }
    num_iter++;
  }
}

int Nasoq::edit_kkt_batch(int add_del, std::vector<idx_val> nxt_list) {
  std::vector<int> rows;
  for (size_t i = 0; i + 1 < nxt_list.size(); ++i) rows.push_back(nxt_list[i].idx);
  ss->add_del_matrix_qp(add_del, rows);
  return 1;
}

double Nasoq::primal_step_length_batch(const std::vector<idx_val> &nxt_list) {
  double step = std::numeric_limits<double>::max();
  for (const idx_val &p : nxt_list) {
    double bdotx = 0, ddotb = 0;
    for (int i = BT->p[p.idx]; i < BT->p[p.idx + 1]; ++i) {
      bdotx += BT->x[i] * primal_vars[BT->i[i]];
      ddotb += BT->x[i] * descent[BT->i[i]];
    }
    if (ddotb < zero_thresh) return std::numeric_limits<double>::max();
    step = std::min(step, -(b[p.idx] - bdotx) / ddotb);
  }
  return step;
}

int Nasoq::primal_feasibility_batch(std::vector<idx_val> &pair_list) {
  pair_list.clear();
  double *tmp = workspace;
  spmv_small(B->nrow, B->ncol, B->p, B->i, B->x, primal_vars, tmp);
  for (size_t i = 0; i < B->nrow; ++i) {
    tmp[i] -= b[i];
    if (tmp[i] > zero_thresh) pair_list.emplace_back((int)i, tmp[i]);
  }
  std::sort(pair_list.begin(), pair_list.end(), CMP);
  return (int)pair_list.size();
}

int Nasoq::dual_feasibility_inner(int &most_neg) {
  int neg = 0;
  most_neg = -1;
  double mn = std::numeric_limits<double>::max();
  for (size_t i = 0; i < B->nrow; ++i)
    if (lagrange_mult[i] < 0) {
      neg++;
      if (lagrange_mult[i] < mn) {
        mn = lagrange_mult[i];
        most_neg = (int)i;
      }
    }
  return neg;
}

int Nasoq::update_active_set_batch(int add_drop, const std::vector<idx_val> nxt_lst) {
  // adds every listed row but the last; the reference leaves removal
  // unimplemented (returns 0)
  if (!add_drop) return 0;
  for (size_t i = 0; i + 1 < nxt_lst.size(); ++i) {
    n_active++;
    active_set.push_back(nxt_lst[i].idx);
    used_const[nxt_lst[i].idx] = 1;
  }
  return 1;
}

}  // namespace nasoq

// ---- C ABI of the QP solve --------------------------------------------------
extern "C" void nqg_qp_default_settings(nqg_qp_settings *s) {
  if (!s) return;
  s->variant = nasoq::Fixed;
  s->eps_abs = 1e-3;
  s->diag_perturb = 1e-9;
  s->stop_tol = 1e-15;
  s->max_iter = 0;
  s->max_iter_nas = 4000;
  s->precision = NQG_FP64;
  s->scaling = 0;
}

extern "C" int nqg_qp_solve(int n, const int *Hp, const int *Hi, const double *Hx, const double *q, int meq,
                            const int *Ap, const int *Ai, const double *Ax, const double *a, int mineq, const int *Bp,
                            const int *Bi, const double *Bx, const double *b, const nqg_qp_settings *settings,
                            const double *x0, const double *z0, const double *y0, int n_as, const int *as0, double *x,
                            double *y, double *z, int *active_set, nqg_qp_result *result) {
  if (n <= 0 || !Hp || !Hi || !Hx || !q || meq < 0 || mineq < 0 || !x) return NQG_ERR_ARG;
  if (meq > 0 && (!Ap || !Ai || !Ax || !a || !y)) return NQG_ERR_ARG;
  if (mineq > 0 && (!Bp || !Bi || !Bx || !b || !z)) return NQG_ERR_ARG;
  nqg_qp_settings st;
  if (settings) st = *settings;
  else nqg_qp_default_settings(&st);
  // private copies: the solver object borrows its input arrays
  std::vector<int> hp(Hp, Hp + n + 1), hi(Hi, Hi + Hp[n]);
  std::vector<double> hx(Hx, Hx + Hp[n]), qq(q, q + n);
  std::vector<int> ap(n + 1, 0), ai, bp(n + 1, 0), bi;
  std::vector<double> ax, av, bx, bv;
  if (meq > 0) {
    ap.assign(Ap, Ap + n + 1);
    ai.assign(Ai, Ai + Ap[n]);
    ax.assign(Ax, Ax + Ap[n]);
    av.assign(a, a + meq);
  }
  if (mineq > 0) {
    bp.assign(Bp, Bp + n + 1);
    bi.assign(Bi, Bi + Bp[n]);
    bx.assign(Bx, Bx + Bp[n]);
    bv.assign(b, b + mineq);
  }
  ai.push_back(0);
  ax.push_back(0);
  av.push_back(0);
  bi.push_back(0);
  bx.push_back(0);
  bv.push_back(0);
  nasoq::Nasoq *qm;
  if (meq > 0)
    qm = new nasoq::Nasoq(n, hp.data(), hi.data(), hx.data(), qq.data(), meq, n, ap.data(), ai.data(), ax.data(),
                          av.data(), mineq, n, bp.data(), bi.data(), bx.data(), bv.data());
  else
    qm = new nasoq::Nasoq(n, hp.data(), hi.data(), hx.data(), qq.data(), mineq, n, bp.data(), bi.data(), bx.data(),
                          bv.data());
  qm->diag_perturb = st.diag_perturb;
  qm->eps_abs = st.eps_abs;
  qm->max_iter = st.max_iter;
  qm->stop_tol = st.stop_tol;
  qm->max_iter_nas = st.max_iter_nas;
  qm->variant = (nasoq::nasoq_mode)st.variant;
  qm->gpu_precision = st.precision == NQG_FP32 ? 1 : 0;
  qm->scaling = st.scaling;
  int status;
  const bool warm = x0 && z0 && as0 && n_as >= 0;
  if (!warm) {
    status = qm->solve();
  } else {
    // warm start: the documented steps, with the equality duals passed along
    qm->warm_start = 1;
    qm->qi->tot_st = qm->qi->tic();
    qm->auto_reg_en = qm->variant == nasoq::AUTO ? 2 : (qm->variant == nasoq::Fixed ? 1 : 0);
    if (qm->scaling > 0) qm->scale_data();
    if (qm->symbolic_QP() < 0) {
      delete qm;
      return NQG_ERR_SYMBOLIC;
    }
    std::vector<double> xw(x0, x0 + n), zw(z0, z0 + mineq), yw(meq, 0.0);
    if (y0) yw.assign(y0, y0 + meq);
    if (qm->scaling > 0) {  // the starting point in the scaled variables
      for (int i = 0; i < n; ++i) xw[i] *= qm->Dinv[i];
      for (int k = 0; k < mineq; ++k) zw[k] *= qm->Finv[k] * qm->c;
      for (int r = 0; r < meq; ++r) yw[r] *= qm->Einv[r] * qm->c;
    }
    std::vector<int> asw(as0, as0 + n_as);
    qm->set_warm_start(xw.data(), zw.data(), asw, meq > 0 ? yw.data() : nullptr);
    int conv = qm->numeric_QP();
    if (qm->scaling > 0) {
      qm->unscale_data();
      qm->unscale_solution();
    }
    qm->qi->tot_end = qm->qi->toc();
    qm->qi->tot = qm->qi->elapsed_time(qm->qi->tot_st, qm->qi->tot_end);
    qm->compute_objective();
    status = qm->check_solve_status(conv);
  }
  std::copy(qm->primal_vars, qm->primal_vars + n, x);
  if (meq > 0) std::copy(qm->dual_vars_eq, qm->dual_vars_eq + meq, y);
  if (mineq > 0) std::copy(qm->dual_vars, qm->dual_vars + mineq, z);
  if (active_set)
    for (size_t k = 0; k < qm->active_set.size() && (int)k < mineq; ++k) active_set[k] = qm->active_set[k];
  if (result) {
    result->status = status;
    result->num_iter = qm->num_iter;
    result->active_size = (int)qm->active_set.size();
    result->objective = qm->objective;
    result->primal_obj = qm->primal_obj;
    result->dual_obj = qm->dual_obj;
    result->lag_res = qm->lag_res;
    result->cons_sat_norm = qm->cons_sat_norm;
    result->non_negativity_infn = qm->non_negativity_infn;
    result->complementarity_infn = qm->complementarity_infn;
    result->total_seconds = qm->qi->tot;
    result->factor_seconds = qm->qi->factt;
  }
  int gst = qm->ss ? qm->ss->last_gpu_status : 0;
  delete qm;
  return gst < 0 ? gst : NQG_OK;
}
