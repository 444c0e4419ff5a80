// nasoq::SolverSettings over the C ABI (drop-in for the reference's
// src/QP/linear_solver_wrapper.cpp).  Host work: the QP super-KKT assembly,
// the perturbation bookkeeping, the hidden-column assembly-tree edits of the
// QP mode (SYM_REMOV) and the supernode marking of each row/column edit.
// Everything numeric runs on the GPU through nqg_* calls.
#include "nasoq/QP/linear_solver_wrapper.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <iostream>
#include <queue>

#include "nasoq_gb300.h"
#include "symbolic.hpp"

namespace nasoq {

profiling_solver_info::profiling_solver_info(int nt)
    : fact_time(0), analysis_time(0), solve_time(0), iter_time(0), ordering_time(0), update_time(0), piv_reord(0) {
  timing_chol = new double[4 + nt]();
}
profiling_solver_info::profiling_solver_info(int nt, double ft, double at, double st, double it, double ot, double ut,
                                             double pr)
    : fact_time(ft), analysis_time(at), solve_time(st), iter_time(it), ordering_time(ot), update_time(ut),
      piv_reord(pr) {
  timing_chol = new double[4 + nt]();
}
profiling_solver_info::~profiling_solver_info() { delete[] timing_chol; }
std::chrono::time_point<std::chrono::system_clock> profiling_solver_info::tic() {
  return std::chrono::system_clock::now();
}
std::chrono::time_point<std::chrono::system_clock> profiling_solver_info::toc() {
  return std::chrono::system_clock::now();
}
double profiling_solver_info::elapsed_time(std::chrono::time_point<std::chrono::system_clock> beg,
                                           std::chrono::time_point<std::chrono::system_clock> lst) {
  elapsed_seconds = lst - beg;
  return elapsed_seconds.count();
}
void profiling_solver_info::print_profiling() {
  std::cout << "analysis time: " << analysis_time << ";";
  std::cout << "fact time: " << fact_time << ";";
  std::cout << "update time: " << update_time << ";";
  std::cout << "reordering pivot time: " << piv_reord << ";";
  std::cout << "solve time: " << solve_time << ";";
}

static CSC *transpose_csc(const CSC *B) {
  // column-compressed transpose of an nrow-by-ncol matrix (rows sorted)
  auto *T = new CSC;
  T->nrow = B->ncol;
  T->ncol = B->nrow;
  size_t nnz = B->ncol ? (size_t)B->p[B->ncol] : 0;
  T->nzmax = nnz;
  T->p = new int[T->ncol + 1]();
  T->i = new int[std::max<size_t>(nnz, 1)];
  T->x = new double[std::max<size_t>(nnz, 1)];
  for (size_t q = 0; q < nnz; ++q) T->p[B->i[q] + 1]++;
  for (size_t r = 0; r < T->ncol; ++r) T->p[r + 1] += T->p[r];
  std::vector<int> pos(T->p, T->p + T->ncol);
  for (size_t j = 0; j < B->ncol; ++j)
    for (int q = B->p[j]; q < B->p[j + 1]; ++q) {
      int t = pos[B->i[q]]++;
      T->i[t] = (int)j;
      T->x[t] = B->x[q];
    }
  T->stype = B->stype;
  T->xtype = B->xtype;
  T->packed = B->packed;
  T->sorted = TRUE;
  return T;
}

static void free_csc(CSC *&A) {
  if (!A) return;
  delete[] A->p;
  delete[] A->i;
  delete[] A->x;
  delete A;
  A = nullptr;
}

SolverSettings::SolverSettings(CSC *Amat, double *rhs_in) {
  default_setting();
  A = Amat;
  rhs = rhs_in;
  solver_mode = 0;
  remove_trans = 0;
}

SolverSettings::SolverSettings(CSC *Amat, double *rhs_in, CSC *Bmat) : SolverSettings(Amat, rhs_in) {
  B = Bmat;
  BT = transpose_csc(B);
  remove_trans = 1;
  solver_mode = 1;
}

SolverSettings::SolverSettings(CSC *Amat, double *rhs_in, CSC *Bmat, double *b) : SolverSettings(Amat, rhs_in, Bmat) {
  extra_rhs = b;
}

SolverSettings::SolverSettings(CSC *Amat, double *rhs_in, CSC *Bmat, CSC *BTmat) : SolverSettings(Amat, rhs_in) {
  B = Bmat;
  BT = BTmat;
  solver_mode = 1;
}

SolverSettings::SolverSettings(CSC *Amat, double *rhs_in, CSC *Bmat, CSC *BTmat, CSC *Cmat, CSC *CTmat)
    : SolverSettings(Amat, rhs_in, Bmat, BTmat) {
  C = Cmat;
  CT = CTmat;
  solver_mode = 1;
}

SolverSettings::~SolverSettings() {
  if (plan) nqg_plan_destroy(plan);
  if (L) {
    delete[] L->Perm;
    delete[] L->IPerm;
    delete[] L->ColCount;
    delete[] L->Parent;
    delete[] L->super;
    delete[] L->col2Sup;
    delete[] L->sParent;
    delete[] L->s;
    delete[] L->p;
    delete[] L->i_ptr;
    delete L;
  }
  free_csc(A_ord);
  delete psi;
  delete[] perm_piv;
  delete[] marked;
  delete[] valL;
  delete[] d_val;
  delete[] visible_cnt;
  delete[] extra_cols;
  delete[] atree;
  delete[] visible_sn;
  delete[] child_sn_ptr;
  delete[] child_sn_no;
  delete[] num_sn_child;
  delete[] etree_mod;
  delete[] child_ptr;
  delete[] child_no;
  delete[] num_child;
  delete[] s_level_ptr;
  delete[] s_level_set;
  delete[] ws;
  delete[] ws_int;
  delete[] ws_zeroed;
  if (own_simplicial) {
    delete[] l_pb;
    delete[] l_pe;
    delete[] l_i;
  }
  if (remove_trans) free_csc(BT);
  if (solver_mode == 1) {
    delete[] sm_rhs;
    delete[] sm_solution;
    free_csc(SM);
  } else {
    delete SM;
  }
}

void SolverSettings::default_setting() {
  // reference defaults, src/QP/linear_solver_wrapper.cpp:205-244
  solver_mode = 0;
  L = nullptr;
  valL = d_val = x = rhs = nullptr;
  A = SM = AorSM = A_ord = AT_ord = B = BT = C = CT = nullptr;
  dim1 = base = 0;
  perm_piv = pinv = nullptr;
  a_consistent = 1;
  ldl_variant = 2;
  ldl_update_variant = 2;
  sm_rhs = sm_solution = nullptr;
  l_pb = l_pe = l_i = nullptr;
  l_x = nullptr;
  is_super = 1;
  simplicial_alloc = 0;
  ws_int_size = ws_dbl_size = 0;
  n_level = n_par = n_level_s = n_par_s = 0;
  level_ptr = level_set = par_ptr = par_set = nullptr;
  level_ptr_s = par_ptr_s = par_set_s = nullptr;
  s_level_ptr = s_level_set = nullptr;
  s_level_no = -1;
  prune_ptr = prune_set = nullptr;
  extra_cols = nullptr;
  n_relax[0] = 4;
  n_relax[1] = 16;
  n_relax[2] = 48;
  z_relax[0] = 0.8;
  z_relax[1] = 0.1;
  z_relax[2] = 0.05;
  max_sup_wid = max_col = 0;
  ordering_type = 0;
  atree = etree = etree_mod = nullptr;
  visible_cnt = nullptr;
  child_ptr = child_no = num_child = nullptr;
  child_sn_ptr = child_sn_no = num_sn_child = nullptr;
  col_del = 0;
  to_del = 0;
  reg_diag = 1e-8;
  num_pivot = 0;
  req_ref_iter = 2;
  max_iter = req_ref_iter;
  max_inner_iter = 2;
  num_ref_iter = 0;
  tol_abs = 1e-15;
  tol_rel = 1e-15;
  regularization = 1;
  num_thread = 1;
  cost_param = num_thread;
  level_param = -3;
  final_seq_node = 50;
  chunk = 1;
  thread_thresh = 25;
  psi = new profiling_solver_info(num_thread);
  marked = visible_sn = nullptr;
  ws = ws_zeroed = nullptr;
  ws_int = nullptr;
  extra_rhs = nullptr;
  remove_trans = 0;
  A_l1 = x_l1 = rhs_l1 = res_l1 = bwd_err = 0;
  gpu_precision = 0;
  plan = nullptr;
  last_gpu_status = 0;
  own_simplicial = false;
}

int SolverSettings::build_super_matrix() {
  // SM = [H ; C(eq) ; B(ineq)] lower-stored, inequality values 0, one zero
  // diagonal per constraint column (reference :246-350).
  const size_t n = A->ncol;
  const size_t meq = C ? C->nrow : 0, mineq = B ? B->nrow : 0;
  const size_t N = n + meq + mineq;
  SM = SM ? SM : new CSC;
  int *SMp = new int[N + 1];
  SMp[0] = 0;
  for (size_t j = 0; j < n; ++j) {
    int cnt = A->p[j + 1] - A->p[j];
    if (meq) cnt += C->p[j + 1] - C->p[j];
    if (mineq) cnt += B->p[j + 1] - B->p[j];
    SMp[j + 1] = SMp[j] + cnt;
  }
  for (size_t k = n; k < N; ++k) SMp[k + 1] = SMp[k] + 1;
  size_t nnz = SMp[N];
  int *SMi = new int[std::max<size_t>(nnz, 1)];
  double *SMx = new double[std::max<size_t>(nnz, 1)]();
  for (size_t j = 0; j < n; ++j) {
    size_t t = SMp[j];
    for (int q = A->p[j]; q < A->p[j + 1]; ++q, ++t) {
      SMi[t] = A->i[q];
      SMx[t] = A->x[q];
    }
    if (meq)
      for (int q = C->p[j]; q < C->p[j + 1]; ++q, ++t) {
        SMi[t] = (int)n + C->i[q];
        SMx[t] = C->x[q];
      }
    if (mineq)
      for (int q = B->p[j]; q < B->p[j + 1]; ++q, ++t) {
        SMi[t] = (int)(n + meq) + B->i[q];
        SMx[t] = 0.0;
      }
  }
  for (size_t k = n; k < N; ++k) SMi[SMp[k]] = (int)k;
  SM->ncol = SM->nrow = N;
  SM->p = SMp;
  SM->i = SMi;
  SM->x = SMx;
  SM->stype = -1;
  SM->xtype = CHOLMOD_REAL;
  SM->packed = TRUE;
  SM->sorted = TRUE;
  SM->nzmax = nnz;
  sm_rhs = new double[N]();
  sm_solution = new double[N]();
  return 0;
}

void SolverSettings::find_perturbation(double tol) {
  // reference :352-363: a diagonal smaller than tol in magnitude is replaced
  // by reg_diag in the caller's matrix and remembered
  for (size_t i = 0; i < AorSM->ncol; ++i) {
    if (std::abs(AorSM->x[AorSM->p[i]]) < tol) {
      perturbed_value pv;
      pv.col_idx = (int)i;
      pv.per_value = reg_diag;
      AorSM->x[AorSM->p[i]] = reg_diag;
      perturbed_diags.push_back(pv);
    }
  }
}

void SolverSettings::apply_perturbation(double tol) {
  // reference :365-372 (quasi-definite shift of the caller's matrix)
  for (size_t i = 0; i < AorSM->ncol; ++i) AorSM->x[AorSM->p[i]] += i < A->ncol ? tol : -tol;
}

// On the host ordered copy, with the reference's arithmetic (:374-394): the
// sign follows the ordered column index.  The plan's own refinement matrix
// is the exactly unperturbed one.
void SolverSettings::add_perturbation(double tol) {
  for (size_t i = 0; i < A_ord->ncol; ++i) {
    const size_t ord_col = (size_t)L->IPerm[i];
    A_ord->x[A_ord->p[ord_col]] += ord_col < A->ncol ? tol : -tol;
  }
}

void SolverSettings::remove_perturbation(double tol) {
  for (size_t i = 0; i < A_ord->ncol; ++i) {
    const size_t ord_col = (size_t)L->IPerm[i];
    A_ord->x[A_ord->p[ord_col]] -= ord_col < A->ncol ? tol : -tol;
  }
}

// Lower-stored P K P^T of the caller's matrix (current host values) under
// the current L->IPerm, as the reference's double transpose builds A_ord.
static CSC *ordered_copy(const CSC *K, const int *iperm) {
  const int N = (int)K->ncol;
  nqg::Csc k, lo;
  k.n = N;
  k.p.assign(K->p, K->p + N + 1);
  k.i.assign(K->i, K->i + K->p[N]);
  k.x.assign(K->x, K->x + K->p[N]);
  std::vector<int> ip(iperm, iperm + N);
  nqg::sym_permute(k, ip, &lo, nullptr);
  CSC *O = new CSC;
  O->ncol = O->nrow = N;
  O->nzmax = lo.nnz();
  O->p = new int[N + 1];
  O->i = new int[std::max<int64_t>(lo.nnz(), 1)];
  O->x = new double[std::max<int64_t>(lo.nnz(), 1)];
  std::copy(lo.p.begin(), lo.p.end(), O->p);
  std::copy(lo.i.begin(), lo.i.end(), O->i);
  std::copy(lo.x.begin(), lo.x.end(), O->x);
  O->stype = -1;
  return O;
}

int SolverSettings::symbolic_analysis() {
  psi->start = psi->tic();
  if (solver_mode == 0) {
    AorSM = A;
    base = 0;
    x = new double[std::max<size_t>(AorSM->ncol, 1)];
  } else {
    build_super_matrix();
    for (size_t i = 0; i < A->ncol; ++i) sm_rhs[i] = rhs[i];
    rhs = sm_rhs;
    x = sm_solution;
    AorSM = SM;
    base = C == nullptr ? A->ncol : A->ncol + C->nrow;
  }
  const int N = (int)AorSM->ncol;
  extra_cols = new int[std::max(N, 1)]();
  if (solver_mode == 1)
    for (int j = (int)base; j < N; ++j) extra_cols[j] = 1;
  std::vector<double> orig(AorSM->x, AorSM->x + AorSM->p[N]);
  if (regularization == 1) find_perturbation(reg_diag);
  else apply_perturbation(reg_diag);
  nqg_settings st;
  nqg_default_settings(&st);
  st.precision = gpu_precision ? NQG_FP32 : NQG_FP64;
  // FP32 factor: FP32 triangular solves inside flexible GMRES, whose residual
  // is the true FP64 one (left-preconditioned GMRES stops on the
  // preconditioned residual, which an FP32 factor can make small while the
  // true residual is not)
  st.solve_precision = gpu_precision ? NQG_FP32 : NQG_FP64;
  st.req_ref_iter = std::max(req_ref_iter, 0);
  st.max_inner_iter = std::max(max_inner_iter, 0);
  st.tol_abs = tol_abs;
  st.tol_rel = tol_rel;
  st.reg_diag = reg_diag;
  st.regularization = regularization == 1 ? 1 : 0;
  st.perturb_plus_cols = (int)A->ncol;
  std::copy(n_relax, n_relax + 3, st.n_relax);
  std::copy(z_relax, z_relax + 3, st.z_relax);
  last_gpu_status = nqg_plan_create(N, AorSM->p, AorSM->i, orig.data(), extra_cols, &st, &plan);
  psi->end = psi->toc();
  psi->analysis_time = psi->elapsed_time(psi->start, psi->end);
  if (last_gpu_status != NQG_OK) {
    std::cerr << "nasoq_gb300: symbolic analysis failed: " << nqg_status_str(last_gpu_status) << "\n";
    return 0;
  }
  // host mirror of the symbolic factor
  const nqg_symbolic *sh = nullptr;
  nqg_get_symbolic(plan, &sh);
  nqg_symbolic_info info;
  nqg_symbolic_get_info(sh, &info);
  L = new BCSC;
  L->n = N;
  L->nsuper = info.nsuper;
  L->ssize = info.ssize;
  L->xsize = info.xsize;
  L->nzmax = info.xsize;
  L->Perm = new int[N];
  L->IPerm = new int[N];
  L->ColCount = new int[N];
  L->Parent = new int[N];
  L->super = new int[info.nsuper + 1];
  L->col2Sup = new int[N];
  L->sParent = new int[std::max(info.nsuper, 1)];
  L->s = new int[std::max<int64_t>(info.ssize, 1)];
  std::vector<int64_t> lpi(info.nsuper + 1), colp(N + 1);
  std::vector<int> pex(N);
  nqg_symbolic_export(sh, L->Perm, L->IPerm, L->Parent, L->ColCount, L->super, L->sParent, L->col2Sup, lpi.data(),
                      L->s, colp.data(), pex.data());
  L->p = new size_t[N + 1];
  L->i_ptr = new size_t[N + 1];
  for (int j = 0; j <= N; ++j) L->p[j] = (size_t)colp[j];
  for (int j = 0; j < N; ++j) L->i_ptr[j] = (size_t)lpi[L->col2Sup[j]];
  L->i_ptr[N] = info.nsuper > 0 ? (size_t)lpi[info.nsuper] : 0;
  std::copy(pex.begin(), pex.end(), extra_cols);
  max_sup_wid = info.max_sup_wid;
  max_col = info.max_col;
  etree = L->Parent;
  d_val = new double[2 * std::max(N, 1)]();
  visible_cnt = new int[std::max(info.nsuper, 1)]();
  perm_piv = new int[std::max(N, 1)];
  marked = new bool[std::max<int64_t>(std::max<int64_t>(N, info.nsuper), 1)]();
  // ordered copy of the matrix (fill-reducing ordering of the analysis)
  A_ord = ordered_copy(AorSM, L->IPerm);
  allocate_workspace();
  if (solver_mode == 1) {
    const int ns = info.nsuper;
    atree = new int[std::max(ns, 1)];
    visible_sn = new bool[std::max(ns, 1)];
    std::copy(L->sParent, L->sParent + ns, atree);
    for (int l = 0; l < N; ++l) marked[l] = true;
    // children of every supernode in increasing order (reference populateChildren)
    child_sn_ptr = new int[ns + 1]();
    child_sn_no = new int[std::max(ns, 1)];
    num_sn_child = new int[std::max(ns, 1)]();
    for (int k = 0; k < ns; ++k)
      if (atree[k] >= 0) num_sn_child[atree[k]]++;
    for (int k = 0; k < ns; ++k) child_sn_ptr[k + 1] = child_sn_ptr[k] + num_sn_child[k];
    {
      std::vector<int> cnt(ns, 0);
      for (int l = 0; l < ns; ++l) {
        int p = atree[l];
        if (p >= 0) child_sn_no[child_sn_ptr[p] + cnt[p]++] = l;
      }
    }
    children_vec.assign(ns, {});
    for (int k = 0; k < ns; ++k)
      for (int q = child_sn_ptr[k]; q < child_sn_ptr[k + 1]; ++q) children_vec[k].push_back(child_sn_no[q]);
    for (int j = (int)base; j < N; ++j) delete_node_tree_simple(j);
    for (int m = 0; m < ns; ++m) {
      if (marked[m]) modified_sns.push_back(m);
      visible_sn[m] = marked[m];
    }
    architecture_related_params();
    // SM value index of every entry of every inequality constraint, in BT order
    const int mineq = B ? (int)B->nrow : 0;
    const_val_idx.assign(mineq, {});
    for (int v = 0; v < (int)A->ncol; ++v)
      for (int q = SM->p[v]; q < SM->p[v + 1]; ++q)
        if (SM->i[q] >= (int)base) const_val_idx[SM->i[q] - base].push_back(q);
  }
  return 1;
}

void SolverSettings::reset_symbolic_factor() {
  if (sm_rhs && SM) std::fill(sm_rhs, sm_rhs + SM->ncol, 0.0);
  if (sm_solution && SM) std::fill(sm_solution, sm_solution + SM->ncol, 0.0);
}

void SolverSettings::architecture_related_params() {
  // level sets of the supernodal tree for many-thread schedules (reference
  // :553-561): level of a supernode = longest path from a leaf below it,
  // supernodes of a level in increasing order (parents follow children in
  // the numbering, so one forward pass settles every level)
  delete[] s_level_ptr;
  delete[] s_level_set;
  s_level_ptr = s_level_set = nullptr;
  s_level_no = -1;
  if (num_thread <= thread_thresh || !L) return;
  const int ns = (int)L->nsuper;
  std::vector<int> lev(ns, 0);
  int nlev = ns > 0 ? 1 : 0;
  for (int k = 0; k < ns; ++k) {
    const int p = L->sParent[k];
    if (p >= 0) lev[p] = std::max(lev[p], lev[k] + 1);
    nlev = std::max(nlev, lev[k] + 1);
  }
  s_level_ptr = new int[nlev + 1]();
  s_level_set = new int[std::max(ns, 1)];
  for (int k = 0; k < ns; ++k) s_level_ptr[lev[k] + 1]++;
  for (int l = 0; l < nlev; ++l) s_level_ptr[l + 1] += s_level_ptr[l];
  std::vector<int> fill(s_level_ptr, s_level_ptr + nlev);
  for (int k = 0; k < ns; ++k) s_level_set[fill[lev[k]]++] = k;
  s_level_no = nlev;
}

void SolverSettings::allocate_workspace() {
  // the reference's sizes (:563-600): the update routine's integer and
  // dense scratch, two n-vectors, and the solve + GMRES scratch
  const size_t n = AorSM->ncol, ns = L ? L->nsuper : 0;
  const size_t upd_int = 4 * (size_t)(max_sup_wid + 1) + 2 * n + 3 * ns;
  const size_t upd_dbl = 2 * (size_t)(max_sup_wid + 1) * (size_t)(max_col + 1);
  ws_int_size = std::max(upd_int, 3 * n);
  ws_dbl_size = std::max(upd_dbl, 2 * n);
  size_t slve = 2 * n;
  if (max_iter > 0) {
    const size_t mi = (size_t)max_inner_iter;
    slve += 4 * (mi + 1) + (mi + 1) * (mi + 2) + 1 + n + (mi + 1) * n + 1;
  }
  ws_dbl_size = std::max(slve, ws_dbl_size);
  delete[] ws;
  delete[] ws_int;
  delete[] ws_zeroed;
  ws = new double[ws_dbl_size]();
  ws_int = new int[ws_int_size]();
  ws_zeroed = new double[(size_t)std::max(num_thread, 1) * n]();
}

int SolverSettings::numerical_factorization() {
  psi->start = psi->tic();
  last_gpu_status = nqg_factor(plan);
  psi->end = psi->toc();
  psi->fact_time += psi->elapsed_time(psi->start, psi->end);
  if (last_gpu_status < 0) {
    std::cerr << "nasoq_gb300: numerical factorization failed: " << nqg_status_str(last_gpu_status) << "\n";
    return -1;
  }
  return 1;
}

// ---- hidden-column bookkeeping of the QP mode (reference :770-907) -------
int SolverSettings::delete_node_tree_simple(int k) {
  const int ord_nod = L->IPerm[k];
  const int cur_sn = L->col2Sup[ord_nod];
  const int cur_par_sn = atree[cur_sn];
  if (cur_par_sn == -1) {
    for (int c : children_vec[cur_sn])
      if (atree[c] != INVISIBLE) atree[c] = cur_par_sn;
    children_vec[cur_sn].clear();
  } else if (cur_par_sn >= 0) {
    auto &pv = children_vec[cur_par_sn];
    pv.erase(std::remove(pv.begin(), pv.end(), cur_sn), pv.end());
    for (int c : children_vec[cur_sn])
      if (atree[c] != INVISIBLE) {
        atree[c] = cur_par_sn;
        children_vec[cur_par_sn].push_back(c);
      }
  }
  children_vec[cur_sn].clear();
  atree[cur_sn] = INVISIBLE;
  visible_sn[cur_sn] = false;
  marked[cur_sn] = false;
  extra_cols[ord_nod] = 1;
  return 1;
}

void SolverSettings::bfs_tree(int cur_sn) {
  std::queue<int> qu;
  qu.push(cur_sn);
  while (!qu.empty()) {
    int v = qu.front();
    qu.pop();
    for (int q = child_sn_ptr[v]; q < child_sn_ptr[v + 1]; ++q) {
      int cc = child_sn_no[q];
      qu.push(cc);
      if (visible_sn[cc] && atree[cc] == ROOT) {
        atree[cc] = cur_sn;
        children_vec[cur_sn].push_back(cc);
      }
    }
  }
}

int SolverSettings::add_node_tree_simple(int k) {
  const int ord_nod = L->IPerm[k];
  const int cur_sn = L->col2Sup[ord_nod];
  int k_par = L->sParent[cur_sn];
  while (k_par != -1) {  // first visible ancestor in the original tree
    if (atree[k_par] != INVISIBLE) break;
    k_par = L->sParent[k_par];
  }
  if (k_par != ROOT) {
    // children of k_par that lie below cur_sn move under cur_sn
    std::vector<int> keep;
    for (int orig_cc : children_vec[k_par]) {
      int cc = orig_cc;
      while (cc != -1) {
        if (cc == cur_sn) {
          children_vec[cur_sn].push_back(orig_cc);
          atree[orig_cc] = cur_sn;
          break;
        }
        cc = L->sParent[cc];
      }
      if (cc == -1) keep.push_back(orig_cc);
    }
    if (keep.size() != children_vec[k_par].size()) children_vec[k_par] = keep;
    children_vec[k_par].push_back(cur_sn);
  } else {
    bfs_tree(cur_sn);
  }
  atree[cur_sn] = k_par;
  visible_sn[cur_sn] = true;
  extra_cols[ord_nod] = 0;
  marked[cur_sn] = true;
  for (int q = child_sn_ptr[cur_sn]; q < child_sn_ptr[cur_sn + 1]; ++q) {
    int c = child_sn_no[q];
    if (atree[c] != INVISIBLE && atree[c] != cur_sn) {
      int pc = atree[c];
      if (pc != -1) {
        auto &pv = children_vec[pc];
        pv.erase(std::remove(pv.begin(), pv.end(), c), pv.end());
      }
      atree[c] = cur_sn;
      children_vec[cur_sn].push_back(c);
    }
  }
  return 1;
}

// etree_mod / child_ptr / child_no / num_child of the column elimination
// tree (children in increasing order), and a private assembly tree in the
// plain-solve mode, built when a column-tree edit first needs them
static void ensure_column_tree(SolverSettings &S) {
  const int N = (int)S.AorSM->ncol, ns = (int)S.L->nsuper;
  if (!S.etree_mod) {
    S.etree_mod = new int[std::max(N, 1)];
    std::copy(S.L->Parent, S.L->Parent + N, S.etree_mod);
  }
  if (!S.child_ptr) {
    S.child_ptr = new int[N + 1]();
    S.child_no = new int[std::max(N, 1)];
    S.num_child = new int[std::max(N, 1)]();
    for (int j = 0; j < N; ++j)
      if (S.L->Parent[j] >= 0) S.num_child[S.L->Parent[j]]++;
    for (int j = 0; j < N; ++j) S.child_ptr[j + 1] = S.child_ptr[j] + S.num_child[j];
    std::vector<int> fill(S.child_ptr, S.child_ptr + N);
    for (int j = 0; j < N; ++j)
      if (S.L->Parent[j] >= 0) S.child_no[fill[S.L->Parent[j]]++] = j;
  }
  if (!S.atree) {
    S.atree = new int[std::max(ns, 1)];
    std::copy(S.L->sParent, S.L->sParent + ns, S.atree);
  }
}

int SolverSettings::delete_node_tree(int k) {
  // reference :937-964: children of column k move to k's parent, k hidden;
  // its supernode is hidden once all of its columns are
  ensure_column_tree(*this);
  const int ord_nod = L->IPerm[k];
  const int par_k = etree_mod[ord_nod];
  const int cur_par_sn = par_k >= 0 ? L->col2Sup[par_k] : ROOT;
  for (int q = child_ptr[ord_nod]; q < child_ptr[ord_nod + 1]; ++q) {
    const int c = child_no[q];
    if (etree_mod[c] == INVISIBLE) continue;
    etree_mod[c] = par_k;
    const int csn = L->col2Sup[c];
    if (csn != cur_par_sn) atree[csn] = cur_par_sn;
  }
  etree_mod[ord_nod] = INVISIBLE;
  const int cur_sn = L->col2Sup[ord_nod];
  visible_cnt[cur_sn]++;
  if (L->super[cur_sn + 1] - L->super[cur_sn] == visible_cnt[cur_sn]) {
    atree[cur_sn] = INVISIBLE;
    marked[cur_sn] = false;
  }
  return 1;
}

int SolverSettings::add_node_tree(int k) {
  // reference :966-993: column k re-attaches below its first visible
  // ancestor and takes its visible children back
  ensure_column_tree(*this);
  const int ord_nod = L->IPerm[k];
  int k_par = etree[ord_nod];
  while (k_par != -1 && etree_mod[k_par] == INVISIBLE) k_par = etree[k_par];
  etree_mod[ord_nod] = k_par;
  const int cur_sn = L->col2Sup[ord_nod];
  for (int q = child_ptr[ord_nod]; q < child_ptr[ord_nod + 1]; ++q) {
    const int c = child_no[q];
    if (etree_mod[c] == INVISIBLE) continue;
    etree_mod[c] = ord_nod;
    const int csn = L->col2Sup[c];
    if (csn != cur_sn) atree[csn] = cur_sn;
  }
  return 1;
}

int SolverSettings::update_somod(std::vector<int> add_drp_const, const int n_rhs, const double *new_rhs) {
  const int dim = (int)AorSM->nrow;
  for (int k : add_drp_const)
    for (int j = 0; j < n_rhs; ++j) rhs[(k + base) + j * dim] = new_rhs[k + j * dim];
  return add_del_matrix_qp(1, add_drp_const);
}

int SolverSettings::downdate_somod(std::vector<int> add_drp_const, int n_rhs) {
  const int dim = (int)AorSM->nrow;
  for (int k : add_drp_const)
    for (int j = 0; j < n_rhs; ++j) rhs[(k + base) + j * dim] = 0;
  return add_del_matrix_qp(0, add_drp_const);
}

int SolverSettings::add_del_matrix_qp(int add_del, std::vector<int> add_drp_const) {
  // tree edits (SYM_REMOV): unhide on add, hide after the next update on drop
  for (int col : add_drp_const) {
    if (add_del) {
      add_node_tree_simple(col + (int)base);
      to_del = 0;
    } else {
      col_del = col + (int)base;
      to_del = 1;
    }
  }
  // mark the assembly-tree paths of every touched column and edit the values
  std::vector<long long> idx;
  std::vector<double> vals;
  for (int col : add_drp_const) {
    if (BT->p[col + 1] - BT->p[col] <= 0) continue;
    const int ord_col = L->IPerm[base + col];
    for (int s = L->col2Sup[ord_col]; s >= 0; s = atree[s]) modified_sns.push_back(s);
    const auto &vi = const_val_idx[col];
    int t = 0;
    for (int j = BT->p[col]; j < BT->p[col + 1]; ++j, ++t) {
      const int ord_row = L->IPerm[BT->i[j]];
      for (int s = L->col2Sup[ord_row]; s >= 0; s = atree[s]) modified_sns.push_back(s);
      idx.push_back(vi[t]);
      vals.push_back(add_del ? BT->x[j] : 0.0);
    }
  }
  if (!idx.empty()) {
    std::vector<int64_t> i64(idx.begin(), idx.end());
    last_gpu_status = nqg_edit_values(plan, (int)i64.size(), i64.data(), vals.data());
    for (size_t t = 0; t < idx.size(); ++t) SM->x[idx[t]] = vals[t];
  }
  std::sort(modified_sns.begin(), modified_sns.end());
  modified_sns.erase(std::unique(modified_sns.begin(), modified_sns.end()), modified_sns.end());
  for (int s : modified_sns) marked[s] = true;
  return 0;
}

int SolverSettings::update_factorization() {
  psi->start = psi->tic();
  last_gpu_status = nqg_refactor(plan, (int)modified_sns.size(), modified_sns.data());
  psi->end = psi->toc();
  psi->update_time += psi->elapsed_time(psi->start, psi->end);
  if (to_del) delete_node_tree_simple(col_del);
  return last_gpu_status >= 0 ? 1 : 0;
}

int SolverSettings::edit_matrix() { return 1; }
int SolverSettings::edit_rhs() { return 1; }
double *SolverSettings::edit_solve_rhs() { return nullptr; }
int SolverSettings::edit_update_factorization(int, std::vector<int>) { return 1; }
double *SolverSettings::update_solve() { return nullptr; }

double *SolverSettings::solve_only(const int n_rhs, double *rhs_in) {
  std::copy(rhs_in, rhs_in + AorSM->ncol, rhs);
  return solve_only();
}

double *SolverSettings::solve_only() {
  psi->start = psi->toc();
  const int N = (int)AorSM->ncol;
  if (solver_mode == 1) {
    const int ns = (int)L->nsuper;
    std::vector<uint8_t> vis(ns), hid(N);
    for (int s = 0; s < ns; ++s) vis[s] = visible_sn[s] ? 1 : 0;
    for (int j = 0; j < N; ++j) hid[j] = extra_cols[j] ? 1 : 0;
    nqg_set_visibility(plan, vis.data(), hid.data());
  }
  last_gpu_status = nqg_solve(plan, rhs, x);
  if (last_gpu_status < 0) std::cerr << "nasoq_gb300: solve failed: " << nqg_status_str(last_gpu_status) << "\n";
  nqg_timings t;
  nqg_get_timings(plan, &t);
  num_ref_iter = t.num_ref_iter;
  if (solver_mode == 1) {
    for (int s : modified_sns) marked[s] = false;
    modified_sns.clear();
  }
  psi->end = psi->toc();
  psi->solve_time += psi->elapsed_time(psi->start, psi->end);
  return x;
}

double *SolverSettings::iterative_ref_only() {
  const int N = (int)AorSM->ncol;
  if (solver_mode == 1) {
    const int ns = (int)L->nsuper;
    std::vector<uint8_t> vis(ns), hid(N);
    for (int s = 0; s < ns; ++s) vis[s] = visible_sn[s] ? 1 : 0;
    for (int j = 0; j < N; ++j) hid[j] = extra_cols[j] ? 1 : 0;
    nqg_set_visibility(plan, vis.data(), hid.data());
  }
  last_gpu_status = nqg_refine_only(plan, rhs, x);
  if (last_gpu_status < 0) std::cerr << "nasoq_gb300: refinement failed: " << nqg_status_str(last_gpu_status) << "\n";
  nqg_timings t;
  nqg_get_timings(plan, &t);
  num_ref_iter = t.num_ref_iter;
  return x;
}

void SolverSettings::reorder_matrix() {
  if (!plan || !L) return;
  const int N = (int)AorSM->ncol;
  nqg_get_factor(plan, nullptr, nullptr, L->Perm, nullptr);
  for (int i = 0; i < N; ++i) L->IPerm[L->Perm[i]] = i;
  free_csc(A_ord);
  A_ord = ordered_copy(AorSM, L->IPerm);
  for (int i = 0; i < N; ++i) perm_piv[i] = i;  // the pivots are part of L->Perm now
}

void SolverSettings::convert_supernode_to_simplicial() {
  // per column j of supernode s: its values start (j - first column) rows
  // into the supernode's column and use the supernode's row list from there
  if (!L) return;
  const int N = (int)L->n;
  if (!l_pb) {
    l_pb = new int[std::max(N, 1)];
    l_pe = new int[std::max(N, 1)];
    l_i = new int[std::max<size_t>(L->xsize, 1)];
    own_simplicial = true;
  }
  for (size_t sn = 0; sn < L->nsuper; ++sn) {
    const int c0 = L->super[sn], c1 = L->super[sn + 1];
    for (int j = c0; j < c1; ++j) {
      l_pb[j] = (int)L->p[j] + (j - c0);
      l_pe[j] = (int)L->p[j + 1];
      size_t kk = L->i_ptr[c0] + (size_t)(j - c0);
      for (int k = l_pb[j]; k < l_pe[j]; ++k, ++kk) l_i[k] = L->s[kk];
    }
  }
}

void SolverSettings::copy_lsuper_to_l() {}  // an empty routine in the reference too (:1519-1521)

int SolverSettings::check_ldlt_factor() {
  if (!download_factor()) return 0;
  const size_t N = L->n;
  for (size_t i = 0; i < L->xsize; ++i)
    if (!std::isfinite(valL[i])) return 0;
  for (size_t i = 0; i < 2 * N; ++i)
    if (!std::isfinite(d_val[i])) return 0;
  std::vector<char> seen(N, 0);
  for (size_t i = 0; i < N; ++i) {
    const int p = L->Perm[i];
    if (p < 0 || (size_t)p >= N || seen[p]) return 0;
    seen[p] = 1;
  }
  return 1;
}

void SolverSettings::set_diags(double d) {
  // The GPU plan keeps the perturbed values for the factorization and the
  // unperturbed ones for the refinement residual; this only updates the host
  // copy of the ordered matrix.
  for (auto &pv : perturbed_diags) {
    int ord_col = L->IPerm[pv.col_idx];
    A_ord->x[A_ord->p[ord_col]] = d == 0 ? 0 : pv.per_value;
  }
}

void SolverSettings::compute_norms() {
  // infinity norms of A, x, rhs and of the residual rhs - A x (unperturbed A)
  const int N = (int)AorSM->ncol;
  std::vector<double> ax(N, 0.0), rowsum(N, 0.0);
  std::vector<double> vals(AorSM->x, AorSM->x + AorSM->p[N]);
  for (auto &pv : perturbed_diags) vals[AorSM->p[pv.col_idx]] = 0.0;
  for (int j = 0; j < N; ++j)
    for (int q = AorSM->p[j]; q < AorSM->p[j + 1]; ++q) {
      int i = AorSM->i[q];
      ax[i] += vals[q] * x[j];
      rowsum[i] += std::abs(vals[q]);
      if (i != j) {
        ax[j] += vals[q] * x[i];
        rowsum[j] += std::abs(vals[q]);
      }
    }
  x_l1 = rhs_l1 = res_l1 = A_l1 = 0;
  for (int i = 0; i < N; ++i) {
    x_l1 = std::max(x_l1, std::abs(x[i]));
    rhs_l1 = std::max(rhs_l1, std::abs(rhs[i]));
    res_l1 = std::max(res_l1, std::abs(rhs[i] - ax[i]));
    A_l1 = std::max(A_l1, rowsum[i]);
  }
}

double SolverSettings::backward_error() {
  compute_norms();
  bwd_err = (A_l1 * x_l1 + rhs_l1 > 0) ? res_l1 / (A_l1 * x_l1 + rhs_l1) : 0;
  return bwd_err;
}

int SolverSettings::download_factor() {
  if (!plan || !L) return 0;
  if (!valL) valL = new double[std::max<size_t>(L->xsize, 1)];
  int rc = nqg_get_factor(plan, valL, d_val, L->Perm, L->s);
  for (size_t i = 0; i < L->n; ++i) L->IPerm[L->Perm[i]] = (int)i;
  return rc == NQG_OK ? 1 : 0;
}

}  // namespace nasoq
