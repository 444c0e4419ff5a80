/* Oracle driver: runs the reference NASOQ library (compiled out-of-tree from
 * its own sources by oracle/Makefile) through its public API and dumps every
 * array the GPU build is checked against.  Test infrastructure only: it is
 * built and run in the development container, never on the product path.
 *
 *   ref_dump lbl  <in.nqa> <out.nqa>   SolverSettings mode-0 flow
 *                                      (examples/lbl_main.cpp:34-43)
 *   ref_dump qp   <in.nqa> <out.nqa>   Nasoq::solve() steps (src/nasoq.cpp:656-710)
 *   ref_dump smp  <in.yml> <out.nqa>   SMP file -> NASOQ inequality form
 *                                      (nasoq_driver.cpp:87-89)
 */
#include <cmath>
#include <cstdlib>
#include <iostream>
#include <string>
#include <vector>

#include "nasoq/QP/linear_solver_wrapper.h"
#include "nasoq/nasoq.h"
#include "nqa_io.h"
#include <mp_format_converter.h>

using namespace nasoq;

static void dump_symbolic(nqa::File &out, const std::string &pfx, SolverSettings *ss, size_t n) {
  BCSC *L = ss->L;
  out.put(pfx + "Perm", L->Perm, n);
  out.put(pfx + "IPerm", L->IPerm, n);
  out.put(pfx + "Parent", L->Parent, n);
  out.put(pfx + "ColCount", L->ColCount, n);
  out.put(pfx + "super", L->super, L->nsuper + 1);
  out.put(pfx + "sParent", L->sParent, L->nsuper);
  out.put(pfx + "col2Sup", L->col2Sup, n);
  std::vector<int64_t> iptr(n + 1), p(n + 1);
  for (size_t i = 0; i <= n; ++i) {
    iptr[i] = (int64_t)L->i_ptr[i];
    p[i] = (int64_t)L->p[i];
  }
  out.put(pfx + "i_ptr", iptr);
  out.put(pfx + "p", p);
  out.put(pfx + "s", L->s, L->i_ptr[n]);
  out.put(pfx + "extra_cols", ss->extra_cols, n);
  out.put_scalar(pfx + "xsize", (double)L->xsize);
  out.put_scalar(pfx + "max_sup_wid", (double)ss->max_sup_wid);
  out.put_scalar(pfx + "max_col", (double)ss->max_col);
}

static int run_lbl(const nqa::File &in, nqa::File &out) {
  std::vector<int> Ap = in.vec<int>("Ap"), Ai = in.vec<int>("Ai");
  std::vector<double> Ax = in.vec<double>("Ax"), rhs = in.vec<double>("rhs");
  size_t n = Ap.size() - 1;
  CSC *H = new CSC;
  H->nzmax = Ap[n];
  H->ncol = H->nrow = n;
  H->p = Ap.data();
  H->i = Ai.data();
  H->x = Ax.data();
  H->stype = -1;
  H->packed = 1;
  H->sorted = 1;
  H->nz = NULL;
  std::vector<double> q(rhs);
  auto *lbl = new SolverSettings(H, q.data());
  lbl->ldl_variant = (int)in.scalar("ldl_variant", 2);
  lbl->req_ref_iter = (int)in.scalar("req_ref_iter", 2);
  lbl->max_inner_iter = (int)in.scalar("max_inner_iter", 2);
  lbl->solver_mode = 0;
  lbl->reg_diag = in.scalar("reg_diag", 1e-9);
  lbl->tol_abs = in.scalar("tol_abs", 1e-15);
  lbl->tol_rel = in.scalar("tol_rel", 1e-15);
  if (!lbl->symbolic_analysis()) return 2;
  dump_symbolic(out, "sym_", lbl, n);
  out.put("Ax_perturbed", Ax);
  lbl->numerical_factorization();
  BCSC *L = lbl->L;
  out.put("valL", lbl->valL, L->xsize);
  out.put("d_val", lbl->d_val, 2 * n);
  out.put("fac_Perm", L->Perm, n);
  out.put("fac_s", L->s, L->i_ptr[n]);
  out.put("perm_piv", lbl->perm_piv, n);
  int keep = lbl->req_ref_iter;
  lbl->req_ref_iter = 0;
  double *x = lbl->solve_only();
  out.put("x_noref", x, n);
  lbl->req_ref_iter = keep;
  x = lbl->solve_only();
  out.put("x", x, n);
  out.put_scalar("num_ref_iter", lbl->num_ref_iter);
  delete[] x;
  delete lbl;
  delete H;
  return 0;
}

static int run_qp(const nqa::File &in, nqa::File &out) {
  std::vector<int> Hp = in.vec<int>("Hp"), Hi = in.vec<int>("Hi");
  std::vector<double> Hx = in.vec<double>("Hx"), q = in.vec<double>("q");
  std::vector<int> Ap = in.vec<int>("Ap"), Ai = in.vec<int>("Ai");
  std::vector<double> Axv = in.vec<double>("Ax"), b = in.vec<double>("b");
  std::vector<int> Cp = in.vec<int>("Cp"), Ci = in.vec<int>("Ci");
  std::vector<double> Cx = in.vec<double>("Cx"), d = in.vec<double>("d");
  size_t n = Hp.size() - 1;
  size_t meq = (size_t)in.scalar("meq", 0), mineq = (size_t)in.scalar("mineq", 0);
  if (Ai.empty()) Ai.push_back(0);
  if (Axv.empty()) Axv.push_back(0);
  if (b.empty()) b.push_back(0);
  if (Ci.empty()) Ci.push_back(0);
  if (Cx.empty()) Cx.push_back(0);
  if (d.empty()) d.push_back(0);
  Nasoq *qm;
  if (meq > 0)
    qm = new Nasoq(n, Hp.data(), Hi.data(), Hx.data(), q.data(), meq, n, Ap.data(), Ai.data(), Axv.data(), b.data(),
                   mineq, n, Cp.data(), Ci.data(), Cx.data(), d.data());
  else
    qm = new Nasoq(n, Hp.data(), Hi.data(), Hx.data(), q.data(), mineq, n, Cp.data(), Ci.data(), Cx.data(),
                   d.data());
  qm->diag_perturb = in.scalar("diag_perturb", 1e-9);
  qm->eps_abs = in.scalar("eps_abs", 1e-6);
  qm->max_iter = (int)in.scalar("max_iter", 2);
  qm->stop_tol = in.scalar("stop_tol", 1e-15);
  qm->max_iter_nas = (int)in.scalar("max_iter_nas", 200000);
  int variant = (int)in.scalar("variant", 0);
  qm->variant = (nasoq_mode)variant;
  qm->scaling = (int)in.scalar("scaling", 0);
  // Nasoq::solve() for Fixed/AUTO/PREDET, unrolled so the symbolic state can
  // be dumped between symbolic_QP and initialize_x.
  qm->warm_start = 0;
  qm->auto_reg_en = variant == AUTO ? 2 : (variant == Fixed ? 1 : 0);
  if (qm->scaling > 0) qm->scale_data();
  qm->symbolic_QP();
  dump_symbolic(out, "sym_", qm->ss, qm->ss->SM->ncol);
  qm->initialize_x();
  int status = qm->numeric_QP();
  if (qm->scaling > 0) {
    qm->unscale_data();
    qm->unscale_solution();
  }
  qm->compute_objective();
  int ret = qm->check_solve_status(status);
  qm->detect_solver_name();
  out.put_scalar("status", ret);
  out.put_scalar("converged", status);
  out.put_scalar("num_iter", qm->num_iter);
  out.put("x", qm->primal_vars, n);
  if (meq > 0) out.put("y", qm->dual_vars_eq, meq);
  out.put("z", qm->dual_vars, mineq);
  out.put_scalar("objective", qm->objective);
  out.put_scalar("primal_obj", qm->primal_obj);
  out.put_scalar("dual_obj", qm->dual_obj);
  out.put_scalar("lag_res", qm->lag_res);
  out.put_scalar("cons_sat_norm", qm->cons_sat_norm);
  out.put_scalar("non_negativity_infn", qm->non_negativity_infn);
  out.put_scalar("complementarity_infn", qm->complementarity_infn);
  out.put_scalar("outer_iter_ref", qm->outer_iter_ref);
  out.put_scalar("inner_iter_ref", qm->inner_iter_ref);
  out.put_scalar("diag_perturb_used", qm->diag_perturb);
  out.put_scalar("stop_tol_used", qm->stop_tol);
  out.put("active_set", qm->active_set);
  delete qm;
  return 0;
}

static void put_csc(nqa::File &out, const std::string &pfx, format::CSC *A, size_t ncol) {
  if (!A || A->m == 0 || A->n == 0) {
    std::vector<int> p(ncol + 1, 0);
    out.put(pfx + "p", p);
    out.put(pfx + "i", std::vector<int>());
    out.put(pfx + "x", std::vector<double>());
    return;
  }
  out.put(pfx + "p", A->p, A->n + 1);
  out.put(pfx + "i", A->i, A->p[A->n]);
  out.put(pfx + "x", A->x, A->p[A->n]);
}

static int run_smp(const std::string &path, nqa::File &out) {
  auto *QPFC = new format::QPFormatConverter();
  if (!QPFC->load_smp(path)) return 3;
  QPFC->smp_to_ie();
  auto *ie = QPFC->ief_;
  size_t n = ie->H->n;
  put_csc(out, "H", ie->H, n);
  out.put("q", ie->q->a, n);
  size_t meq = ie->A ? ie->A->m : 0, mineq = ie->C ? ie->C->m : 0;
  out.put_scalar("meq", (double)meq);
  out.put_scalar("mineq", (double)mineq);
  put_csc(out, "A", meq ? ie->A : nullptr, n);
  if (meq) out.put("b", ie->b->a, meq); else out.put("b", std::vector<double>());
  put_csc(out, "C", mineq ? ie->C : nullptr, n);
  if (mineq) out.put("d", ie->d->a, mineq); else out.put("d", std::vector<double>());
  delete QPFC;
  return 0;
}

int main(int argc, char **argv) {
  if (argc < 4) {
    std::cerr << "usage: ref_dump lbl|qp|smp <in> <out.nqa>\n";
    return 1;
  }
  std::string cmd = argv[1];
  nqa::File out;
  int rc = 1;
  if (cmd == "smp") {
    rc = run_smp(argv[2], out);
  } else {
    nqa::File in;
    in.load(argv[2]);
    if (cmd == "lbl") rc = run_lbl(in, out);
    else if (cmd == "qp") rc = run_qp(in, out);
  }
  if (rc == 0) out.save(argv[3]);
  return rc;
}
