// A caller of nasoq::SolverSettings written against the reference's public
// header (include/nasoq/QP/linear_solver_wrapper.h), built unchanged against
// this library's include/ and libnasoq_gb300.so.  It walks both solver modes
// and the maintenance methods, and prints every result as "key: values" for
// the test to check against dense solves.
#include <nasoq/QP/linear_solver_wrapper.h>

#include <cmath>
#include <cstdio>
#include <vector>

static void print_vec(const char *key, const double *v, int n) {
  std::printf("%s:", key);
  for (int i = 0; i < n; ++i) std::printf(" %.17g", v[i]);
  std::printf("\n");
}

static nasoq::CSC *make_csc(int nrow, int ncol, std::vector<int> &p, std::vector<int> &i, std::vector<double> &x,
                            int stype) {
  auto *A = new nasoq::CSC;
  A->nrow = nrow;
  A->ncol = ncol;
  A->nzmax = x.size();
  A->p = p.data();
  A->i = i.data();
  A->x = x.data();
  A->stype = stype;
  A->packed = 1;
  return A;
}

int main() {
  // ---- mode 0: one symmetric indefinite system, two right-hand sides
  // K = [4 1 0 1; 1 3 1 0; 0 1 -2 1; 1 0 1 -3], lower CSC
  std::vector<int> Kp = {0, 3, 5, 7, 8}, Ki = {0, 1, 3, 1, 2, 2, 3, 3};
  std::vector<double> Kx = {4, 1, 1, 3, 1, -2, 1, -3};
  std::vector<double> b1 = {1, 2, 3, 4}, b2 = {-1, 0.5, 2, 0};
  nasoq::CSC *K = make_csc(4, 4, Kp, Ki, Kx, -1);
  auto *lbl = new nasoq::SolverSettings(K, b1.data());
  lbl->ldl_variant = 2;
  lbl->req_ref_iter = 2;
  lbl->solver_mode = 0;
  lbl->reg_diag = std::pow(10, -9);
  if (lbl->symbolic_analysis() != 1) return 2;
  if (lbl->numerical_factorization() != 1) return 3;
  double *x = lbl->solve_only();
  print_vec("x1", x, 4);
  lbl->solve_only(1, b2.data());
  print_vec("x2", x, 4);
  std::printf("bwd_err: %.17g\n", lbl->backward_error());
  // refinement alone, from x = rhs (= b2 now)
  x = lbl->iterative_ref_only();
  print_vec("xr", x, 4);
  std::printf("check: %d\n", lbl->check_ldlt_factor());
  lbl->reorder_matrix();
  std::printf("perm:");
  for (int i = 0; i < 4; ++i) std::printf(" %d", lbl->L->Perm[i]);
  std::printf("\n");
  lbl->convert_supernode_to_simplicial();
  long long cnt = 0;
  for (int j = 0; j < 4; ++j) cnt += lbl->l_pe[j] - lbl->l_pb[j];
  std::printf("simplicial_nnz: %lld\n", cnt);
  lbl->num_thread = 64;
  lbl->architecture_related_params();
  std::printf("levels: %d %d %zu\n", lbl->s_level_no, lbl->s_level_no > 0 ? lbl->s_level_ptr[lbl->s_level_no] : -1,
              lbl->L->nsuper);
  lbl->allocate_workspace();
  std::printf("workspace: %zu %zu\n", lbl->ws_dbl_size, lbl->ws_int_size);
  std::printf("stubs: %d %d %d %d %d\n", lbl->edit_matrix(), lbl->edit_rhs(), lbl->edit_solve_rhs() == nullptr,
              lbl->edit_update_factorization(1, {}), lbl->update_solve() == nullptr);
  delete lbl;

  // ---- mode 1: H x = q with inequality rows switched on and off (SoMod)
  // H = [3 1; 1 2], rows of B: [1 0], [1 1]
  std::vector<int> Hp = {0, 2, 3}, Hi = {0, 1, 1};
  std::vector<double> Hx = {3, 1, 2}, q = {-1, -2};
  std::vector<int> Bp = {0, 2, 3}, Bi = {0, 1, 1};
  std::vector<double> Bx = {1, 1, 1}, d = {0.5, 1.0};
  nasoq::CSC *H = make_csc(2, 2, Hp, Hi, Hx, -1);
  nasoq::CSC *B = make_csc(2, 2, Bp, Bi, Bx, 0);
  auto *qp = new nasoq::SolverSettings(H, q.data(), B, d.data());
  qp->req_ref_iter = 2;
  qp->solver_mode = 1;
  qp->reg_diag = std::pow(10, -9);
  if (qp->symbolic_analysis() != 1) return 4;
  if (qp->numerical_factorization() != 1) return 5;
  x = qp->solve_only();
  print_vec("m1_none", x, 4);
  std::vector<int> inds = {0};
  qp->update_somod(inds, 1, d.data());
  qp->update_factorization();
  x = qp->solve_only();
  print_vec("m1_row0", x, 4);
  inds = {1};
  qp->update_somod(inds, 1, d.data());
  qp->update_factorization();
  x = qp->solve_only();
  print_vec("m1_rows01", x, 4);
  inds = {0};
  qp->downdate_somod(inds, 1);
  qp->update_factorization();
  x = qp->solve_only();
  print_vec("m1_row1", x, 4);
  delete qp;
  delete K;
  delete H;
  delete B;
  return 0;
}
