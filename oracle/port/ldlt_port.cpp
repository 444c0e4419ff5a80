/* Oracle restatement (CPU, FP64) of the reference's numeric LBL path, used
 * ONLY as a checker in tests and as the timed CPU baseline of the benchmark.
 * Parity: pinned against the reference built from its sources (oracle/_ref)
 * on the golden fixtures (tests/test_oracle_port.py).
 *
 * It follows, operation by operation:
 *   ldl_left_sn_02_v2        src/ldl/Serial_blocked_ldl_02_2.cpp:18-183
 *   ereach_sn                src/common/Reach.cpp:96-125
 *   blocked_2by2_mult        src/common/Sym_BLAS.cpp:573-599
 *   reorder_after_sytrf      src/common/Sym_BLAS.cpp:128-196
 *   blocked_2by2_solver      src/common/Sym_BLAS.cpp:492-529
 *   row_reordering           src/common/Sym_BLAS.cpp:327-490 (restated as a
 *                            rename-and-sort of each affected row segment)
 *   reorder_matrix           src/QP/linear_solver_wrapper.cpp:1432-1460
 *   blockedLsolve/LTsolve    src/triangularSolve/Triangular_BCSC.cpp:20-118
 *   pmgmres_ldlt_auto        src/gmres/mgmres.cpp:1015-1211
 *   spmv_csc_sym_one_int     src/matrixVector/spmv_CSC.cpp:26-102
 * and, for the QP path (nqp_qp_solve), the active-set loop of Nasoq::numeric_QP
 * (src/nasoq.cpp:478-610) over the SoMod partial refactorization
 * (update_ldl_left_sn_02_v2, src/ldl/Serial_update_ldl.cpp:18-277) and the
 * masked solves (solve_phase.cpp:133-161).
 * BLAS/LAPACK (dgemm, dtrsm, dgemv, dscal, dsytrf, dlapmt) come from the
 * OpenBLAS build bundled with SciPy, resolved with dlopen at run time.
 */
#include <dlfcn.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>

namespace {

enum { RowMajor = 101, ColMajor = 102, NoTrans = 111, Trans = 112, ConjTrans = 113, Upper = 121, Lower = 122,
       NonUnit = 131, Unit = 132, Left = 141, Right = 142 };

typedef void (*dgemm_t)(int, int, int, int, int, int, double, const double *, int, const double *, int, double,
                        double *, int);
typedef void (*dtrsm_t)(int, int, int, int, int, int, int, double, const double *, int, double *, int);
typedef void (*dgemv_t)(int, int, int, int, double, const double *, int, const double *, int, double, double *,
                        int);
typedef void (*dscal_t)(int, double, double *, int);
typedef int (*dsytrf_t)(int, char, int, double *, int, int *);
typedef int (*dlapmt_t)(int, int, int, int, double *, int, int *);
typedef void (*setthr_t)(int);

struct Blas {
  dgemm_t gemm = nullptr;
  dtrsm_t trsm = nullptr;
  dgemv_t gemv = nullptr;
  dscal_t scal = nullptr;
  dsytrf_t sytrf = nullptr;
  dlapmt_t lapmt = nullptr;
  setthr_t setthreads = nullptr;
} B;

template <class F> bool sym(void *h, const char *a, const char *b, F &out) {
  void *p = dlsym(h, a);
  if (!p) p = dlsym(h, b);
  out = reinterpret_cast<F>(p);
  return p != nullptr;
}

using clk = std::chrono::steady_clock;

// ---------------------------------------------------------------------------
struct Sym {
  int n, ns;
  const int *perm, *super, *sparent, *col2sup;
  const int64_t *lpi, *colp;
};

void sym_permute_lower(int n, const int *Ap, const int *Ai, const double *Ax, const std::vector<int> &pinv,
                       std::vector<int> &Cp, std::vector<int> &Ci, std::vector<double> &Cx) {
  // lower-stored C = P A P^T with sorted rows
  std::vector<int64_t> cnt(n + 1, 0);
  for (int j = 0; j < n; ++j)
    for (int q = Ap[j]; q < Ap[j + 1]; ++q) {
      int a = pinv[Ai[q]], b = pinv[j];
      cnt[std::min(a, b) + 1]++;
    }
  Cp.assign(n + 1, 0);
  for (int j = 0; j < n; ++j) Cp[j + 1] = Cp[j] + (int)cnt[j + 1];
  Ci.resize(Cp[n]);
  Cx.resize(Cp[n]);
  std::vector<int> pos(Cp.begin(), Cp.end() - 1);
  for (int j = 0; j < n; ++j)
    for (int q = Ap[j]; q < Ap[j + 1]; ++q) {
      int a = pinv[Ai[q]], b = pinv[j];
      int c = std::min(a, b), r = std::max(a, b);
      int t = pos[c]++;
      Ci[t] = r;
      Cx[t] = Ax[q];
    }
  for (int j = 0; j < n; ++j) {
    std::vector<std::pair<int, double>> v;
    for (int q = Cp[j]; q < Cp[j + 1]; ++q) v.emplace_back(Ci[q], Cx[q]);
    std::sort(v.begin(), v.end(), [](auto &x, auto &y) { return x.first < y.first; });
    for (int q = Cp[j], t = 0; q < Cp[j + 1]; ++q, ++t) {
      Ci[q] = v[t].first;
      Cx[q] = v[t].second;
    }
  }
}

// upper-stored pattern (rows of the lower matrix)
void transpose_pattern(int n, const std::vector<int> &Lp, const std::vector<int> &Li, std::vector<int> &Up,
                       std::vector<int> &Ui) {
  Up.assign(n + 1, 0);
  for (int q = 0; q < Lp[n]; ++q) Up[Li[q] + 1]++;
  for (int j = 0; j < n; ++j) Up[j + 1] += Up[j];
  Ui.resize(Lp[n]);
  std::vector<int> pos(Up.begin(), Up.end() - 1);
  for (int j = 0; j < n; ++j)
    for (int q = Lp[j]; q < Lp[j + 1]; ++q) Ui[pos[Li[q]]++] = j;
}

int ereach(int ns, const std::vector<int> &Up, const std::vector<int> &Ui, int c1, int c2, const int *col2sup,
           const int *parent, std::vector<int> &stack, std::vector<int> &mark) {
  int top = ns;
  std::vector<int> path;
  mark[col2sup[c1]] = 1;
  for (int k = c1; k < c2; ++k)
    for (int q = Up[k]; q < Up[k + 1]; ++q) {
      int r = Ui[q];
      if (r > k) continue;
      int i = col2sup[r];
      path.clear();
      while (i >= 0 && !mark[i]) {
        path.push_back(i);
        mark[i] = 1;
        i = parent[i];
      }
      for (int t = (int)path.size() - 1; t >= 0; --t) stack[--top] = path[t];
    }
  for (int t = top; t < ns; ++t) mark[stack[t]] = 0;
  mark[col2sup[c1]] = 0;
  return top;
}

struct Factor {
  std::vector<double> L, D;
  std::vector<int> ls, perm;  // ls after row renaming, combined permutation
};

// Upper-stored pattern of P A P^T in the entry order of the reference's
// permuted symmetric transpose (ptranspose, src/common/Transpose.cpp:7-131):
// column c lists the rows contributed by earlier columns in increasing order,
// then the entries of original column perm[c] in original-row order.  The
// elimination-reach order, and with it the summation order of the Schur
// updates, follows this order.
void ordered_upper_like_reference(int n, const int *Ap0, const int *Ai0, const int *perm, const std::vector<int> &pinv,
                                  std::vector<int> &Up, std::vector<int> &Ui) {
  Up.assign(n + 1, 0);
  for (int j = 0; j < n; ++j) {
    int jold = perm[j];
    for (int q = Ap0[jold]; q < Ap0[jold + 1]; ++q) {
      int iold = Ai0[q];
      if (iold < jold) continue;
      int i = pinv[iold];
      Up[std::max(i, j) + 1]++;
    }
  }
  for (int j = 0; j < n; ++j) Up[j + 1] += Up[j];
  Ui.resize(Up[n]);
  std::vector<int> wi(Up.begin(), Up.end() - 1);
  for (int j = 0; j < n; ++j) {
    int jold = perm[j];
    for (int q = Ap0[jold]; q < Ap0[jold + 1]; ++q) {
      int iold = Ai0[q];
      if (iold < jold) continue;
      int i = pinv[iold];
      if (i > j) Ui[wi[i]++] = j;
      else Ui[wi[j]++] = i;
    }
  }
}

int factorize(const Sym &S, const std::vector<int> &Ap, const std::vector<int> &Ai, const std::vector<double> &Ax,
              const std::vector<int> &Up, const std::vector<int> &Ui, std::vector<int> ls, Factor &F) {
  const int n = S.n, ns = S.ns;
  F.L.assign(S.colp[n] > 0 ? S.colp[n] : 1, 0.0);
  F.D.assign(2 * (size_t)n, 0.0);
  int smax = 0, cmax = 0;
  for (int s = 0; s < ns; ++s) {
    smax = std::max(smax, S.super[s + 1] - S.super[s]);
    cmax = std::max<int>(cmax, (int)(S.lpi[s + 1] - S.lpi[s]));
  }
  std::vector<double> contribs((size_t)(smax + 1) * (cmax + 1)), trn((size_t)(smax + 1) * (cmax + 1));
  std::vector<int> map(n), stack(ns), mark(ns, 0), ipiv(smax + 1), swapv(smax + 1), tmpsort(smax + 1),
      pivots(smax + 1);
  std::vector<int> perm_piv(n);
  std::iota(perm_piv.begin(), perm_piv.end(), 0);
  std::vector<int> pivoted_sn;
  double *Lv = F.L.data();
  double *D = F.D.data();
  for (int s = 0; s < ns; ++s) {
    const int c0 = S.super[s], c1 = S.super[s + 1], w = c1 - c0;
    const int nr = (int)(S.lpi[s + 1] - S.lpi[s]);
    const int *rows = ls.data() + S.lpi[s];
    for (int i = 0; i < nr; ++i) map[rows[i]] = i;
    double *cur = Lv + S.colp[c0];
    for (int i = c0; i < c1; ++i)
      for (int q = Ap[i]; q < Ap[i + 1]; ++q) Lv[S.colp[i] + map[Ai[q]]] = Ax[q];
    int top = ereach(ns, Up, Ui, c0, c1, S.col2sup, S.sparent, stack, mark);
    for (int t = top; t < ns; ++t) {
      const int d = stack[t];
      const int dc0 = S.super[d], dw = S.super[d + 1] - dc0;
      const int dnr = (int)(S.lpi[d + 1] - S.lpi[d]);
      const int *drows = ls.data() + S.lpi[d];
      int lb = 0, ub = 0;
      bool sw = true;
      for (int j = 0; j < dnr; ++j) {
        if (drows[j] >= c0 && sw) {
          lb = j;
          sw = false;
        }
        if (drows[j] < c1 && !sw) ub = j;
      }
      const int nSupRs = dnr - lb, ndrow1 = ub - lb + 1;
      const double *src = Lv + S.colp[dc0] + lb;
      // T = L_d D_d on the rows from lb (1x1 and 2x2 blocks)
      const double *Dd = D + dc0;
      for (int l = 0; l < dw;) {
        if (Dd[l + n] == 0) {
          double tmp = Dd[l];
          for (int l1 = 0; l1 < nSupRs; ++l1) trn[(size_t)l * nSupRs + l1] = tmp * src[(size_t)l * dnr + l1];
          l++;
        } else {
          double d1 = Dd[l], d2 = Dd[l + 1], e = Dd[l + n];
          for (int l1 = 0; l1 < nSupRs; ++l1) {
            trn[(size_t)l * nSupRs + l1] = d1 * src[(size_t)l * dnr + l1] + e * src[(size_t)(l + 1) * dnr + l1];
            trn[(size_t)(l + 1) * nSupRs + l1] = e * src[(size_t)l * dnr + l1] + d2 * src[(size_t)(l + 1) * dnr + l1];
          }
          l += 2;
        }
      }
      B.gemm(ColMajor, NoTrans, ConjTrans, nSupRs, ndrow1, dw, 1.0, trn.data(), nSupRs, src, dnr, 0.0,
             contribs.data(), nSupRs);
      for (int i = 0; i < ndrow1; ++i) {
        const int col = map[drows[i + lb]];
        for (int j = i; j < nSupRs; ++j) cur[(size_t)col * nr + map[drows[j + lb]]] -= contribs[(size_t)i * nSupRs + j];
      }
    }
    B.sytrf(ColMajor, 'L', w, cur, nr, ipiv.data());
    // LAPACK pivots -> explicit-form row swaps + local permutation
    bool skip = false, perm_any = false;
    for (int j = 0; j < w; ++j) {
      swapv[j] = j;
      tmpsort[j] = j;
    }
    for (int i = 0; i < w; ++i) {
      if (skip) {
        pivots[i] = 0;
        skip = false;
        continue;
      }
      int cv = ipiv[i];
      if (cv > 0) {
        if (cv != i + 1) {
          swapv[i] = swapv[cv - 1];
          perm_any = true;
        }
        pivots[i] = 1;
      } else {
        if (-cv != i + 2) {
          swapv[i + 1] = swapv[-cv - 1];
          perm_any = true;
        }
        pivots[i] = 2;
        D[c0 + i + n] = cur[(size_t)i * nr + i + 1];
        cur[(size_t)i * nr + i + 1] = 0.0;
        skip = true;
      }
    }
    if (perm_any)
      for (int k = 0; k < w; ++k) {
        int cv = swapv[k];
        if (k != cv) {
          int len = pivots[k] == 0 ? k - 1 : k;
          for (int c = 0; c < len; ++c) std::swap(cur[k + (size_t)c * nr], cur[cv + (size_t)c * nr]);
          std::swap(tmpsort[k], tmpsort[cv]);
        }
      }
    const int rowNo = nr - w;
    if (perm_any) {
      std::vector<int> k1(w);
      for (int m = 0; m < w; ++m) k1[m] = tmpsort[m] + 1;
      B.lapmt(ColMajor, 1, rowNo, w, cur + w, nr, k1.data());
      pivoted_sn.push_back(s);
    }
    for (int m = 0; m < w; ++m) perm_piv[c0 + m] = c0 + tmpsort[m];
    for (int l = 0; l < w; ++l) {
      D[c0 + l] = cur[l + (size_t)l * nr];
      cur[l + (size_t)l * nr] = 1.0;
    }
    B.trsm(ColMajor, Right, Lower, ConjTrans, Unit, rowNo, w, 1.0, cur, nr, cur + w, nr);
    double *Dc = D + c0;
    for (int i = 0; i < w; ++i) {
      double *col = cur + w + (size_t)i * nr;
      if (Dc[i + n] == 0) {
        double tmp = 1.0 / Dc[i];
        B.scal(rowNo, tmp, col, 1);
      } else {
        double sd = Dc[i + n];
        double det = Dc[i] * Dc[i + 1] - sd * sd;
        double od = 1.0 / det;
        double *col2 = col + nr;
        for (int j = 0; j < rowNo; ++j) {
          double x1 = col[j], x2 = col2[j];
          col[j] = x1 * Dc[i + 1] - x2 * sd;
          col2[j] = x2 * Dc[i] - x1 * sd;
        }
        B.scal(rowNo, od, col, 1);
        B.scal(rowNo, od, col2, 1);
        ++i;
      }
    }
  }
  // rename rows of descendants that fall in pivoted supernodes and re-sort them
  for (int s : pivoted_sn) {
    const int c0 = S.super[s], c1 = S.super[s + 1], w = c1 - c0;
    std::vector<int> inv(w);
    for (int m = 0; m < w; ++m) inv[perm_piv[c0 + m] - c0] = m;
    int top = ereach(ns, Up, Ui, c0, c1, S.col2sup, S.sparent, stack, mark);
    for (int t = top; t < ns; ++t) {
      const int d = stack[t];
      const int dc0 = S.super[d], dw = S.super[d + 1] - dc0;
      const int dnr = (int)(S.lpi[d + 1] - S.lpi[d]);
      int *drows = ls.data() + S.lpi[d];
      int lb = (int)(std::lower_bound(drows, drows + dnr, c0) - drows);
      int ub = (int)(std::lower_bound(drows, drows + dnr, c1) - drows);
      const int len = ub - lb;
      if (len <= 0) continue;
      std::vector<std::pair<int, int>> key(len);
      for (int e = 0; e < len; ++e) key[e] = {c0 + inv[drows[lb + e] - c0], e};
      std::sort(key.begin(), key.end());
      std::vector<double> tmp(len);
      for (int c = 0; c < dw; ++c) {
        double *col = Lv + S.colp[dc0 + c] + lb;
        for (int e = 0; e < len; ++e) tmp[e] = col[key[e].second];
        std::copy(tmp.begin(), tmp.end(), col);
      }
      for (int e = 0; e < len; ++e) drows[lb + e] = key[e].first;
    }
  }
  F.ls = ls;
  F.perm.resize(n);
  for (int i = 0; i < n; ++i) F.perm[i] = S.perm[perm_piv[i]];
  return 0;
}

// blockedLsolve / D / blockedLTsolve on an ordered vector
void ldlt_solve(const Sym &S, const Factor &F, double *x) {
  const int n = S.n, ns = S.ns;
  std::vector<double> tmp(n);
  for (int s = 0; s < ns; ++s) {
    const int c0 = S.super[s], w = S.super[s + 1] - c0;
    const int nr = (int)(S.lpi[s + 1] - S.lpi[s]);
    const double *Ls = F.L.data() + S.colp[c0];
    B.trsm(ColMajor, Left, Lower, NoTrans, NonUnit, w, 1, 1.0, Ls, nr, x + c0, n);
    if (nr > w) {
      B.gemv(ColMajor, NoTrans, nr - w, w, 1.0, Ls + w, nr, x + c0, 1, 0.0, tmp.data(), 1);
      const int *rows = F.ls.data() + S.lpi[s];
      for (int k = 0; k < nr - w; ++k) x[rows[w + k]] -= tmp[k];
    }
  }
  const double *D = F.D.data();
  for (int i = 0; i < n; ++i) {
    if (D[i + n] == 0) {
      x[i] *= 1.0 / D[i];
    } else {
      double sd = D[i + n], det = D[i] * D[i + 1] - sd * sd, od = 1.0 / det;
      double x1 = x[i], x2 = x[i + 1];
      x[i] = (x1 * D[i + 1] - x2 * sd) * od;
      x[i + 1] = (x2 * D[i] - x1 * sd) * od;
      ++i;
    }
  }
  for (int s = ns - 1; s >= 0; --s) {
    const int c0 = S.super[s], w = S.super[s + 1] - c0;
    const int nr = (int)(S.lpi[s + 1] - S.lpi[s]);
    const double *Ls = F.L.data() + S.colp[c0];
    if (nr > w) {
      const int *rows = F.ls.data() + S.lpi[s];
      for (int k = 0; k < nr - w; ++k) tmp[k] = x[rows[w + k]];
      B.gemv(ColMajor, Trans, nr - w, w, -1.0, Ls + w, nr, tmp.data(), 1, 1.0, x + c0, 1);
    }
    B.trsm(ColMajor, Left, Lower, Trans, NonUnit, w, 1, 1.0, Ls, nr, x + c0, n);
  }
}

// y = K x, K lower-stored symmetric (column sweep)
void spmv_sym(int n, const std::vector<int> &Kp, const std::vector<int> &Ki, const std::vector<double> &Kx,
              const double *x, double *y) {
  std::fill(y, y + n, 0.0);
  for (int j = 0; j < n; ++j) {
    double yj = 0.0;
    const double xj = x[j];
    for (int q = Kp[j]; q < Kp[j + 1]; ++q) {
      int i = Ki[q];
      if (i == j) y[i] += Kx[q] * xj;
      else if (i > j) {
        y[i] += Kx[q] * xj;
        yj += Kx[q] * x[i];
      }
    }
    y[j] += yj;
  }
}

double dot(int n, const double *a, const double *b) {
  double v = 0.0;
  for (int i = 0; i < n; ++i) v = v + a[i] * b[i];
  return v;
}

int gmres(const Sym &S, const Factor &F, const std::vector<int> &Kp, const std::vector<int> &Ki,
          const std::vector<double> &Kx, double *x, const double *rhs, int itr_max, int mr, double tol_abs,
          double tol_rel) {
  const int n = S.n;
  const double delta = 1.0e-03;
  std::vector<double> c(mr + 1), sn(mr + 1), g(mr + 1), y(mr + 1), r(n);
  std::vector<std::vector<double>> h(mr + 1, std::vector<double>(mr, 0.0)), v(mr + 1, std::vector<double>(n));
  int itr_used = 0, k_copy = 0;
  double rho = 0, rho_tol = 0;
  for (int itr = 0; itr < itr_max; itr++) {
    spmv_sym(n, Kp, Ki, Kx, x, r.data());
    for (int i = 0; i < n; i++) r[i] = rhs[i] - r[i];
    ldlt_solve(S, F, r.data());
    rho = std::sqrt(dot(n, r.data(), r.data()));
    if (rho < tol_abs) return itr_used;
    if (itr == 0) rho_tol = rho * tol_rel;
    for (int i = 0; i < n; i++) v[0][i] = r[i] / rho;
    g[0] = rho;
    for (int i = 1; i < mr + 1; i++) g[i] = 0.0;
    for (auto &row : h) std::fill(row.begin(), row.end(), 0.0);
    for (int k = 0; k < mr; k++) {
      k_copy = k;
      spmv_sym(n, Kp, Ki, Kx, v[k].data(), v[k + 1].data());
      ldlt_solve(S, F, v[k + 1].data());
      double av = std::sqrt(dot(n, v[k + 1].data(), v[k + 1].data()));
      for (int j = 0; j <= k; j++) {
        h[j][k] = dot(n, v[k + 1].data(), v[j].data());
        for (int i = 0; i < n; i++) v[k + 1][i] = v[k + 1][i] - h[j][k] * v[j][i];
      }
      h[k + 1][k] = std::sqrt(dot(n, v[k + 1].data(), v[k + 1].data()));
      if ((av + delta * h[k + 1][k]) == av) {
        for (int j = 0; j < k + 1; j++) {
          double ht = dot(n, v[k + 1].data(), v[j].data());
          h[j][k] = h[j][k] + ht;
          for (int i = 0; i < n; i++) v[k + 1][i] = v[k + 1][i] - ht * v[j][i];
        }
        h[k + 1][k] = std::sqrt(dot(n, v[k + 1].data(), v[k + 1].data()));
      }
      if (h[k + 1][k] != 0.0)
        for (int i = 0; i < n; i++) v[k + 1][i] = v[k + 1][i] / h[k + 1][k];
      if (0 < k) {
        for (int i = 0; i < k + 2; i++) y[i] = h[i][k];
        for (int j = 0; j < k; j++) {
          double g1 = c[j] * y[j] - sn[j] * y[j + 1], g2 = sn[j] * y[j] + c[j] * y[j + 1];
          y[j] = g1;
          y[j + 1] = g2;
        }
        for (int i = 0; i < k + 2; i++) h[i][k] = y[i];
      }
      double mu = std::sqrt(h[k][k] * h[k][k] + h[k + 1][k] * h[k + 1][k]);
      if (mu == 0) return itr_used;
      c[k] = h[k][k] / mu;
      sn[k] = -h[k + 1][k] / mu;
      h[k][k] = c[k] * h[k][k] - sn[k] * h[k + 1][k];
      h[k + 1][k] = 0.0;
      double g1 = c[k] * g[k] - sn[k] * g[k + 1], g2 = sn[k] * g[k] + c[k] * g[k + 1];
      g[k] = g1;
      g[k + 1] = g2;
      rho = std::fabs(g[k + 1]);
      itr_used++;
      if (rho <= rho_tol && rho <= tol_abs) break;
    }
    int k = k_copy;
    if (h[k][k] == 0) return itr_used;
    y[k] = g[k] / h[k][k];
    for (int i = k - 1; 0 <= i; i--) {
      y[i] = g[i];
      for (int j = i + 1; j < k + 1; j++) y[i] = y[i] - h[i][j] * y[j];
      y[i] = y[i] / h[i][i];
    }
    for (int i = 0; i < n; i++)
      for (int j = 0; j < k + 1; j++) x[i] = x[i] + v[j][i] * y[j];
    if (rho <= rho_tol && rho <= tol_abs) break;
  }
  return itr_used;
}

// ---------------------------------------------------------------------------
// NASOQ's dual active-set QP loop over the SoMod partial refactorization
// (Nasoq::numeric_QP, src/nasoq.cpp:478-610; update_ldl_left_sn_02_v2,
// src/ldl/Serial_update_ldl.cpp:18-277; masked solves solve_phase.cpp:133-161;
// add_del_matrix_qp, linear_solver_wrapper.cpp:1020-1137), one problem,
// serial.  The super-KKT matrix [H; A; C] keeps its original numbering;
// inactive constraint entries read as zero, and the ordered columns a
// supernode needs are formed from the current composed ordering (the
// reference rebuilds A_ord after each pivoting refactorization,
// reorder_matrix).  Renamed rows are not re-sorted: every consumer maps them
// through the target supernode's row list.  Dense steps call the same
// BLAS/LAPACK routines as the reference (dgemm, dsytrf, dlapmt, dtrsm, dgemv).
struct QP {
  int n, meq, mineq, N, base, ns;
  Sym S;
  std::vector<int> Rp, Rj, Rq, ent, bt_ptr, bt_var, bt_q, eq_ptr, eq_var, eq_q, sn_con, con_sn;
  std::vector<int> pair_ptr, pair_d, pair_lb, pair_ub;
  const double *kv, *q, *b, *d;
  std::vector<uint8_t> pert;
  double reg;
  // state
  std::vector<int> perm, iperm, ls;
  std::vector<double> L, D;
  std::vector<uint8_t> act, vis, mark;
  std::vector<int> mlist;
  // workspace
  std::vector<double> contribs, trn, tmp;
  std::vector<int> map, ipiv, swapv, tmpsort, pivots, lperm;
};

double qp_fact_val(const QP &P, int vq) {
  const int e = P.ent[vq];
  double v = P.kv[vq];
  if (e >= 0) return P.act[e] ? v : 0.0;
  if (e <= -2 && P.pert[-2 - e]) return P.reg;
  return v;
}
double qp_ref_val(const QP &P, int vq) {
  const int e = P.ent[vq];
  double v = P.kv[vq];
  if (e >= 0) return P.act[e] ? v : 0.0;
  if (e <= -2 && P.pert[-2 - e]) return 0.0;
  return v;
}

void qp_factor_sn(QP &P, int s, std::vector<uint8_t> &piv) {
  const Sym &S = P.S;
  const int n = P.N;
  const int c0 = S.super[s], c1 = S.super[s + 1], w = c1 - c0;
  const int nr = (int)(S.lpi[s + 1] - S.lpi[s]);
  const int *rows = P.ls.data() + S.lpi[s];
  for (int i = 0; i < nr; ++i) P.map[rows[i]] = i;
  double *cur = P.L.data() + S.colp[c0];
  std::fill(cur, cur + (size_t)nr * w, 0.0);
  for (int m = 0; m < w; ++m) {
    const int col = c0 + m, j = P.perm[col];
    for (int qq = P.Rp[j]; qq < P.Rp[j + 1]; ++qq) {
      const int oi = P.iperm[P.Rj[qq]];
      if (oi >= col) cur[(size_t)m * nr + P.map[oi]] = qp_fact_val(P, P.Rq[qq]);
    }
  }
  double *Dv = P.D.data();
  for (int pq = P.pair_ptr[s]; pq < P.pair_ptr[s + 1]; ++pq) {
    const int dd = P.pair_d[pq];
    if (!P.vis[dd]) continue;
    const int dc0 = S.super[dd], dw = S.super[dd + 1] - dc0;
    const int dnr = (int)(S.lpi[dd + 1] - S.lpi[dd]);
    const int *drows = P.ls.data() + S.lpi[dd];
    const int lb = P.pair_lb[pq], ub = P.pair_ub[pq];
    const int nSupRs = dnr - lb, ndrow1 = ub - lb + 1;
    const double *src = P.L.data() + S.colp[dc0] + lb;
    const double *Dd = Dv + dc0;
    for (int l = 0; l < dw;) {  // T = L_d D_d (blocked_2by2_mult)
      if (Dd[l + n] == 0) {
        for (int l1 = 0; l1 < nSupRs; ++l1) P.trn[(size_t)l * nSupRs + l1] = Dd[l] * src[(size_t)l * dnr + l1];
        l++;
      } else {
        const double d1 = Dd[l], d2 = Dd[l + 1], e = Dd[l + n];
        for (int l1 = 0; l1 < nSupRs; ++l1) {
          P.trn[(size_t)l * nSupRs + l1] = d1 * src[(size_t)l * dnr + l1] + e * src[(size_t)(l + 1) * dnr + l1];
          P.trn[(size_t)(l + 1) * nSupRs + l1] = e * src[(size_t)l * dnr + l1] + d2 * src[(size_t)(l + 1) * dnr + l1];
        }
        l += 2;
      }
    }
    B.gemm(ColMajor, NoTrans, ConjTrans, nSupRs, ndrow1, dw, 1.0, P.trn.data(), nSupRs, src, dnr, 0.0,
           P.contribs.data(), nSupRs);
    for (int i = 0; i < ndrow1; ++i) {
      const int col = P.map[drows[i + lb]];
      for (int j = i; j < nSupRs; ++j) {
        int rp = P.map[drows[j + lb]], cp = col;
        if (rp < cp) std::swap(rp, cp);  // renamed rows: keep to the lower triangle
        cur[(size_t)cp * nr + rp] -= P.contribs[(size_t)i * nSupRs + j];
      }
    }
  }
  B.sytrf(ColMajor, 'L', w, cur, nr, P.ipiv.data());
  for (int i = 0; i < w; ++i) Dv[c0 + i + n] = 0.0;
  bool skip = false, perm_any = false;
  for (int j = 0; j < w; ++j) {
    P.swapv[j] = j;
    P.tmpsort[j] = j;
  }
  for (int i = 0; i < w; ++i) {  // reorder_after_sytrf
    if (skip) {
      P.pivots[i] = 0;
      skip = false;
      continue;
    }
    const int cv = P.ipiv[i];
    if (cv > 0) {
      if (cv != i + 1) {
        P.swapv[i] = P.swapv[cv - 1];
        perm_any = true;
      }
      P.pivots[i] = 1;
    } else {
      if (-cv != i + 2) {
        P.swapv[i + 1] = P.swapv[-cv - 1];
        perm_any = true;
      }
      P.pivots[i] = 2;
      Dv[c0 + i + n] = cur[(size_t)i * nr + i + 1];
      cur[(size_t)i * nr + i + 1] = 0.0;
      skip = true;
    }
  }
  if (perm_any)
    for (int k = 0; k < w; ++k) {
      const int cv = P.swapv[k];
      if (k != cv) {
        const int len = P.pivots[k] == 0 ? k - 1 : k;
        for (int c = 0; c < len; ++c) std::swap(cur[k + (size_t)c * nr], cur[cv + (size_t)c * nr]);
        std::swap(P.tmpsort[k], P.tmpsort[cv]);
      }
    }
  const int rowNo = nr - w;
  if (perm_any) {
    std::vector<int> k1(w);
    for (int m = 0; m < w; ++m) k1[m] = P.tmpsort[m] + 1;
    if (rowNo > 0) B.lapmt(ColMajor, 1, rowNo, w, cur + w, nr, k1.data());
  }
  piv[s] = perm_any ? 1 : 0;
  for (int m = 0; m < w; ++m) P.lperm[c0 + m] = P.tmpsort[m];
  for (int l = 0; l < w; ++l) {
    Dv[c0 + l] = cur[l + (size_t)l * nr];
    cur[l + (size_t)l * nr] = 1.0;
  }
  if (rowNo > 0) {
    B.trsm(ColMajor, Right, Lower, ConjTrans, Unit, rowNo, w, 1.0, cur, nr, cur + w, nr);
    double *Dc = Dv + c0;
    for (int i = 0; i < w; ++i) {
      double *col = cur + w + (size_t)i * nr;
      if (Dc[i + n] == 0) {
        B.scal(rowNo, 1.0 / Dc[i], col, 1);
      } else {
        const double sd = Dc[i + n], od = 1.0 / (Dc[i] * Dc[i + 1] - sd * sd);
        double *col2 = col + nr;
        for (int j = 0; j < rowNo; ++j) {
          const double x1 = col[j], x2 = col2[j];
          col[j] = x1 * Dc[i + 1] - x2 * sd;
          col2[j] = x2 * Dc[i] - x1 * sd;
        }
        B.scal(rowNo, od, col, 1);
        B.scal(rowNo, od, col2, 1);
        ++i;
      }
    }
  }
}

// Partial refactorization of the marked supernodes (ascending), then the
// pivots into the descendants' row lists and into the ordering.
void qp_refactor(QP &P) {
  std::sort(P.mlist.begin(), P.mlist.end());
  std::vector<uint8_t> piv(P.ns, 0);
  for (int s : P.mlist) qp_factor_sn(P, s, piv);
  for (int s : P.mlist) {
    P.mark[s] = 0;
    if (!piv[s]) continue;
    const int c0 = P.S.super[s], w = P.S.super[s + 1] - c0;
    std::vector<int> inv(w), old(w);
    for (int m = 0; m < w; ++m) inv[P.lperm[c0 + m]] = m;
    for (int pq = P.pair_ptr[s]; pq < P.pair_ptr[s + 1]; ++pq) {
      int *rd = P.ls.data() + P.S.lpi[P.pair_d[pq]];
      for (int i = P.pair_lb[pq]; i <= P.pair_ub[pq]; ++i) rd[i] = c0 + inv[rd[i] - c0];
    }
    for (int m = 0; m < w; ++m) old[m] = P.perm[c0 + P.lperm[c0 + m]];
    for (int m = 0; m < w; ++m) {
      P.perm[c0 + m] = old[m];
      P.iperm[old[m]] = c0 + m;
    }
  }
  P.mlist.clear();
}

void qp_mark_path(QP &P, int s) {
  for (; s >= 0; s = P.S.sparent[s])
    if (!P.mark[s]) {
      P.mark[s] = 1;
      P.mlist.push_back(s);
    }
}

// x <- (L D L^T)^-1 x in the factor's order, visible supernodes only.
void qp_ldlt_solve(QP &P, double *x) {
  const Sym &S = P.S;
  const int n = P.N;
  for (int s = 0; s < P.ns; ++s) {
    if (!P.vis[s]) continue;
    const int c0 = S.super[s], w = S.super[s + 1] - c0;
    const int nr = (int)(S.lpi[s + 1] - S.lpi[s]);
    const double *Ls = P.L.data() + S.colp[c0];
    B.trsm(ColMajor, Left, Lower, NoTrans, Unit, w, 1, 1.0, Ls, nr, x + c0, n);
    if (nr > w) {
      B.gemv(ColMajor, NoTrans, nr - w, w, 1.0, Ls + w, nr, x + c0, 1, 0.0, P.tmp.data(), 1);
      const int *rows = P.ls.data() + S.lpi[s];
      for (int k = 0; k < nr - w; ++k) x[rows[w + k]] -= P.tmp[k];
    }
  }
  const double *D = P.D.data();
  for (int i = 0; i < n; ++i) {
    if (!P.vis[S.col2sup[i]]) continue;
    if (D[i + n] == 0) {
      x[i] *= 1.0 / D[i];
    } else {
      const double sd = D[i + n], od = 1.0 / (D[i] * D[i + 1] - sd * sd);
      const double x1 = x[i], x2 = x[i + 1];
      x[i] = (x1 * D[i + 1] - x2 * sd) * od;
      x[i + 1] = (x2 * D[i] - x1 * sd) * od;
      ++i;
    }
  }
  for (int s = P.ns - 1; s >= 0; --s) {
    if (!P.vis[s]) continue;
    const int c0 = S.super[s], w = S.super[s + 1] - c0;
    const int nr = (int)(S.lpi[s + 1] - S.lpi[s]);
    const double *Ls = P.L.data() + S.colp[c0];
    if (nr > w) {
      const int *rows = P.ls.data() + S.lpi[s];
      for (int k = 0; k < nr - w; ++k) P.tmp[k] = x[rows[w + k]];
      B.gemv(ColMajor, Trans, nr - w, w, -1.0, Ls + w, nr, P.tmp.data(), 1, 1.0, x + c0, 1);
    }
    B.trsm(ColMajor, Left, Lower, Trans, Unit, w, 1, 1.0, Ls, nr, x + c0, n);
  }
}

// out = M^-1 v in the original numbering (hidden rows zero)
void qp_precond(QP &P, const double *v, double *out, std::vector<double> &xo) {
  for (int c = 0; c < P.N; ++c) xo[c] = P.vis[P.S.col2sup[c]] ? v[P.perm[c]] : 0.0;
  qp_ldlt_solve(P, xo.data());
  for (int c = 0; c < P.N; ++c) out[P.perm[c]] = xo[c];
}

void qp_spmv(const QP &P, const double *x, double *y) {
  for (int i = 0; i < P.N; ++i) {
    double acc = 0.0;
    for (int qq = P.Rp[i]; qq < P.Rp[i + 1]; ++qq) acc += qp_ref_val(P, P.Rq[qq]) * x[P.Rj[qq]];
    y[i] = acc;
  }
}

// The reference's left-preconditioned restarted GMRES (pmgmres_ldlt_auto).
int qp_gmres(QP &P, double *x, const double *rhs, int itr_max, int mr, double tol_abs, double tol_rel) {
  const int n = P.N;
  if (itr_max <= 0 || mr <= 0) return 0;
  const double delta = 1.0e-03;
  std::vector<double> c(mr + 1), sn(mr + 1), g(mr + 1), y(mr + 1), r(n), xo(n);
  std::vector<std::vector<double>> h(mr + 1, std::vector<double>(mr, 0.0)), v(mr + 1, std::vector<double>(n));
  int itr_used = 0, k_copy = 0;
  double rho = 0, rho_tol = 0;
  for (int itr = 0; itr < itr_max; itr++) {
    qp_spmv(P, x, r.data());
    for (int i = 0; i < n; i++) r[i] = rhs[i] - r[i];
    qp_precond(P, r.data(), r.data(), xo);
    rho = std::sqrt(dot(n, r.data(), r.data()));
    if (rho < tol_abs) return itr_used;
    if (itr == 0) rho_tol = rho * tol_rel;
    for (int i = 0; i < n; i++) v[0][i] = r[i] / rho;
    g[0] = rho;
    for (int i = 1; i < mr + 1; i++) g[i] = 0.0;
    for (auto &row : h) std::fill(row.begin(), row.end(), 0.0);
    for (int k = 0; k < mr; k++) {
      k_copy = k;
      qp_spmv(P, v[k].data(), v[k + 1].data());
      qp_precond(P, v[k + 1].data(), v[k + 1].data(), xo);
      const double av = std::sqrt(dot(n, v[k + 1].data(), v[k + 1].data()));
      for (int j = 0; j <= k; j++) {
        h[j][k] = dot(n, v[k + 1].data(), v[j].data());
        for (int i = 0; i < n; i++) v[k + 1][i] -= h[j][k] * v[j][i];
      }
      h[k + 1][k] = std::sqrt(dot(n, v[k + 1].data(), v[k + 1].data()));
      if ((av + delta * h[k + 1][k]) == av) {
        for (int j = 0; j < k + 1; j++) {
          const double ht = dot(n, v[k + 1].data(), v[j].data());
          h[j][k] += ht;
          for (int i = 0; i < n; i++) v[k + 1][i] -= ht * v[j][i];
        }
        h[k + 1][k] = std::sqrt(dot(n, v[k + 1].data(), v[k + 1].data()));
      }
      if (h[k + 1][k] != 0.0)
        for (int i = 0; i < n; i++) v[k + 1][i] /= h[k + 1][k];
      if (0 < k) {
        for (int i = 0; i < k + 2; i++) y[i] = h[i][k];
        for (int j = 0; j < k; j++) {
          const double g1 = c[j] * y[j] - sn[j] * y[j + 1], g2 = sn[j] * y[j] + c[j] * y[j + 1];
          y[j] = g1;
          y[j + 1] = g2;
        }
        for (int i = 0; i < k + 2; i++) h[i][k] = y[i];
      }
      const double mu = std::sqrt(h[k][k] * h[k][k] + h[k + 1][k] * h[k + 1][k]);
      if (mu == 0) return itr_used;
      c[k] = h[k][k] / mu;
      sn[k] = -h[k + 1][k] / mu;
      h[k][k] = c[k] * h[k][k] - sn[k] * h[k + 1][k];
      h[k + 1][k] = 0.0;
      const double g1 = c[k] * g[k] - sn[k] * g[k + 1], g2 = sn[k] * g[k] + c[k] * g[k + 1];
      g[k] = g1;
      g[k + 1] = g2;
      rho = std::fabs(g[k + 1]);
      itr_used++;
      if (rho <= rho_tol && rho <= tol_abs) break;
    }
    const int k = k_copy;
    if (h[k][k] == 0) return itr_used;
    y[k] = g[k] / h[k][k];
    for (int i = k - 1; 0 <= i; i--) {
      y[i] = g[i];
      for (int j = i + 1; j < k + 1; j++) y[i] -= h[i][j] * y[j];
      y[i] /= h[i][i];
    }
    for (int i = 0; i < n; i++)
      for (int j = 0; j < k + 1; j++) x[i] += v[j][i] * y[j];
    if (rho <= rho_tol && rho <= tol_abs) break;
  }
  return itr_used;
}

void qp_edit(QP &P, int k, bool add) {
  P.act[k] = add ? 1 : 0;
  P.vis[P.con_sn[k]] = add ? 1 : 0;
  qp_mark_path(P, P.con_sn[k]);
  for (int e = P.bt_ptr[k]; e < P.bt_ptr[k + 1]; ++e) qp_mark_path(P, P.S.col2sup[P.iperm[P.bt_var[e]]]);
}

// Pattern set-up: full symmetric CSR, entry kinds, constraint / equality row
// lists, constraint supernodes, descendant pairs (elimination-tree reach on
// the analysis ordering).
int qp_setup(QP &P, const int *Kp, const int *Ki) {
  const int N = P.N, n = P.n, base = P.base;
  P.Rp.assign(N + 1, 0);
  for (int j = 0; j < N; ++j)
    for (int q = Kp[j]; q < Kp[j + 1]; ++q) {
      P.Rp[j + 1]++;
      if (Ki[q] != j) P.Rp[Ki[q] + 1]++;
    }
  for (int r = 0; r < N; ++r) P.Rp[r + 1] += P.Rp[r];
  P.Rj.assign(P.Rp[N], 0);
  P.Rq.assign(P.Rp[N], 0);
  std::vector<int> pos(P.Rp.begin(), P.Rp.end() - 1);
  for (int j = 0; j < N; ++j)
    for (int q = Kp[j]; q < Kp[j + 1]; ++q) {
      const int i = Ki[q];
      P.Rj[pos[j]] = i;
      P.Rq[pos[j]++] = q;
      if (i != j) {
        P.Rj[pos[i]] = j;
        P.Rq[pos[i]++] = q;
      }
    }
  P.ent.assign(Kp[N], -1);
  std::vector<std::vector<int>> btv(P.mineq), btq(P.mineq), eqv(P.meq), eqq(P.meq);
  for (int j = 0; j < N; ++j)
    for (int q = Kp[j]; q < Kp[j + 1]; ++q) {
      const int i = Ki[q];
      if (i == j) P.ent[q] = -2 - j;
      else if (i >= base) {
        P.ent[q] = i - base;
        btv[i - base].push_back(j);
        btq[i - base].push_back(q);
      } else if (i >= n) {
        eqv[i - n].push_back(j);
        eqq[i - n].push_back(q);
      }
    }
  auto flat = [](std::vector<std::vector<int>> &a, std::vector<std::vector<int>> &b, std::vector<int> &ptr,
                 std::vector<int> &x, std::vector<int> &y) {
    ptr.assign(a.size() + 1, 0);
    for (size_t k = 0; k < a.size(); ++k) {
      ptr[k + 1] = ptr[k] + (int)a[k].size();
      x.insert(x.end(), a[k].begin(), a[k].end());
      y.insert(y.end(), b[k].begin(), b[k].end());
    }
  };
  flat(btv, btq, P.bt_ptr, P.bt_var, P.bt_q);
  flat(eqv, eqq, P.eq_ptr, P.eq_var, P.eq_q);
  std::vector<int> pinv(N);
  for (int k = 0; k < N; ++k) pinv[P.S.perm[k]] = k;
  P.sn_con.assign(P.ns, -1);
  P.con_sn.assign(P.mineq, -1);
  for (int k = 0; k < P.mineq; ++k) {
    const int s = P.S.col2sup[pinv[base + k]];
    if (P.S.super[s + 1] - P.S.super[s] != 1) return -3;
    P.con_sn[k] = s;
    P.sn_con[s] = k;
  }
  // pairs from the reach of every supernode in the ordered pattern
  std::vector<double> dummy(Kp[N], 0.0);
  std::vector<int> Cp, Ci, Up, Ui;
  std::vector<double> Cx;
  sym_permute_lower(N, Kp, Ki, dummy.data(), pinv, Cp, Ci, Cx);
  transpose_pattern(N, Cp, Ci, Up, Ui);
  std::vector<int> stack(P.ns), mark(P.ns, 0);
  P.pair_ptr.assign(P.ns + 1, 0);
  for (int s = 0; s < P.ns; ++s) {
    const int c1 = P.S.super[s], c2 = P.S.super[s + 1];
    const int top = ereach(P.ns, Up, Ui, c1, c2, P.S.col2sup, P.S.sparent, stack, mark);
    for (int t = top; t < P.ns; ++t) {
      const int d = stack[t];
      const int *rows = P.ls.data() + P.S.lpi[d];
      const int nr = (int)(P.S.lpi[d + 1] - P.S.lpi[d]);
      const int lb = (int)(std::lower_bound(rows, rows + nr, c1) - rows);
      const int ub = (int)(std::lower_bound(rows, rows + nr, c2) - rows) - 1;
      if (lb >= nr || ub < lb) continue;
      P.pair_d.push_back(d);
      P.pair_lb.push_back(lb);
      P.pair_ub.push_back(ub);
    }
    P.pair_ptr[s + 1] = (int)P.pair_d.size();
  }
  return 0;
}

}  // namespace

extern "C" {

// Loads the OpenBLAS shared library (SciPy's bundled build exports
// "scipy_"-prefixed names).  Returns 0 on success.
int nqp_init(const char *openblas_path) {
  void *h = dlopen(openblas_path, RTLD_NOW | RTLD_LOCAL);
  if (!h) return -1;
  bool ok = sym(h, "scipy_cblas_dgemm", "cblas_dgemm", B.gemm) && sym(h, "scipy_cblas_dtrsm", "cblas_dtrsm", B.trsm) &&
            sym(h, "scipy_cblas_dgemv", "cblas_dgemv", B.gemv) && sym(h, "scipy_cblas_dscal", "cblas_dscal", B.scal) &&
            sym(h, "scipy_LAPACKE_dsytrf", "LAPACKE_dsytrf", B.sytrf) &&
            sym(h, "scipy_LAPACKE_dlapmt", "LAPACKE_dlapmt", B.lapmt);
  sym(h, "scipy_openblas_set_num_threads", "openblas_set_num_threads", B.setthreads);
  return ok ? 0 : -2;
}

void nqp_set_threads(int t) {
  if (B.setthreads) B.setthreads(t);
}

// y = K x for K lower-stored symmetric CSC (n columns), the column sweep of
// spmv_sym (alpha = 1, beta = 0).
int nqp_spmv(int n, const int *Ap, const int *Ai, const double *Ax, const double *x, double *y) {
  if (n < 0 || !Ap || (n > 0 && (!Ai || !Ax || !x || !y))) return -1;
  std::vector<int> Kp(Ap, Ap + n + 1), Ki(Ai, Ai + Ap[n]);
  std::vector<double> Kx(Ax, Ax + Ap[n]);
  spmv_sym(n, Kp, Ki, Kx, x, y);
  return 0;
}

// Factor (perturbed values Ax) + solve with refinement on Ax_ref.  Symbolic
// arrays as produced by the analysis (perm, super, lpi, ls, colp, sparent,
// col2sup).  Outputs x (original ordering) and, when non-NULL, the factor
// (values, D[2n], combined perm, row lists after renaming).  times[0] =
// factor seconds, times[1] = solve seconds.
int nqp_solve(int n, const int *Ap, const int *Ai, const double *Ax, const double *Ax_ref, int nsuper,
              const int *perm, const int *super, const int64_t *lpi, const int *ls, const int64_t *colp,
              const int *sparent, const int *col2sup, const double *rhs, int req_ref_iter, int max_inner_iter,
              double tol_abs, double tol_rel, double *x, double *times, int *num_ref_iter, double *L_out,
              double *D_out, int *perm_out, int *ls_out) {
  if (!B.gemm) return -1;
  Sym S{n, nsuper, perm, super, sparent, col2sup, lpi, colp};
  std::vector<int> pinv(n);
  for (int k = 0; k < n; ++k) pinv[perm[k]] = k;
  auto t0 = clk::now();
  std::vector<int> Cp, Ci;
  std::vector<double> Cx;
  sym_permute_lower(n, Ap, Ai, Ax, pinv, Cp, Ci, Cx);
  std::vector<int> lsv(ls, ls + lpi[nsuper]);
  std::vector<int> Up, Ui;
  ordered_upper_like_reference(n, Ap, Ai, perm, pinv, Up, Ui);
  Factor F;
  factorize(S, Cp, Ci, Cx, Up, Ui, lsv, F);
  auto t1 = clk::now();
  // refinement matrix in the final (pivoted) ordering
  std::vector<int> pinv2(n);
  for (int k = 0; k < n; ++k) pinv2[F.perm[k]] = k;
  std::vector<int> Rp, Ri;
  std::vector<double> Rx;
  sym_permute_lower(n, Ap, Ai, Ax_ref, pinv2, Rp, Ri, Rx);
  std::vector<double> xo(n), bo(n);
  for (int i = 0; i < n; ++i) xo[i] = bo[i] = rhs[F.perm[i]];
  ldlt_solve(S, F, xo.data());
  int used = 0;
  if (req_ref_iter > 0) used = gmres(S, F, Rp, Ri, Rx, xo.data(), bo.data(), req_ref_iter, max_inner_iter, tol_abs, tol_rel);
  for (int i = 0; i < n; ++i) x[F.perm[i]] = xo[i];
  auto t2 = clk::now();
  if (times) {
    times[0] = std::chrono::duration<double>(t1 - t0).count();
    times[1] = std::chrono::duration<double>(t2 - t1).count();
  }
  if (num_ref_iter) *num_ref_iter = used;
  if (L_out) std::copy(F.L.begin(), F.L.end(), L_out);
  if (D_out) std::copy(F.D.begin(), F.D.end(), D_out);
  if (perm_out) std::copy(F.perm.begin(), F.perm.end(), perm_out);
  if (ls_out) std::copy(F.ls.begin(), F.ls.end(), ls_out);
  return 0;
}


// One QP by the reference's NASOQ method (Fixed / PREDET / AUTO settings
// resolved by the caller: reg = diag_perturb, outer x inner refinement steps,
// tol = stop_tol).  K: the lower-stored super-KKT [H; A; C] (N = n + meq +
// mineq columns, every constraint value present, zero constraint
// diagonals); symbolic arrays of its analysis (constraint columns hidden).
// Outputs x, y, z, the final active set (insertion order), info = {status,
// iterations, active size} and norms = {objective, lagrangian residual,
// constraint violation, non-negativity, complementarity}.
int nqp_qp_solve(int N, int n, int meq, int mineq, const int *Kp, const int *Ki, const double *Kx, const double *q,
                 const double *b, const double *d, int nsuper, const int *perm, const int *super, const int64_t *lpi,
                 const int *ls, const int64_t *colp, const int *sparent, const int *col2sup, double reg, int outer,
                 int inner, double tol, double eps_abs, int max_iter_nas, double zero_thresh, double *x, double *y,
                 double *z, int *active, int *info, double *norms) {
  if (!B.gemm) return -1;
  QP P;
  P.n = n;
  P.meq = meq;
  P.mineq = mineq;
  P.N = N;
  P.base = n + meq;
  P.ns = nsuper;
  P.S = Sym{N, nsuper, perm, super, sparent, col2sup, lpi, colp};
  P.kv = Kx;
  P.q = q;
  P.b = b;
  P.d = d;
  P.reg = reg;
  P.ls.assign(ls, ls + lpi[nsuper]);
  int rc = qp_setup(P, Kp, Ki);
  if (rc) return rc;
  P.pert.assign(N, 0);
  for (int j = 0; j < N; ++j) P.pert[j] = std::abs(Kx[Kp[j]]) < reg ? 1 : 0;
  P.perm.assign(perm, perm + N);
  P.iperm.assign(N, 0);
  for (int c = 0; c < N; ++c) P.iperm[P.perm[c]] = c;
  P.L.assign(std::max<int64_t>(colp[N], 1), 0.0);
  P.D.assign(2 * (size_t)N, 0.0);
  P.act.assign(std::max(mineq, 1), 0);
  P.vis.assign(nsuper, 0);
  P.mark.assign(nsuper, 0);
  int smax = 1, cmax = 1;
  for (int s = 0; s < nsuper; ++s) {
    smax = std::max(smax, super[s + 1] - super[s]);
    cmax = std::max<int>(cmax, (int)(lpi[s + 1] - lpi[s]));
  }
  P.contribs.assign((size_t)(smax + 1) * (cmax + 1), 0.0);
  P.trn.assign((size_t)(smax + 1) * (cmax + 1), 0.0);
  P.tmp.assign(cmax + 1, 0.0);
  P.map.assign(N, 0);
  P.ipiv.assign(smax + 1, 0);
  P.swapv.assign(smax + 1, 0);
  P.tmpsort.assign(smax + 1, 0);
  P.pivots.assign(smax + 1, 0);
  P.lperm.assign(N, 0);
  for (int s = 0; s < nsuper; ++s) P.vis[s] = P.sn_con[s] < 0 ? 1 : 0;
  // initialize_x: factor the visible supernodes, solve [-q; b; 0]
  for (int s = 0; s < nsuper; ++s)
    if (P.vis[s]) {
      P.mark[s] = 1;
      P.mlist.push_back(s);
    }
  qp_refactor(P);
  std::vector<double> rhs(N, 0.0), sol(N, 0.0), xo(N), tmp(N);
  for (int i = 0; i < n; ++i) rhs[i] = -q[i];
  for (int i = 0; i < meq; ++i) rhs[n + i] = b[i];
  qp_precond(P, rhs.data(), sol.data(), xo);
  qp_gmres(P, sol.data(), rhs.data(), outer, inner, tol, tol);
  std::vector<double> xv(sol.begin(), sol.begin() + n), yv(meq), zv(mineq, 0.0);
  for (int i = 0; i < meq; ++i) yv[i] = sol[n + i];
  std::vector<int> alist;
  const double DMAX = std::numeric_limits<double>::max();
  int num_iter = 0, converged = 0, nxt_active = -1, nxt_drop = -1, to_add = 1;
  bool update = false;
  for (;;) {
    if (num_iter > max_iter_nas) {
      converged = 0;
      break;
    }
    if (to_add == 1) {  // primal_feasibility
      int viol = 0;
      double best = eps_abs;
      nxt_active = -1;
      for (int k = 0; k < mineq; ++k) {
        double t = 0.0;
        for (int e = P.bt_ptr[k]; e < P.bt_ptr[k + 1]; ++e) t += Kx[P.bt_q[e]] * xv[P.bt_var[e]];
        t -= d[k];
        if (t > eps_abs) viol++;
        if (t > best) {
          best = t;
          nxt_active = k;
        }
      }
      if (viol == 0) {
        converged = 1;
        break;
      }
      if (nxt_active < 0) {
        converged = 0;
        break;
      }
      std::fill(rhs.begin(), rhs.end(), 0.0);  // update_rhs
      for (int e = P.bt_ptr[nxt_active]; e < P.bt_ptr[nxt_active + 1]; ++e) rhs[P.bt_var[e]] = Kx[P.bt_q[e]];
    }
    if (update) {
      qp_refactor(P);
      update = false;
    }
    qp_precond(P, rhs.data(), sol.data(), xo);
    qp_gmres(P, sol.data(), rhs.data(), outer, inner, tol, tol);
    double dual_step = DMAX;  // dual_step_length
    for (int k = 0; k < mineq; ++k) {
      const double lm = sol[P.base + k];
      if (lm > 0 && P.act[k]) {
        const double r = zv[k] / lm;
        if (r < dual_step) {
          dual_step = r;
          nxt_drop = k;
        }
      }
    }
    double bdotx = 0.0, ddotb = 0.0, prime_step = DMAX;  // primal_step_length
    for (int e = P.bt_ptr[nxt_active]; e < P.bt_ptr[nxt_active + 1]; ++e) {
      bdotx += Kx[P.bt_q[e]] * xv[P.bt_var[e]];
      ddotb += Kx[P.bt_q[e]] * sol[P.bt_var[e]];
    }
    if (!(ddotb < zero_thresh)) prime_step = -(d[nxt_active] - bdotx) / ddotb;
    const double step = prime_step > dual_step ? dual_step : prime_step;
    if (step == DMAX) {
      converged = 0;
      break;
    }
    const bool dual_only = prime_step == DMAX && step == dual_step;
    if (!dual_only)
      for (int i = 0; i < n; ++i) xv[i] -= step * sol[i];
    for (int i = 0; i < meq; ++i) yv[i] -= step * sol[n + i];
    for (int k : alist) zv[k] -= step * sol[P.base + k];
    zv[nxt_active] += step;
    int add = -1, del = -1;
    if (dual_only) del = nxt_drop;
    else if (step == prime_step) add = nxt_active;
    else if (step == dual_step) del = nxt_drop;
    if (add >= 0) {
      qp_edit(P, add, true);
      alist.push_back(add);
      to_add = 1;
      update = true;
    } else if (del >= 0) {
      qp_edit(P, del, false);
      alist.erase(std::remove(alist.begin(), alist.end(), del), alist.end());
      to_add = 0;
      update = true;
    }
    num_iter++;
  }
  // objective and KKT norms
  std::vector<double> full(N, 0.0);
  for (int i = 0; i < n; ++i) full[i] = xv[i];
  for (int i = 0; i < meq; ++i) full[n + i] = yv[i];
  for (int k = 0; k < mineq; ++k) full[P.base + k] = zv[k];
  double quad = 0, lin = 0, lag = 0, cons = 0, dual_obj = 0, nonneg = 0, comp = 0;
  for (int i = 0; i < n; ++i) {
    double hx = 0, fl = 0;
    for (int qq = P.Rp[i]; qq < P.Rp[i + 1]; ++qq) {
      const int j = P.Rj[qq];
      const double v = Kx[P.Rq[qq]];
      if (j < n) hx += v * xv[j];
      fl += v * full[j];
    }
    quad += hx * xv[i];
    lin += q[i] * xv[i];
    lag = std::max(lag, std::abs(fl + q[i]));
  }
  for (int k = 0; k < mineq; ++k) {
    double t = -d[k];
    for (int e = P.bt_ptr[k]; e < P.bt_ptr[k + 1]; ++e) t += Kx[P.bt_q[e]] * xv[P.bt_var[e]];
    cons = std::max(cons, t < 0 ? 0.0 : t);
    dual_obj += t * zv[k];
    nonneg = std::max(nonneg, zv[k] > 0 ? 0.0 : std::abs(zv[k]));
    comp = std::max(comp, std::abs(zv[k] * t));
  }
  for (int r = 0; r < meq; ++r) {
    double t = -b[r];
    for (int e = P.eq_ptr[r]; e < P.eq_ptr[r + 1]; ++e) t += Kx[P.eq_q[e]] * xv[P.eq_var[e]];
    cons = std::max(cons, std::abs(t));
  }
  int st;
  if (!converged) st = 0;
  else if (lag <= eps_abs && cons <= eps_abs && nonneg <= eps_abs) st = 1;
  else if (cons <= eps_abs) st = 2;
  else st = 3;
  std::copy(xv.begin(), xv.end(), x);
  if (y) std::copy(yv.begin(), yv.end(), y);
  if (z) std::copy(zv.begin(), zv.end(), z);
  if (active)
    for (size_t t = 0; t < alist.size(); ++t) active[t] = alist[t];
  info[0] = st;
  info[1] = num_iter;
  info[2] = (int)alist.size();
  norms[0] = 0.5 * quad + lin + dual_obj;
  norms[1] = lag;
  norms[2] = cons;
  norms[3] = nonneg;
  norms[4] = comp;
  return 0;
}

}  // extern "C"
