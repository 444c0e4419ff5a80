// Settings rules of the reference's NASOQ driver (see qp_rules.hpp).
#include "qp_rules.hpp"

#include <cmath>

namespace nqg {

double qp_frob_lower(int n, const int *p, const int *i, const double *x) {
  double frob = 0, s = 0;
  for (int j = 0; j < n; ++j)
    for (int q = p[j]; q < p[j + 1]; ++q) {
      s = std::abs(x[q]);
      if (i[q] == j) frob += s * s;
      else if (i[q] > j) frob += 2 * s * s;
    }
  return std::isfinite(s) ? std::sqrt(frob) : 0.0;
}

void qp_auto_perturbation2(size_t dim, size_t total_nnz, double H_norm2, double, int n_ineq, double ineq_ratio,
                           double acc_thresh, double &reg, int &outer, int &inner, double &tol) {
  reg = std::pow(10, -8);
  int iter_low = 2, iter_high = 9, iter_large = 0;
  if (acc_thresh >= 1e-3) {
    iter_low /= 2;
    iter_high /= 2;
  } else if (acc_thresh < 1e-8) {
    iter_low *= 2;
    iter_large *= 2;
    iter_large += 1;
  }
  inner = outer = iter_large;
  if (total_nnz < 3e5) {
    inner = outer = iter_low;
    tol = 1e-10;
    if (H_norm2 < 1) {
      reg = std::pow(10, -7);
      inner = outer = iter_low;
      tol = 1e-15;
    } else if (ineq_ratio > 2.5) {
      reg = std::pow(10, -10);
      tol = 1e-16;
      inner = outer = iter_low;
    } else if (dim > 1e4 && n_ineq >= 1e4) {
      reg = std::pow(10, -11);
      inner = outer = iter_high;
      tol = 1e-15;
    }
  } else if (H_norm2 < 1) {
    reg = std::pow(10, -7);
    inner = outer = 2;
    tol = 1e-15;
  }
}

void qp_determine_iterations(size_t total_nnz, double acc_thresh, int &outer, int &inner) {
  if (acc_thresh >= 1e-3) inner = outer = 0;
  else if (acc_thresh <= 1e-4 && acc_thresh > 1e-7) inner = outer = 1;
  else if (acc_thresh <= 1e-7 && acc_thresh > 1e-10) inner = outer = 2;
  else inner = outer = 4;
  if (total_nnz <= 20000) inner = outer = 3;
}

}  // namespace nqg
