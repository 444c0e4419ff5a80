// Settings rules of the reference's NASOQ driver, shared by the host QP loop
// (nasoq_qp.cpp) and the batched solver (batch_host.cpp).
#pragma once
#include <cstddef>

namespace nqg {

// Frobenius norm of a lower-stored symmetric CSC (off-diagonals counted
// twice); 0 when the last value read is not finite (reference
// Nasoq::symbolic_QP's H norm).
double qp_frob_lower(int n, const int *p, const int *i, const double *x);

// AUTO variant: regularization, refinement iterations and tolerance from the
// problem's size and norms (reference Nasoq::auto_perturbation2,
// src/nasoq.cpp:320-371).
void qp_auto_perturbation2(size_t dim, size_t total_nnz, double H_norm2, double range, int n_ineq, double ineq_ratio,
                           double acc_thresh, double &reg, int &outer, int &inner, double &tol);

// Fixed variant: refinement iterations from the accuracy target (reference
// Nasoq::determine_iterations, src/nasoq.cpp:373-395).
void qp_determine_iterations(size_t total_nnz, double acc_thresh, int &outer, int &inner);

}  // namespace nqg
