// Host-side symbolic analysis of a sparse symmetric matrix for the supernodal
// LDL^T factorization.  Produces the same ordering, elimination tree,
// supernode partition and supernodal row structure as the reference's
// symbolic_analysis_lin_solve (src/symbolic/symbolic_phase.cpp:167-890).
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace nqg {

// Lower- or upper-stored square CSC with sorted rows.
struct Csc {
  int n = 0;
  std::vector<int> p, i;
  std::vector<double> x;  // may be empty for pattern-only matrices
  int64_t nnz() const { return p.empty() ? 0 : p[n]; }
};

struct Symbolic {
  int n = 0;
  std::vector<int> perm, iperm;   // perm[k] = original column at position k
  std::vector<int> parent;        // elimination tree (postordered labels)
  std::vector<int> colcount;      // column counts of L (postordered)
  int nsuper = 0;
  std::vector<int> super;         // nsuper+1, first column of each supernode
  std::vector<int> sparent;       // nsuper, supernodal assembly tree
  std::vector<int> col2sup;       // n
  std::vector<int64_t> lpi;       // nsuper+1, start of each supernode's row list in ls
  std::vector<int> ls;            // row lists (sorted, diagonal block first)
  std::vector<int64_t> lpx;       // nsuper+1, start of each supernode's values (col-major nrow x ncol)
  std::vector<int64_t> colp;      // n+1, value offset of each column (reference L->p)
  std::vector<int> extra_cols;    // n, permuted hidden-column flags
  int max_sup_wid = 0, max_col = 0;
  int64_t xsize = 0;
  double metis_seconds = 0.0, total_seconds = 0.0;
};

// Symmetric permutation of a lower-stored matrix: returns the lower-stored
// C = P A P^T (rows sorted) and, when `upper` is non-null, the upper-stored
// transpose.  `pinv[old] = new`.  Values follow the entries.
void sym_permute(const Csc &A_lower, const std::vector<int> &pinv, Csc *lower, Csc *upper);

// Full symbolic analysis.  `extra_cols` (nullable) flags columns that must
// stay single-column supernodes (hidden constraint rows of the QP KKT).
// Returns an empty string on success, else an error message.
std::string analyze(const Csc &A_lower, const int *extra_cols, const int nrelax[3], const double zrelax[3],
                    Symbolic &out);

// Elimination-tree reach of supernode s (reference ereach_sn,
// src/common/Reach.cpp:96-125): supernodes whose columns update s, in the
// reference's stack order.  `upper` is the upper-stored ordered matrix.
void ereach_sn(const Symbolic &S, const Csc &upper, int s, const std::vector<int> &tree, std::vector<int> &mark,
               std::vector<int> &stack, std::vector<int> &outlist);

}  // namespace nqg
