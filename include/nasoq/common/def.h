// Drop-in data types of the NASOQ C++ API (reference include/nasoq/common/
// def.h:73-220): the compressed-column matrix `CSC` callers hand to
// SolverSettings / Nasoq, and the supernodal factor descriptor `BCSC`.  Field
// names and meanings are kept so that caller code compiles unchanged.
#ifndef NASOQ_GB300_DEF_H
#define NASOQ_GB300_DEF_H

#include <cstddef>

namespace nasoq {

#ifndef TRUE
#define TRUE 1
#endif
#ifndef FALSE
#define FALSE 0
#endif
#define EMPTY -1
#define INVISIBLE -2
#define ROOT -1
#define CHOLMOD_PATTERN 0
#define CHOLMOD_REAL 1
#define CHOLMOD_METIS 3

// Compressed sparse column matrix, 0-based.  Symmetric matrices are stored
// lower (stype = -1) with sorted rows and the diagonal first in each column.
struct CSC {
  size_t nrow = 0, ncol = 0;  // nrow-by-ncol
  size_t nzmax = 0;           // number of stored entries
  int *p = nullptr;           // ncol+1 column pointers
  int *i = nullptr;           // row indices
  int *nz = nullptr;          // unused (packed matrices only)
  double *x = nullptr;        // values
  double *z = nullptr;        // unused
  int stype = 0;              // 0 unsymmetric, <0 lower, >0 upper
  int itype = 0, xtype = CHOLMOD_REAL, dtype = 0;
  int sorted = TRUE, packed = TRUE;
};

// Supernodal factor descriptor.  The host copy holds the symbolic structure;
// the numeric values live on the GPU (SolverSettings::valL / d_val are filled
// on request by SolverSettings::download_factor()).
struct BCSC {
  size_t n = 0;
  size_t minor = 0;
  int *Perm = nullptr;      // n, combined fill-reducing and pivot permutation
  int *ColCount = nullptr;  // n
  int *IPerm = nullptr;     // n
  size_t nzmax = 0;
  size_t *p = nullptr;      // n+1, value offset of each column
  int *i = nullptr;
  size_t nsuper = 0;
  size_t ssize = 0;
  size_t xsize = 0;
  size_t maxcsize = 0, maxesize = 0;
  int *super = nullptr;     // nsuper+1, first column of each supernode
  int *col2Sup = nullptr;   // n
  size_t *i_ptr = nullptr;  // n+1, row-list start of each column's supernode
  int *s = nullptr;         // row lists
  int *sParent = nullptr;   // nsuper, supernodal assembly tree
  int *Parent = nullptr;    // n, elimination tree
  int ordering = CHOLMOD_METIS;
  int is_ll = FALSE, is_super = TRUE, is_monotonic = TRUE;
  int itype = 0, xtype = CHOLMOD_REAL, dtype = 0;
  int useGPU = 1;
};

}  // namespace nasoq
#endif
