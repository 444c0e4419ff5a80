// Drop-in subset of the reference's include/nasoq/QP/qp_utils.h: the
// (index, value) pair of the batched active-set variant and its helpers
// (qp_utils.h:121-132).
#ifndef NASOQ_GB300_QP_UTILS_H
#define NASOQ_GB300_QP_UTILS_H

#include <vector>

#include "nasoq/common/def.h"

namespace nasoq {

struct idx_val {
  double val;
  int idx;
  idx_val();
  idx_val(int i, double v);
};

// ascending by value
bool CMP(idx_val a, idx_val b);

// erases the first pair with idx == c_no; 1 if one was found
int remove_from_list(std::vector<idx_val> &list_const, int c_no);

}  // namespace nasoq
#endif
