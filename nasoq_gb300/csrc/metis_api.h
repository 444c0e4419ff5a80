// The two public METIS 5 entry points this library calls, declared with the
// 64-bit idx_t of the CUDA toolkit's static METIS build (libmetis_static.a).
#pragma once
#include <cstdint>
extern "C" {
int METIS_SetDefaultOptions(int64_t *options);
int METIS_NodeND(int64_t *nvtxs, int64_t *xadj, int64_t *adjncy, int64_t *vwgt, int64_t *options, int64_t *perm,
                 int64_t *iperm);
}
