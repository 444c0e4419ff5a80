/* Oracle build only: the public METIS 5 entry points, declared with the
 * 64-bit idx_t that the CUDA toolkit's static METIS library uses. */
#ifndef NQ_ORACLE_SHIM_METIS_H
#define NQ_ORACLE_SHIM_METIS_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef int64_t idx_t;
typedef float real_t;
#define METIS_NOPTIONS 40
#define METIS_OK 1
int METIS_SetDefaultOptions(idx_t *options);
int METIS_NodeND(idx_t *nvtxs, idx_t *xadj, idx_t *adjncy, idx_t *vwgt, idx_t *options, idx_t *perm, idx_t *iperm);
#ifdef __cplusplus
}
#endif
#endif
