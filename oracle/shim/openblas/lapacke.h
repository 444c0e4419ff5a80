/* Oracle build only: LAPACKE declarations for SciPy's bundled OpenBLAS
 * ("scipy_" prefixed exports).  Test infrastructure, never part of the GPU
 * product. */
#ifndef NQ_ORACLE_SHIM_LAPACKE_H
#define NQ_ORACLE_SHIM_LAPACKE_H
#ifdef __cplusplus
extern "C" {
#endif
typedef int lapack_int;
typedef int lapack_logical;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
#define LAPACKE_dsytrf scipy_LAPACKE_dsytrf
#define LAPACKE_dlapmt scipy_LAPACKE_dlapmt
lapack_int LAPACKE_dsytrf(int matrix_layout, char uplo, lapack_int n, double *a, lapack_int lda, lapack_int *ipiv);
lapack_int LAPACKE_dlapmt(int matrix_layout, lapack_logical forwrd, lapack_int m, lapack_int n, double *x,
                          lapack_int ldx, lapack_int *k);
#ifdef __cplusplus
}
#endif
#endif
