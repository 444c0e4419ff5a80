/* Oracle build only: CBLAS declarations for the OpenBLAS copy bundled with
 * SciPy, whose exported names carry a "scipy_" prefix.  This header declares
 * the standard CBLAS prototypes the reference calls and maps them to those
 * names.  It is test infrastructure; the GPU product never includes it. */
#ifndef NQ_ORACLE_SHIM_CBLAS_H
#define NQ_ORACLE_SHIM_CBLAS_H
#ifdef __cplusplus
extern "C" {
#endif
typedef int blasint;
typedef enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_ORDER;
typedef enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113, CblasConjNoTrans = 114 } CBLAS_TRANSPOSE;
typedef enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 } CBLAS_UPLO;
typedef enum CBLAS_DIAG { CblasNonUnit = 131, CblasUnit = 132 } CBLAS_DIAG;
typedef enum CBLAS_SIDE { CblasLeft = 141, CblasRight = 142 } CBLAS_SIDE;

#define cblas_dgemm scipy_cblas_dgemm
#define cblas_dtrsm scipy_cblas_dtrsm
#define cblas_dgemv scipy_cblas_dgemv
#define cblas_dscal scipy_cblas_dscal
#define cblas_dsyr scipy_cblas_dsyr
#define openblas_set_num_threads scipy_openblas_set_num_threads
#define openblas_get_num_procs scipy_openblas_get_num_procs
#define openblas_get_config scipy_openblas_get_config

void cblas_dgemm(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, enum CBLAS_TRANSPOSE, blasint m, blasint n, blasint k,
                 double alpha, const double *a, blasint lda, const double *b, blasint ldb, double beta, double *c,
                 blasint ldc);
void cblas_dtrsm(enum CBLAS_ORDER, enum CBLAS_SIDE, enum CBLAS_UPLO, enum CBLAS_TRANSPOSE, enum CBLAS_DIAG,
                 blasint m, blasint n, double alpha, const double *a, blasint lda, double *b, blasint ldb);
void cblas_dgemv(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, blasint m, blasint n, double alpha, const double *a,
                 blasint lda, const double *x, blasint incx, double beta, double *y, blasint incy);
void cblas_dscal(blasint n, double alpha, double *x, blasint incx);
void cblas_dsyr(enum CBLAS_ORDER, enum CBLAS_UPLO, blasint n, double alpha, const double *x, blasint incx,
                double *a, blasint lda);
void openblas_set_num_threads(int);
int openblas_get_num_procs(void);
char *openblas_get_config(void);
#ifdef __cplusplus
}
#endif
#endif
