/*
 * Minimal CBLAS declarations for the CPU oracle (test infrastructure only).
 *
 * The reference links CBLAS from OpenBLAS through pkg-config (palial_src/Makefile:18).
 * No system OpenBLAS exists on these machines, but SciPy bundles OpenBLAS with every
 * symbol prefixed by "scipy_".  This header declares the CBLAS routines that the
 * reference's hot path calls and maps each standard name onto the prefixed export.
 * The enum values are the CBLAS standard ones; the reference relies on them being equal
 * to its own PALIAL_* constants (src/common.h:9-22).
 */
#ifndef PALIAL_ORACLE_CBLAS_H
#define PALIAL_ORACLE_CBLAS_H

#ifdef __cplusplus
extern "C" {
#endif

enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 };
enum CBLAS_DIAG { CblasNonUnit = 131, CblasUnit = 132 };
enum CBLAS_SIDE { CblasLeft = 141, CblasRight = 142 };

#define cblas_dgemm scipy_cblas_dgemm
#define cblas_dtrsm scipy_cblas_dtrsm
#define cblas_dtrmm scipy_cblas_dtrmm
#define cblas_dsyrk scipy_cblas_dsyrk
#define cblas_dscal scipy_cblas_dscal
#define cblas_daxpy scipy_cblas_daxpy
#define cblas_dcopy scipy_cblas_dcopy
#define cblas_dger scipy_cblas_dger
#define cblas_dgemv scipy_cblas_dgemv
#define cblas_dtrmv scipy_cblas_dtrmv

void cblas_dgemm(int order, int transa, int transb, int m, int n, int k, double alpha,
                 const double *a, int lda, const double *b, int ldb, double beta, double *c,
                 int ldc);
void cblas_dtrsm(int order, int side, int uplo, int transa, int diag, int m, int n,
                 double alpha, const double *a, int lda, double *b, int ldb);
void cblas_dtrmm(int order, int side, int uplo, int transa, int diag, int m, int n,
                 double alpha, const double *a, int lda, double *b, int ldb);
void cblas_dsyrk(int order, int uplo, int trans, int n, int k, double alpha, const double *a,
                 int lda, double beta, double *c, int ldc);
void cblas_dscal(int n, double alpha, double *x, int incx);
void cblas_daxpy(int n, double alpha, const double *x, int incx, double *y, int incy);
void cblas_dcopy(int n, const double *x, int incx, double *y, int incy);
void cblas_dger(int order, int m, int n, double alpha, const double *x, int incx,
                const double *y, int incy, double *a, int lda);
void cblas_dgemv(int order, int trans, int m, int n, double alpha, const double *a, int lda,
                 const double *x, int incx, double beta, double *y, int incy);
void cblas_dtrmv(int order, int uplo, int trans, int diag, int n, const double *a, int lda,
                 double *x, int incx);

#ifdef __cplusplus
}
#endif
#endif
