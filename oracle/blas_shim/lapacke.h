/*
 * Minimal LAPACKE declarations for the CPU oracle (test infrastructure only).
 *
 * Maps the LAPACKE routines used by the reference's tile kernels (src/cholesky.h:40,
 * src/srclu/dgetrf_no_pivot.h:16, src/srcqr/dgeqrt.h:18-34, src/srcqr/dormqr.h:35-50,
 * src/srcqr/dtsqrt.h:23-26, src/srcqr/dpamm.h:22-29) onto SciPy's bundled OpenBLAS
 * (32-bit integers, "scipy_" symbol prefix).
 */
#ifndef PALIAL_ORACLE_LAPACKE_H
#define PALIAL_ORACLE_LAPACKE_H

#ifdef __cplusplus
extern "C" {
#endif

#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
typedef int lapack_int;

#define LAPACKE_dpotrf scipy_LAPACKE_dpotrf
#define LAPACKE_dgeqr2_work scipy_LAPACKE_dgeqr2_work
#define LAPACKE_dlarft_work scipy_LAPACKE_dlarft_work
#define LAPACKE_dlarfb_work scipy_LAPACKE_dlarfb_work
#define LAPACKE_dlarfg_work scipy_LAPACKE_dlarfg_work
#define LAPACKE_dlacpy scipy_LAPACKE_dlacpy
#define LAPACKE_dlamch_work scipy_LAPACKE_dlamch_work

lapack_int LAPACKE_dpotrf(int layout, char uplo, lapack_int n, double *a, lapack_int lda);
lapack_int LAPACKE_dgeqr2_work(int layout, lapack_int m, lapack_int n, double *a,
                               lapack_int lda, double *tau, double *work);
lapack_int LAPACKE_dlarft_work(int layout, char direct, char storev, lapack_int n,
                               lapack_int k, const double *v, lapack_int ldv,
                               const double *tau, double *t, lapack_int ldt);
lapack_int LAPACKE_dlarfb_work(int layout, char side, char trans, char direct, char storev,
                               lapack_int m, lapack_int n, lapack_int k, const double *v,
                               lapack_int ldv, const double *t, lapack_int ldt, double *c,
                               lapack_int ldc, double *work, lapack_int ldwork);
lapack_int LAPACKE_dlarfg_work(lapack_int n, double *alpha, double *x, lapack_int incx,
                               double *tau);
lapack_int LAPACKE_dlacpy(int layout, char uplo, lapack_int m, lapack_int n, const double *a,
                          lapack_int lda, double *b, lapack_int ldb);
double LAPACKE_dlamch_work(char cmach);

#ifdef __cplusplus
}
#endif
#endif
