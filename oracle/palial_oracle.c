/*
 * palial_oracle.c -- CPU oracle for the tiled Cholesky / LU / QR hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg load this library, and only as the checker or the timed CPU baseline.  The
 * GPU library never links, loads or calls it.
 *
 * It restates the reference's algorithm in plain C: the three right-looking tile DAGs of
 * src/cholesky.h, src/lu.h and src/qr.h, and PALIAL's own tile kernels in src/srclu and
 * src/srcqr.  The arithmetic goes through the same CBLAS/LAPACKE routines with the same
 * arguments (here: SciPy's bundled OpenBLAS, via blas_shim/), so in serial program order
 * the results are bit-identical to the reference built against the same OpenBLAS.
 *
 * Storage is the reference's tile layout (include/tile_address.h:9-17): tile (m,n) is an
 * NB x NB column-major block at element offset NB*NB*(m + MT*n), MT = N/NB.
 *
 * nthreads <= 1 runs the DAG in serial program order (the parity oracle).  nthreads > 1
 * runs it as OpenMP tasks with tile dependences, which is how the reference executes it.
 * For LU, `racy_deps` = 1 reproduces the reference's dependence clauses on the two TRSM
 * tasks (src/lu.h:62 and :104 name the element one tile past the written tile), which lets
 * GEMMs overtake the TRSMs they read; 0 uses the true dependences.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <sys/time.h>

#include "cblas.h"
#include "lapacke.h"

enum { ORC_LEFT = 141, ORC_TRANS = 112, ORC_NOTRANS = 111, ORC_UPPER = 121 };

static inline double *tile_at(double *base, int n, int nb, int m, int k)
{
    return base + (size_t)nb * nb * ((size_t)m + (size_t)(n / nb) * (size_t)k);
}

static double wall_seconds(void)
{
    struct timeval tv;
    gettimeofday(&tv, NULL);
    return (double)tv.tv_sec + 1e-6 * (double)tv.tv_usec;
}

/* ------------------------------------------------------------------------------------ */
/* Tile kernels                                                                          */
/* ------------------------------------------------------------------------------------ */

/* Unblocked no-pivot LU of one tile (src/srclu/dgetrf_no_pivot.h:11-57, reached through
 * the single-iteration blocked wrapper src/srclu/dgetrf.h:11-59).  Column i is scaled by
 * the reciprocal of the pivot when |pivot| > safe minimum, divided otherwise, and left
 * alone when the pivot is exactly zero; the rank-1 trailing update always runs. */
int orc_dgetrf_nopiv(int nb, double *a, int lda)
{
    if (nb == 0) return 0;
    const double sfmin = LAPACKE_dlamch_work('S');
    for (int i = 0; i < nb; i++) {
        double piv = a[(size_t)i * lda + i];
        if (piv != 0.0) {
            if (fabs(piv) > sfmin) {
                cblas_dscal(nb - i - 1, 1.0 / piv, &a[(size_t)i * lda + i + 1], 1);
            } else {
                for (int r = i + 1; r < nb; r++) a[(size_t)i * lda + r] /= piv;
            }
        }
        cblas_dger(CblasColMajor, nb - i - 1, nb - i - 1, -1.0, &a[(size_t)i * lda + i + 1], 1,
                   &a[(size_t)(i + 1) * lda + i], lda, &a[(size_t)(i + 1) * lda + i + 1], lda);
    }
    return 0;
}

/* GEQRT with inner block = NB (src/srcqr/dgeqrt.h:9-56): dgeqr2 on the tile, then the
 * forward column-wise triangular factor T with dlarft.  The dlarfb branch at :35-53 never
 * runs because the inner block covers the tile.  tau[] receives the reflector scalars. */
int orc_dgeqrt(int nb, double *a, int lda, double *t, int ldt, double *tau, double *work)
{
    if (nb == 0) return 0;
    LAPACKE_dgeqr2_work(LAPACK_COL_MAJOR, nb, nb, a, lda, tau, work);
    LAPACKE_dlarft_work(LAPACK_COL_MAJOR, 'F', 'C', nb, nb, a, lda, tau, t, ldt);
    return 0;
}

/* ORMQR, left / transpose, one block reflector over the whole tile
 * (src/srcqr/dormqr.h:9-53): C <- (I - V T V^T)^T C with V unit lower triangular. */
int orc_dormqr(int nb, const double *v, int ldv, const double *t, int ldt, double *c, int ldc,
               double *work)
{
    if (nb == 0) return 0;
    LAPACKE_dlarfb_work(LAPACK_COL_MAJOR, 'L', 'T', 'F', 'C', nb, nb, nb, v, ldv, t, ldt, c, ldc,
                        work, nb);
    return 0;
}

/* TSQRT: QR of the stacked pair [A1 upper triangle; A2] (src/srcqr/dtsqrt.h:11-109).
 * Column by column: dlarfg over (A1(i,i), A2(:,i)); apply the reflector to the columns
 * right of i (dcopy + dgemv + daxpy + dger); then T(0:i,i) = -tau_i * T(0:i,0:i) *
 * A2(:,0:i)^T A2(:,i) (dgemv + dtrmv) and T(i,i) = tau_i.  The trailing TSMQR at :88-106
 * is dead because the inner block covers the tile. */
int orc_dtsqrt(int nb, double *a1, int lda1, double *a2, int lda2, double *t, int ldt,
               double *tau, double *work)
{
    if (nb == 0) return 0;
    for (int i = 0; i < nb; i++) {
        LAPACKE_dlarfg_work(nb + 1, &a1[(size_t)lda1 * i + i], &a2[(size_t)lda2 * i], 1, &tau[i]);
        if (i + 1 < nb) {
            const int rest = nb - i - 1;
            const double mtau = -tau[i];
            cblas_dcopy(rest, &a1[(size_t)lda1 * (i + 1) + i], lda1, work, 1);
            cblas_dgemv(CblasColMajor, CblasTrans, nb, rest, 1.0, &a2[(size_t)lda2 * (i + 1)],
                        lda2, &a2[(size_t)lda2 * i], 1, 1.0, work, 1);
            cblas_daxpy(rest, mtau, work, 1, &a1[(size_t)lda1 * (i + 1) + i], lda1);
            cblas_dger(CblasColMajor, nb, rest, mtau, &a2[(size_t)lda2 * i], 1, work, 1,
                       &a2[(size_t)lda2 * (i + 1)], lda2);
        }
        cblas_dgemv(CblasColMajor, CblasTrans, nb, i, -tau[i], a2, lda2, &a2[(size_t)lda2 * i], 1,
                    0.0, &t[(size_t)ldt * i], 1);
        cblas_dtrmv(CblasColMajor, CblasUpper, CblasNoTrans, CblasNonUnit, i, t, ldt,
                    &t[(size_t)ldt * i], 1);
        t[(size_t)ldt * i + i] = tau[i];
    }
    return 0;
}

/* TSMQR, left / transpose, K = NB, L = 0 (src/srcqr/dtsmqr.h:11-59 -> dparfb.h:14-135 ->
 * dpamm.h).  With L = 0 the only live calls of dpamm are W = V^T A2 (dgemm, beta 0)
 * followed by W += A1 (dpamm.h:64-87), and A2 -= V W (dpamm.h:226-239); between them dparfb
 * forms W = T^T W (dtrmm) and A1 -= W.  `work` holds W (NB x NB). */
int orc_dtsmqr(int nb, double *a1, int lda1, double *a2, int lda2, const double *v, int ldv,
               const double *t, int ldt, double *work)
{
    if (nb == 0) return 0;
    const int ldw = nb;
    cblas_dgemm(CblasColMajor, CblasTrans, CblasNoTrans, nb, nb, nb, 1.0, v, ldv, a2, lda2, 0.0,
                work, ldw);
    for (int j = 0; j < nb; j++)
        cblas_daxpy(nb, 1.0, &a1[(size_t)lda1 * j], 1, &work[(size_t)ldw * j], 1);
    cblas_dtrmm(CblasColMajor, CblasLeft, CblasUpper, CblasTrans, CblasNonUnit, nb, nb, 1.0, t,
                ldt, work, ldw);
    for (int j = 0; j < nb; j++)
        cblas_daxpy(nb, -1.0, &work[(size_t)ldw * j], 1, &a1[(size_t)lda1 * j], 1);
    cblas_dgemm(CblasColMajor, CblasNoTrans, CblasNoTrans, nb, nb, nb, -1.0, v, ldv, work, ldw,
                1.0, a2, lda2);
    return 0;
}

/* ------------------------------------------------------------------------------------ */
/* Task bodies shared by the serial and the OpenMP runners                               */
/* ------------------------------------------------------------------------------------ */

static void chol_potrf(int nb, double *akk) { LAPACKE_dpotrf(LAPACK_COL_MAJOR, 'U', nb, akk, nb); }

static void chol_trsm(int nb, const double *akk, double *akm)
{
    cblas_dtrsm(CblasColMajor, CblasLeft, CblasUpper, CblasTrans, CblasNonUnit, nb, nb, 1.0, akk,
                nb, akm, nb);
}

static void chol_syrk(int nb, const double *akm, double *amm)
{
    cblas_dsyrk(CblasColMajor, CblasUpper, CblasTrans, nb, nb, -1.0, akm, nb, 1.0, amm, nb);
}

static void chol_gemm(int nb, const double *akn, const double *akm, double *anm)
{
    cblas_dgemm(CblasColMajor, CblasTrans, CblasNoTrans, nb, nb, nb, -1.0, akn, nb, akm, nb, 1.0,
                anm, nb);
}

static void lu_trsm_right(int nb, const double *akk, double *amk)
{
    cblas_dtrsm(CblasColMajor, CblasRight, CblasUpper, CblasNoTrans, CblasNonUnit, nb, nb, 1.0,
                akk, nb, amk, nb);
}

static void lu_trsm_left(int nb, const double *akk, double *akn)
{
    cblas_dtrsm(CblasColMajor, CblasLeft, CblasLower, CblasNoTrans, CblasUnit, nb, nb, 1.0, akk, nb,
                akn, nb);
}

static void lu_gemm(int nb, const double *amk, const double *akn, double *amn)
{
    cblas_dgemm(CblasColMajor, CblasNoTrans, CblasNoTrans, nb, nb, nb, -1.0, amk, nb, akn, nb, 1.0,
                amn, nb);
}

static void qr_geqrt(int nb, double *akk, double *skk)
{
    double *tau = (double *)malloc(sizeof(double) * (size_t)nb);
    double *work = (double *)malloc(sizeof(double) * (size_t)nb * nb);
    orc_dgeqrt(nb, akk, nb, skk, nb, tau, work);
    free(work);
    free(tau);
}

static void qr_ormqr(int nb, const double *akk, const double *skk, double *akn)
{
    double *work = (double *)malloc(sizeof(double) * (size_t)nb * nb);
    orc_dormqr(nb, akk, nb, skk, nb, akn, nb, work);
    free(work);
}

static void qr_tsqrt(int nb, double *akk, double *amk, double *smk)
{
    double *tau = (double *)malloc(sizeof(double) * (size_t)nb);
    double *work = (double *)malloc(sizeof(double) * (size_t)nb * nb);
    orc_dtsqrt(nb, akk, nb, amk, nb, smk, nb, tau, work);
    free(work);
    free(tau);
}

static void qr_tsmqr(int nb, double *akn, double *amn, const double *amk, const double *smk)
{
    double *work = (double *)malloc(sizeof(double) * (size_t)nb * nb);
    orc_dtsmqr(nb, akn, nb, amn, nb, amk, nb, smk, nb, work);
    free(work);
}

/* ------------------------------------------------------------------------------------ */
/* DAGs                                                                                  */
/* ------------------------------------------------------------------------------------ */

/* Upper tile Cholesky A = U^T U (src/cholesky.h:12-177).  Per step k: POTRF(k,k); TRSM
 * on every A(k,m), m > k; then for each m > k the SYRK into A(m,m) and the GEMMs into
 * A(n,m), k < n < m.  Tiles below the diagonal are never touched. */
static void cholesky_dag(int n, int nb, double *a)
{
    const int mt = n / nb;
    for (int k = 0; k < mt; k++) {
        double *akk = tile_at(a, n, nb, k, k);
#pragma omp task depend(inout : akk[0])
        chol_potrf(nb, akk);
        for (int m = k + 1; m < mt; m++) {
            double *akm = tile_at(a, n, nb, k, m);
#pragma omp task depend(in : akk[0]) depend(inout : akm[0])
            chol_trsm(nb, akk, akm);
        }
        for (int m = k + 1; m < mt; m++) {
            double *akm = tile_at(a, n, nb, k, m);
            double *amm = tile_at(a, n, nb, m, m);
#pragma omp task depend(in : akm[0]) depend(inout : amm[0])
            chol_syrk(nb, akm, amm);
            for (int j = k + 1; j < m; j++) {
                double *akj = tile_at(a, n, nb, k, j);
                double *ajm = tile_at(a, n, nb, j, m);
#pragma omp task depend(in : akj[0], akm[0]) depend(inout : ajm[0])
                chol_gemm(nb, akj, akm, ajm);
            }
        }
    }
}

/* No-pivot tile LU (src/lu.h:11-175).  Per step k: GETRF(k,k); TRSM-right on A(m,k);
 * then for each n > k the TRSM-left on A(k,n) and the GEMMs A(m,n) -= A(m,k) A(k,n). */
static void lu_dag(int n, int nb, double *a, int racy_deps)
{
    const int mt = n / nb;
    /* The reference's TRSM tasks declare their output dependence on tileB[NB*NB]
     * (src/lu.h:62,104): the first element of the NEXT tile in memory. */
    const size_t out_off = racy_deps ? (size_t)nb * nb : 0;
    for (int k = 0; k < mt; k++) {
        double *akk = tile_at(a, n, nb, k, k);
#pragma omp task depend(inout : akk[0])
        orc_dgetrf_nopiv(nb, akk, nb);
        for (int m = k + 1; m < mt; m++) {
            double *amk = tile_at(a, n, nb, m, k);
            double *dep = amk + out_off;
#pragma omp task depend(in : akk[0]) depend(inout : dep[0])
            lu_trsm_right(nb, akk, amk);
        }
        for (int j = k + 1; j < mt; j++) {
            double *akj = tile_at(a, n, nb, k, j);
            double *dep = akj + out_off;
#pragma omp task depend(in : akk[0]) depend(inout : dep[0])
            lu_trsm_left(nb, akk, akj);
            for (int m = k + 1; m < mt; m++) {
                double *amk = tile_at(a, n, nb, m, k);
                double *amj = tile_at(a, n, nb, m, j);
#pragma omp task depend(in : amk[0], akj[0]) depend(inout : amj[0])
                lu_gemm(nb, amk, akj, amj);
            }
        }
    }
}

/* Flat-tree TS tile QR (src/qr.h:15-192).  Per step k: GEQRT(k,k) -> S(k,k); ORMQR on
 * A(k,n); then for each m > k: TSQRT on (A(k,k), A(m,k)) -> S(m,k) and TSMQR on
 * (A(k,n), A(m,n)) with V = A(m,k), T = S(m,k). */
static void qr_dag(int n, int nb, double *a, double *s)
{
    const int mt = n / nb;
    for (int k = 0; k < mt; k++) {
        double *akk = tile_at(a, n, nb, k, k);
        double *skk = tile_at(s, n, nb, k, k);
#pragma omp task depend(inout : akk[0]) depend(out : skk[0])
        qr_geqrt(nb, akk, skk);
        for (int j = k + 1; j < mt; j++) {
            double *akj = tile_at(a, n, nb, k, j);
#pragma omp task depend(in : akk[0], skk[0]) depend(inout : akj[0])
            qr_ormqr(nb, akk, skk, akj);
        }
        for (int m = k + 1; m < mt; m++) {
            double *amk = tile_at(a, n, nb, m, k);
            double *smk = tile_at(s, n, nb, m, k);
#pragma omp task depend(inout : akk[0], amk[0]) depend(out : smk[0])
            qr_tsqrt(nb, akk, amk, smk);
            for (int j = k + 1; j < mt; j++) {
                double *akj = tile_at(a, n, nb, k, j);
                double *amj = tile_at(a, n, nb, m, j);
#pragma omp task depend(inout : akj[0], amj[0]) depend(in : amk[0], smk[0])
                qr_tsmqr(nb, akj, amj, amk, smk);
            }
        }
    }
}

/* ------------------------------------------------------------------------------------ */
/* Exported runners: 0 = Cholesky, 1 = LU, 2 = QR.  Return wall seconds of the whole      */
/* region (tasks included), or a negative value on bad arguments.                        */
/* ------------------------------------------------------------------------------------ */

double orc_run(int alg, int n, int nb, double *a, double *s, int nthreads, int racy_deps)
{
    if (nb <= 0 || n <= 0 || n % nb != 0) return -1.0;
    if (alg == 2 && s == NULL) return -1.0;
    double t0 = wall_seconds();
#ifdef _OPENMP
    if (nthreads > 1) {
#pragma omp parallel num_threads(nthreads)
#pragma omp single
        {
            if (alg == 0) cholesky_dag(n, nb, a);
            else if (alg == 1) lu_dag(n, nb, a, racy_deps);
            else qr_dag(n, nb, a, s);
        }
        return wall_seconds() - t0;
    }
#endif
    /* Outside a parallel region every `omp task` runs immediately: serial program order. */
    if (alg == 0) cholesky_dag(n, nb, a);
    else if (alg == 1) lu_dag(n, nb, a, racy_deps);
    else qr_dag(n, nb, a, s);
    return wall_seconds() - t0;
}

int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
