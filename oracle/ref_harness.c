/*
 * Harness that compiles the REFERENCE's own hot-path sources, unmodified, into a shared
 * library so that tests can run the reference on seeded tile buffers.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by oracle/build_oracle.py into oracle/_ref/ (git-ignored)
 * from the sources where they lie in the reference checkout; nothing here is shipped.
 *
 * It includes include/descriptor.h, include/tile_address.h and src/{cholesky,qr,lu}.h of
 * the reference in the same order as palial_src/main.c:32-40, defines the A(m,n)/S(m,n)
 * macros the way palial_src/main.c:25-27 does, and stubs the three weak trace hooks of
 * include/common.h:9-11 (without them the reference segfaults on the first task).  The
 * algorithm runs inside `omp parallel` + `omp master` as in palial_src/main.c:126-159; the
 * whole parallel region is timed (main.c's own timer stops before the tasks finish).
 * Built twice: without -fopenmp (serial program order: the parity oracle) and with it (the
 * timed CPU baseline).
 */
#define _GNU_SOURCE
#include <assert.h>
#include <sched.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#include <unistd.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "cblas.h"
#include "lapacke.h"

#define A(m, n) MATRIX_tile_address(A, m, n)
#define S(m, n) MATRIX_tile_address(S, m, n)

void palial_set_task_name(const char *name) { (void)name; }
void palial_set_task_cpu_node(int cpu, int node, char *name) { (void)cpu; (void)node; (void)name; }
void palial_get_task_time(struct timeval start, struct timeval end, char *name)
{
    (void)start; (void)end; (void)name;
}

#include "descriptor.h"
#include "tile_address.h"
#include "cholesky.h"
#include "qr.h"
#include "lu.h"

static double ref_now(void)
{
    struct timeval tv;
    gettimeofday(&tv, NULL);
    return (double)tv.tv_sec + 1e-6 * (double)tv.tv_usec;
}

static MATRIX_desc ref_desc(int n, int nb, double *buf)
{
    MATRIX_desc d = matrix_desc_init(nb, (long)n * n, (long)nb * nb, n);
    d.matrix = buf;
    return d;
}

/* 0 = Cholesky, 1 = LU, 2 = QR (S may be NULL otherwise). Returns wall seconds. */
double ref_run(int alg, int n, int nb, double *a, double *s, int nthreads)
{
    MATRIX_desc Ad = ref_desc(n, nb, a);
    MATRIX_desc Sd = ref_desc(n, nb, s);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    double t0 = ref_now();
#pragma omp parallel
#pragma omp master
    {
        if (alg == 0) cholesky(Ad);
        else if (alg == 1) lu(Ad);
        else qr(Ad, Sd);
    }
    return ref_now() - t0;
}

/* The reference's compile-time 4x4 fixture (include/populate.h:13-33, NB = 2), written
 * by the reference's own generator into a tile-layout buffer of 16 doubles. */
#define SPECIAL4x4 1
#include "populate.h"
void ref_populate_special4x4(double *a)
{
    MATRIX_desc Ad = ref_desc(4, 2, a);
    hermitian_positive_generator(Ad);
}

int ref_is_openmp(void)
{
#ifdef _OPENMP
    return 1;
#else
    return 0;
#endif
}
