/*
 * palial -- command-line driver, drop-in for the reference's palial_src/main.c.
 *
 *   palial -a cholesky|qr|lu -m N -b NB [long options]
 *
 * Same flags and semantics as the reference (palial_src/main.c:63-105): missing arguments
 * or an invalid option print a message and exit 0; N % NB != 0 prints "Tile size does not
 * divide the matrix size. Aborting..." and exits 0.  The matrix is a page-aligned N^2 double
 * buffer in tile layout (main.c:110), QR gets a second N x N workspace S (main.c:42-55,138),
 * and the algorithm runs through the header entry points cholesky()/lu()/qr()
 * (palial_entry.h).  Differences: no OMP_NUM_THREADS is needed (the reference crashes
 * without it, main.c:59), the inputs are seeded (the reference uses srand(time(NULL))), the
 * whole factorization is timed, and one JSON result line is printed.
 *
 * Long options:
 *   --gen ref|spd|uniform   input: the reference's pattern (default), B B^T + N I, U[-1,1)
 *   --seed S                generator seed (default 0)
 *   --block BS              scheduler block size (divides NB, multiple of 64)
 *   --priority 0|1          critical-path list order (default) or program order
 *   --trace FILE            write the per-task trace in the reference's "name, ms" format
 *   --trace-csv FILE        side-car CSV with start/end ns and SM id per task record
 *   --check                 report the normwise residual (random probes, on the GPU)
 *   --quiet                 no JSON line
 */
#define _GNU_SOURCE
#include <getopt.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "palial_descriptor.h"
#include "palial_entry.h"

int MSIZE, BSIZE;

static int parse_gen(const char *s)
{
    if (!strcmp(s, "uniform")) return 0;
    if (!strcmp(s, "spd")) return 1;
    return 2;
}

int main(int argc, char *argv[])
{
    char algorithm[16] = "";
    int gen = 2, check = 0, quiet = 0;
    unsigned long long seed = 0;
    const char *trace = NULL, *trace_csv = NULL;
    palial_opts_default(&palial_entry_opts);
    enum { O_GEN = 1000, O_SEED, O_BLOCK, O_PRIO, O_TRACE, O_TRACECSV, O_CHECK, O_QUIET };
    struct option long_options[] = {
        {"Algorithm", required_argument, NULL, 'a'}, {"Matrix size", required_argument, NULL, 'm'},
        {"Tile size", required_argument, NULL, 'b'}, {"gen", required_argument, NULL, O_GEN},
        {"seed", required_argument, NULL, O_SEED},   {"block", required_argument, NULL, O_BLOCK},
        {"priority", required_argument, NULL, O_PRIO}, {"trace", required_argument, NULL, O_TRACE},
        {"trace-csv", required_argument, NULL, O_TRACECSV}, {"check", no_argument, NULL, O_CHECK},
        {"quiet", no_argument, NULL, O_QUIET},       {NULL, no_argument, NULL, 0}};
    if (argc < 2) {
        printf("Missing arguments.\n");
        printf("Aborting...\n");
        return 0;
    }
    int c;
    while ((c = getopt_long(argc, argv, "a:m:b:h", long_options, NULL)) != -1) {
        switch (c) {
            case 'a': snprintf(algorithm, sizeof algorithm, "%s", optarg); break;
            case 'm': MSIZE = atoi(optarg); break;
            case 'b': BSIZE = atoi(optarg); break;
            case 'h': printf("HELP\n"); return 0;
            case O_GEN: gen = parse_gen(optarg); break;
            case O_SEED: seed = strtoull(optarg, NULL, 10); break;
            case O_BLOCK: palial_entry_opts.block = atoi(optarg); break;
            case O_PRIO: palial_entry_opts.priority = atoi(optarg); break;
            case O_TRACE: trace = optarg; palial_entry_opts.trace = 1; break;
            case O_TRACECSV: trace_csv = optarg; palial_entry_opts.trace = 1; break;
            case O_CHECK: check = 1; break;
            case O_QUIET: quiet = 1; break;
            default:
                printf("Invalid arguments.\n");
                printf("Aborting...\n");
                return 0;
        }
    }
    if (BSIZE <= 0 || MSIZE <= 0 || MSIZE % BSIZE != 0) {
        printf("Tile size does not divide the matrix size. Aborting...\n");
        return 0;
    }
    if (strcmp(algorithm, "cholesky") && strcmp(algorithm, "lu") && strcmp(algorithm, "qr")) {
        /* the reference silently does nothing for an unknown algorithm */
        return 0;
    }
    const size_t bytes = (size_t)MSIZE * MSIZE * sizeof(double);
    double *ptr = NULL;
    if (posix_memalign((void **)&ptr, (size_t)getpagesize(), bytes)) {
        printf("Problem allocating contiguous memory.\n");
        return EXIT_FAILURE;
    }
    MATRIX_desc A = palial_matrix_desc_init(BSIZE, (long)MSIZE * MSIZE, (long)BSIZE * BSIZE, MSIZE);
    A.matrix = ptr;
    int rc = palial_gpu_generate(gen, seed, (const palial_desc *)&A);
    if (rc) {
        fprintf(stderr, "palial: input generation failed: %s\n", palial_gpu_error_string(rc));
        free(ptr);
        return 1;
    }
    double *orig = NULL;
    if (check) {
        orig = (double *)malloc(bytes);
        if (orig) memcpy(orig, ptr, bytes);
    }
    MATRIX_desc S = A;
    S.matrix = NULL;
    if (!strcmp(algorithm, "cholesky")) {
        cholesky(A);
    } else if (!strcmp(algorithm, "qr")) {
        if (posix_memalign(&S.matrix, (size_t)getpagesize(), bytes)) {
            printf("Tile allocation failed.\n");
            return 1;
        }
        memset(S.matrix, 0, bytes);
        qr(A, S);
    } else {
        lu(A);
    }
    const palial_status st = palial_entry_status;
    double resid = -1.0;
    if (check && orig && st.code >= 0) {
        const int alg = !strcmp(algorithm, "cholesky") ? 0 : !strcmp(algorithm, "lu") ? 1 : 2;
        palial_gpu_residual_host(alg, orig, (const palial_desc *)&A, 8, 7, &resid);
    }
    if (trace && st.code >= 0) palial_gpu_trace_dump(trace, trace_csv);
    else if (trace_csv && st.code >= 0) palial_gpu_trace_dump("/dev/null", trace_csv);
    if (!quiet)
        printf("{\"algorithm\": \"%s\", \"n\": %d, \"nb\": %d, \"block\": %d, \"code\": %d, \"seconds\": %.6f, "
               "\"total_seconds\": %.6f, \"tflops\": %.4f, \"tasks\": %lld, \"residual_probe\": %.3e}\n",
               algorithm, MSIZE, BSIZE, palial_entry_opts.block, st.code, st.seconds, st.total_seconds, st.tflops,
               st.ntasks, resid);
    free(orig);
    free(S.matrix);
    free(ptr);
    palial_gpu_finalize();
    return st.code < 0 ? 1 : 0;
}
