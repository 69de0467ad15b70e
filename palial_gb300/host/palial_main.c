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
 *   --seed S                generator seed (default 0; 2 for --batch)
 *   --block BS              scheduler block size (divides NB, multiple of 64)
 *   --priority 0|1          critical-path list order (default) or program order
 *   --trace FILE            write the per-task trace in the reference's "name, ms" format
 *   --trace-csv FILE        side-car CSV with start/end ns and SM id per task record
 *   --check                 report the normwise residual (random probes, on the GPU)
 *   --clocks                add the GPU clock report (NVML samples, device clock estimate)
 *   --quiet                 no JSON line
 * Solve mode (A X = B with K seeded uniform right-hand sides instead of the bare factorization):
 *   --rhs K                 K right-hand sides (Cholesky/LU: 1..16, QR: 1..NB)
 *   --precision P           fp64 | bf16 | fp8 | bf16x3 | tf32x3 | auto: trailing-update precision of the
 *                           Cholesky/LU factorization, refined to FP64 accuracy (QR: fp64 only);
 *                           any precision other than fp64 implies --rhs 1 when --rhs is absent
 *   --ir-tol T, --ir-max N  refinement target backward error and iteration cap
 *   --gmres -1|0|1          GMRES-IR never / automatic / always
 *   --butterfly SEED        LU: factor the random-butterfly transform U^T A V (depth 2, seeded;
 *                           SEED 0 = default) as the refinement's preconditioner; no pivoting
 * Tiled-matrix files ("PALTILE1": magic, int64 n, nb, flags, then the tile layout):
 *   --load FILE             the input matrix from FILE (-m/-b optional; must match when given)
 *   --save FILE             write the input matrix to FILE before the run
 *   --save-result FILE      write the factored matrix to FILE (factorization mode)
 * Batch mode (no -a/-m/-b needed):
 *   --batch COUNT           the synthetic uneven batch: COUNT matrices, N log-uniform in
 *                           [32, 2048), half Cholesky half LU, one persistent launch
 *   --autotune              choose the block size per size class by timing (batch mode)
 *   --solve                 batched solves of the batch (one uniform right-hand side each) to
 *                           FP64-level backward error: FP32 factorizations in one persistent
 *                           launch + FP64 refinement (FP64 fallback per matrix); with --autotune
 *                           block size and precision per algorithm and size class
 */
#define _GNU_SOURCE
#include <getopt.h>
#include <math.h>
#include <stdint.h>
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

/* PALIAL_PREC_* codes by name (index = code; 5 is the batched solves' FP32) */
static const char *const precision_names[] = {"fp64", "bf16", "fp8", "bf16x3", "auto", "fp32", "tf32x3"};

static int parse_precision(const char *s)
{
    for (int i = 0; i < 7; i++)
        if (i != PALIAL_PREC_FP32 && !strcmp(s, precision_names[i])) return i;
    return -1;
}

static const char *precision_name(int p)
{
    return p >= 0 && p < 7 ? precision_names[p] : "?";
}

/* uniform [-1, 1) right-hand sides from splitmix64 (seed, index) */
static uint64_t splitmix(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* a JSON number, or null when it is not finite (JSON has no inf / nan) */
static void json_num(const char *key, double v, const char *fmt)
{
    printf(", \"%s\": ", key);
    if (isfinite(v)) printf(fmt, v);
    else printf("null");
}

static void print_clocks(void)
{
    palial_clock_report c;
    if (palial_gpu_clock_report(&c) == PALIAL_OK)
        printf(", \"clocks\": {\"sm_mhz_start\": %.0f, \"sm_mhz_end\": %.0f, \"sm_mhz_max\": %.0f, "
               "\"sm_mhz_device\": %.0f, \"reasons\": %d}",
               c.sm_mhz_start, c.sm_mhz_end, c.sm_mhz_max, c.sm_mhz_device, c.throttle_reasons);
}

static int run_batch(int count, unsigned long long seed, int autotune, int quiet)
{
    palial_batch_report rep;
    palial_status st;
    int rc = palial_gpu_batch_synthetic(count, seed, 0, 1, autotune, NULL, 3, &palial_entry_opts, &st, &rep);
    if (rc) {
        fprintf(stderr, "palial: batch failed: %s (%s)\n", palial_gpu_error_string(rc), st.message);
        return 1;
    }
    if (!quiet) {
        printf("{\"batch\": %d, \"seed\": %llu, \"autotune\": %d, \"seconds\": %.6f, \"matrices_per_s\": %.1f, "
               "\"tflops\": %.4f, \"classes\": [",
               rep.count, seed, autotune, rep.seconds, rep.matrices_per_s, rep.tflops);
        static const int edges[7] = {32, 64, 128, 256, 512, 1024, 2048};
        int first = 1;
        for (int c = 0; c < 6; c++) {
            if (!rep.count_of_class[c]) continue;
            printf("%s{\"n\": [%d, %d], \"count\": %d, \"block\": %d, \"p50_ms\": %.3f, \"p99_ms\": %.3f}",
                   first ? "" : ", ", edges[c], edges[c + 1], rep.count_of_class[c], rep.bs_of_class[c],
                   rep.p50_ms[c], rep.p99_ms[c]);
            first = 0;
        }
        printf("]}\n");
    }
    return 0;
}

static int run_batch_solve(int count, unsigned long long seed, int autotune, int quiet)
{
    palial_batch_solve_report rep;
    palial_status st;
    int rc = palial_gpu_batch_solve_synthetic(count, seed, 0, 1, autotune, NULL, NULL, 3, &palial_entry_opts, &st,
                                              &rep);
    if (rc && rc != PALIAL_ERR_NOT_CONVERGED) {
        fprintf(stderr, "palial: batch solve failed: %s (%s)\n", palial_gpu_error_string(rc), st.message);
        return 1;
    }
    if (!quiet) {
        printf("{\"batch_solve\": %d, \"seed\": %llu, \"autotune\": %d, \"converged\": %s", rep.count, seed,
               autotune, rc == PALIAL_OK ? "true" : "false");
        json_num("seconds", rep.seconds, "%.6f");
        json_num("matrices_per_s", rep.matrices_per_s, "%.1f");
        json_num("tflops", rep.tflops, "%.4f");
        json_num("max_backward_error", rep.max_backward_error, "%.3e");
        printf(", \"max_refinement_steps\": %d, \"fp64_fallbacks\": %d, \"butterfly_solves\": %d, \"choice\": [",
               rep.max_iters, rep.fallbacks, rep.butterflies);
        static const int edges[7] = {32, 64, 128, 256, 512, 1024, 2048};
        for (int k = 0; k < 12; k++)
            printf("%s{\"alg\": \"%s\", \"n\": [%d, %d], \"block\": %d, \"precision\": \"%s\"}", k ? ", " : "",
                   k < 6 ? "cholesky" : "lu", edges[k % 6], edges[k % 6 + 1], rep.bs_of_class[k],
                   rep.prec_of_class[k] == 2 ? "bf16x3-update+ir" : rep.prec_of_class[k] ? "fp32+ir" : "fp64");
        printf("]}\n");
    }
    return rc ? 1 : 0;
}

int main(int argc, char *argv[])
{
    char algorithm[16] = "";
    int gen = 2, check = 0, quiet = 0, nrhs = 0, batch = 0, autotune = 0, clocks = 0, seed_given = 0, solve = 0;
    unsigned long long seed = 0;
    const char *trace = NULL, *trace_csv = NULL, *load = NULL, *save = NULL, *save_result = NULL;
    palial_opts_default(&palial_entry_opts);
    enum {
        O_GEN = 1000, O_SEED, O_BLOCK, O_PRIO, O_TRACE, O_TRACECSV, O_CHECK, O_QUIET, O_PREC, O_RHS, O_IRTOL,
        O_IRMAX, O_GMRES, O_BATCH, O_AUTOTUNE, O_CLOCKS, O_BUTTERFLY, O_LOAD, O_SAVE, O_SAVERES, O_SOLVE
    };
    struct option long_options[] = {
        {"Algorithm", required_argument, NULL, 'a'}, {"Matrix size", required_argument, NULL, 'm'},
        {"Tile size", required_argument, NULL, 'b'}, {"gen", required_argument, NULL, O_GEN},
        {"seed", required_argument, NULL, O_SEED},   {"block", required_argument, NULL, O_BLOCK},
        {"priority", required_argument, NULL, O_PRIO}, {"trace", required_argument, NULL, O_TRACE},
        {"trace-csv", required_argument, NULL, O_TRACECSV}, {"check", no_argument, NULL, O_CHECK},
        {"quiet", no_argument, NULL, O_QUIET},       {"precision", required_argument, NULL, O_PREC},
        {"rhs", required_argument, NULL, O_RHS},     {"ir-tol", required_argument, NULL, O_IRTOL},
        {"ir-max", required_argument, NULL, O_IRMAX}, {"gmres", required_argument, NULL, O_GMRES},
        {"batch", required_argument, NULL, O_BATCH}, {"autotune", no_argument, NULL, O_AUTOTUNE},
        {"clocks", no_argument, NULL, O_CLOCKS},     {"butterfly", required_argument, NULL, O_BUTTERFLY},
        {"load", required_argument, NULL, O_LOAD},   {"save", required_argument, NULL, O_SAVE},
        {"save-result", required_argument, NULL, O_SAVERES}, {"solve", no_argument, NULL, O_SOLVE},
        {NULL, no_argument, NULL, 0}};
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
            case O_SEED: seed = strtoull(optarg, NULL, 10); seed_given = 1; break;
            case O_BLOCK: palial_entry_opts.block = atoi(optarg); break;
            case O_PRIO: palial_entry_opts.priority = atoi(optarg); break;
            case O_TRACE: trace = optarg; palial_entry_opts.trace = 1; break;
            case O_TRACECSV: trace_csv = optarg; palial_entry_opts.trace = 1; break;
            case O_CHECK: check = 1; break;
            case O_QUIET: quiet = 1; break;
            case O_PREC:
                palial_entry_opts.precision = parse_precision(optarg);
                if (palial_entry_opts.precision < 0) {
                    printf("Invalid arguments.\n");
                    printf("Aborting...\n");
                    return 0;
                }
                break;
            case O_RHS: nrhs = atoi(optarg); break;
            case O_IRTOL: palial_entry_opts.ir_tol = atof(optarg); break;
            case O_IRMAX: palial_entry_opts.ir_max_iter = atoi(optarg); break;
            case O_GMRES: palial_entry_opts.gmres = atoi(optarg); break;
            case O_BATCH: batch = atoi(optarg); break;
            case O_AUTOTUNE: autotune = 1; break;
            case O_SOLVE: solve = 1; break;
            case O_CLOCKS: clocks = 1; palial_entry_opts.trace = 1; break;
            case O_BUTTERFLY:
                palial_entry_opts.reserved[6] = 1;
                palial_entry_opts.reserved[7] = (int)strtoul(optarg, NULL, 10);
                break;
            case O_LOAD: load = optarg; break;
            case O_SAVE: save = optarg; break;
            case O_SAVERES: save_result = optarg; break;
            default:
                printf("Invalid arguments.\n");
                printf("Aborting...\n");
                return 0;
        }
    }
    if (batch > 0) {
        const int rc = solve ? run_batch_solve(batch, seed_given ? seed : 2, autotune, quiet)
                             : run_batch(batch, seed_given ? seed : 2, autotune, quiet);
        palial_gpu_finalize();
        return rc;
    }
    if (load) {
        int fn = 0, fnb = 0;
        if (palial_tiles_read(load, &fn, &fnb, NULL) != PALIAL_OK || (MSIZE && MSIZE != fn) ||
            (BSIZE && BSIZE != fnb)) {
            printf("Invalid arguments.\n");
            printf("Aborting...\n");
            return 0;
        }
        MSIZE = fn;
        BSIZE = fnb;
    }
    if (BSIZE <= 0 || MSIZE <= 0 || MSIZE % BSIZE != 0) {
        printf("Tile size does not divide the matrix size. Aborting...\n");
        return 0;
    }
    if (strcmp(algorithm, "cholesky") && strcmp(algorithm, "lu") && strcmp(algorithm, "qr")) {
        /* the reference silently does nothing for an unknown algorithm */
        return 0;
    }
    const int alg = !strcmp(algorithm, "cholesky") ? 0 : !strcmp(algorithm, "lu") ? 1 : 2;
    if (palial_entry_opts.precision != PALIAL_PREC_FP64 && nrhs <= 0) nrhs = 1;
    if ((nrhs > 0 && ((alg != 2 && nrhs > 16) || (alg == 2 && (nrhs > BSIZE || palial_entry_opts.precision)))) ||
        (palial_entry_opts.reserved[6] && (alg != 1 || nrhs <= 0))) {
        printf("Invalid arguments.\n");
        printf("Aborting...\n");
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
    int rc = load ? palial_tiles_read(load, NULL, NULL, ptr) : palial_gpu_generate(gen, seed, (const palial_desc *)&A);
    if (rc) {
        fprintf(stderr, "palial: input %s failed: %s\n", load ? "file" : "generation", palial_gpu_error_string(rc));
        free(ptr);
        return 1;
    }
    if (save && palial_tiles_write(save, (const palial_desc *)&A) != PALIAL_OK) {
        fprintf(stderr, "palial: cannot write %s\n", save);
        free(ptr);
        return 1;
    }
    if (nrhs > 0) {
        /* solve mode: A X = B, X refined to FP64 accuracy (Cholesky/LU) or by the tile QR */
        double *B = (double *)malloc(sizeof(double) * (size_t)MSIZE * nrhs);
        double *X = (double *)calloc((size_t)MSIZE * nrhs, sizeof(double));
        if (!B || !X) {
            printf("Problem allocating contiguous memory.\n");
            return EXIT_FAILURE;
        }
        const uint64_t key = splitmix(seed * 0xD1B54A32D192ED03ull + 2ull);
        for (size_t i = 0; i < (size_t)MSIZE * nrhs; i++)
            B[i] = (double)(splitmix(key + i) >> 11) * 0x1.0p-52 - 1.0;
        palial_status st;
        if (alg == 2)
            rc = palial_gpu_qr_solve_host(MSIZE, MSIZE, BSIZE, ptr, B, X, nrhs, NULL, &palial_entry_opts, &st);
        else
            rc = palial_gpu_solve_ir_host(alg, (const palial_desc *)&A, B, X, nrhs, &palial_entry_opts, &st);
        if (rc < 0) fprintf(stderr, "palial: solve failed: %s (%s)\n", palial_gpu_error_string(rc), st.message);
        if (!quiet) {
            printf("{\"algorithm\": \"%s\", \"mode\": \"solve\", \"n\": %d, \"nb\": %d, \"nrhs\": %d, "
                   "\"precision\": \"%s\", \"code\": %d, \"ir_iters\": %d, \"gmres_iters\": %d, \"tasks\": %lld",
                   algorithm, MSIZE, BSIZE, nrhs, precision_name(palial_entry_opts.precision), rc, st.ir_iters,
                   st.gmres_iters, st.ntasks);
            json_num("seconds", st.seconds, "%.6f");
            json_num("total_seconds", st.total_seconds, "%.6f");
            json_num("tflops", st.tflops, "%.4f");
            json_num("backward_error", st.backward_error, "%.3e");
            json_num("factor_seconds", st.factor_seconds, "%.6f");
            if (clocks) print_clocks();
            printf("}\n");
        }
        free(B);
        free(X);
        free(ptr);
        palial_gpu_finalize();
        return rc < 0 ? 1 : 0;
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
    if (check && orig && st.code >= 0) palial_gpu_residual_host(alg, orig, (const palial_desc *)&A, 8, 7, &resid);
    if (save_result && st.code >= 0 && palial_tiles_write(save_result, (const palial_desc *)&A) != PALIAL_OK)
        fprintf(stderr, "palial: cannot write %s\n", save_result);
    if (trace && st.code >= 0) palial_gpu_trace_dump(trace, trace_csv);
    else if (trace_csv && st.code >= 0) palial_gpu_trace_dump("/dev/null", trace_csv);
    if (!quiet) {
        printf("{\"algorithm\": \"%s\", \"n\": %d, \"nb\": %d, \"block\": %d, \"code\": %d, \"tasks\": %lld",
               algorithm, MSIZE, BSIZE, palial_entry_opts.block, st.code, st.ntasks);
        json_num("seconds", st.seconds, "%.6f");
        json_num("total_seconds", st.total_seconds, "%.6f");
        json_num("tflops", st.tflops, "%.4f");
        json_num("residual_probe", resid, "%.3e");
        if (clocks) print_clocks();
        printf("}\n");
    }
    free(orig);
    free(S.matrix);
    free(ptr);
    palial_gpu_finalize();
    return st.code < 0 ? 1 : 0;
}
