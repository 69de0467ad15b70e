/*
 * palial_gpu.h -- C ABI of libpalial_gpu.so, the GB300 (sm_103a) implementation of PALIAL's
 * tiled dense Cholesky / LU / QR.
 *
 * Plain C types only: host or device pointers, sizes, small POD structs.  Every call is
 * synchronous (results are valid on return) unless it takes a `stream` argument, in which
 * case it is ordered on that CUDA stream (a cudaStream_t passed as void*, NULL = legacy
 * default stream).  Calls are not re-entrant: use one host thread per device.
 *
 * Return value of every entry point: PALIAL_OK (0), or a negative PALIAL_ERR_* code with
 * details in the optional palial_status out-parameter.
 *
 * Storage is the reference's tile layout (reference include/tile_address.h:9-17): tile (m,n)
 * of an N x N matrix with tile size NB is an NB x NB column-major block at element offset
 * NB*NB*(m + (N/NB)*n).  N % NB must be 0 (reference palial_src/main.c:101-105).
 */
#ifndef PALIAL_GPU_H
#define PALIAL_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------------------- */
#define PALIAL_OK 0
#define PALIAL_ERR_ARG -1          /* bad argument (N % NB, NULL buffer, unsupported size)   */
#define PALIAL_ERR_CUDA -2         /* a CUDA runtime call failed; status.cuda_error has it   */
#define PALIAL_ERR_NOT_SPD -3      /* Cholesky met a non-positive pivot (status.tile/column) */
#define PALIAL_ERR_TIMEOUT -4      /* a device dependency wait passed its deadline          */
#define PALIAL_ERR_NO_DEVICE -5    /* no CUDA device / library not initialised             */
#define PALIAL_ERR_NOT_CONVERGED -6 /* iterative refinement stopped above its tolerance     */
#define PALIAL_ERR_NOMEM -7        /* device allocation failed                              */
#define PALIAL_WARN_ZERO_PIVOT 1   /* LU met an exact zero pivot and skipped it (as the
                                      reference does, src/srclu/dgetrf_no_pivot.h:21)       */

/* ---- algorithms, precisions ------------------------------------------------------------ */
#define PALIAL_ALG_CHOLESKY 0
#define PALIAL_ALG_LU 1
#define PALIAL_ALG_QR 2

#define PALIAL_PREC_FP64 0         /* every task in FP64                                    */
#define PALIAL_PREC_BF16 1         /* trailing updates in BF16 on tcgen05, FP32 accumulate  */
#define PALIAL_PREC_FP8 2          /* trailing updates in FP8 e4m3, per-tile scale          */
#define PALIAL_PREC_BF16X3 3       /* trailing updates as 3 BF16 products (split operands)  */
#define PALIAL_PREC_AUTO 4         /* solve_ir: precision ladder BF16 -> BF16x3 -> FP64      */
#define PALIAL_PREC_FP32 5         /* batched solves: FP32 factorization, FP64 refinement    */
#define PALIAL_PREC_TF32X3 6       /* trailing updates as 3 TF32 products (split operands):
                                      FP32-level factors on tcgen05 (kind::tf32)            */

/* ---- descriptor ------------------------------------------------------------------------ */
/* Same field order, types and meaning as the reference's MATRIX_desc
 * (reference include/descriptor.h:13-20), so a MATRIX_desc* may be passed where a
 * palial_desc* is expected. */
typedef struct palial_desc {
    int tile_size;          /* NB                                   */
    long matrix_nelements;  /* N * N                                */
    long tile_nelements;    /* NB * NB                              */
    int matrix_size;        /* N                                    */
    void *matrix;           /* N*N doubles in tile layout (host)    */
} palial_desc;

/* ---- options / status ------------------------------------------------------------------ */
typedef struct palial_opts {
    int precision;          /* PALIAL_PREC_*, plain FP64 = 0                          */
    int block;              /* scheduler block size (divides NB); 0 = automatic       */
    int workers_per_sm;     /* persistent CTAs per SM (1 or 2); 0 = automatic         */
    int max_sms;            /* use at most this many SMs; 0 = all                     */
    int priority;           /* 0 = critical-path list order, 1 = program order,
                               2 = caller-supplied costs (palial_gpu_set_task_costs)  */
    int trace;              /* 1 = record a per-task device trace                     */
    double timeout_s;       /* deadline of every device dependency wait; 0 = 120 s    */
    unsigned int shuffle_seed; /* nonzero: randomise ties in the dispatch order (tests) */
    int ir_max_iter;        /* refinement iteration cap (0 = 50)                      */
    double ir_tol;          /* target normwise backward error (0 = 1e-14 * N)         */
    int gmres;              /* -1 never, 0 automatic (kappa estimate > 1e8), 1 always */
    int reserved[8];
} palial_opts;

typedef struct palial_status {
    int code;               /* same as the return value                               */
    int cuda_error;         /* cudaError_t of the failing call, if any                */
    int task;               /* task index (dispatch order) of a device error          */
    int tile_m, tile_n;     /* tile of a numerical error                              */
    int column;             /* column inside the tile (NOT_SPD)                       */
    long long ntasks;       /* tasks executed                                         */
    double seconds;         /* device time of the factorization (CUDA events)         */
    double total_seconds;   /* wall time of the call, host copies included            */
    double tflops;          /* algorithmic flops / seconds * 1e-12                    */
    int ir_iters;           /* refinement iterations (solve_ir)                       */
    int gmres_iters;        /* total inner GMRES iterations (solve_ir)                */
    double backward_error;  /* final normwise backward error (solve_ir)               */
    double kappa_est;       /* condition estimate used to choose the method (-1: none) */
    double factor_seconds;  /* time of the factorization part (solve_ir)              */
    double shift;           /* diagonal shift used by a low-precision Cholesky        */
    int precision_used;     /* solves: PALIAL_PREC_* of the factorization that produced X
                               (+100: LU of the random-butterfly transform)           */
    int fallbacks;          /* batched solves: matrices refactored in FP64            */
    int butterflies;        /* batched solves: no-pivot LU matrices solved on their
                               random-butterfly transform after FP32 LU failed          */
    char message[160];
} palial_status;

void palial_opts_default(palial_opts *opts);

/* ---- library ---------------------------------------------------------------------------- */
int palial_gpu_init(int device);      /* select device, query SM count; idempotent     */
int palial_gpu_finalize(void);        /* release cached device buffers                  */
int palial_gpu_sm_count(void);
long long palial_gpu_kernel_launches(void);  /* kernels launched by this library so far */
const char *palial_gpu_error_string(int code);

/* ---- whole factorizations on HOST buffers (drop-in for src/{cholesky,lu,qr}.h) ------------
 * Replace reference src/cholesky.h:12 `void cholesky(MATRIX_desc A)`,
 *         reference src/lu.h:11       `void lu(MATRIX_desc A)`,
 *         reference src/qr.h:15       `void qr(MATRIX_desc A, MATRIX_desc S)`.
 * In place on A->matrix (and S->matrix), same output layout and meaning as the reference:
 *  Cholesky: U (A = U^T U) in the upper triangle of tiles A(k,m), k <= m; lower tiles
 *            untouched.
 *  LU:       no pivoting (reference src/srclu/dgetrf.h:11-59); L strictly lower (unit
 *            diagonal implicit), U upper.  ipiv (optional, N ints) receives the identity
 *            permutation ipiv[i] = i + 1, LAPACK style.
 *  QR:       flat-tree TS tile QR; R in the upper triangle, V in the strictly lower part of
 *            A(k,k) and in A(m,k), m > k; T factors in the upper triangles of S(k,k), S(m,k).
 */
int palial_gpu_cholesky(const palial_desc *A, const palial_opts *opts, palial_status *st);
int palial_gpu_lu(const palial_desc *A, int *ipiv, const palial_opts *opts, palial_status *st);
int palial_gpu_qr(const palial_desc *A, const palial_desc *S, const palial_opts *opts,
                  palial_status *st);

/* ---- same, on DEVICE-resident tile buffers (no host copies) ------------------------------ */
int palial_gpu_factor_dev(int alg, double *dA, double *dS, int n, int nb, const palial_opts *opts,
                          palial_status *st, void *stream);

/* ---- mixed precision + iterative refinement (no reference counterpart) ------
 * Solve A X = B for nrhs <= 16 right-hand sides (dB, dX: n x nrhs column-major, device),
 * A an FP64 tile-layout matrix on the device (not modified).  alg: PALIAL_ALG_CHOLESKY or
 * PALIAL_ALG_LU (no pivoting).  opts->precision selects the trailing-update precision
 * (PALIAL_PREC_BF16 / FP8 / BF16X3 on tcgen05 with FP32 accumulation, or FP64); diagonal
 * tiles are factored and panels solved in FP32, residuals r = b - A x and corrections in
 * FP64 storage.  With PALIAL_PREC_FP64 the factorization runs on the FP64 tile scheduler and
 * the refinement solves with the FP64 factors (one step to the target in practice).  Iterates until the normwise backward error max_j |r_j|/(|A| |x_j| + |b_j|) (inf-
 * norms) <= opts->ir_tol (default 1e-14 * n); GMRES-IR when plain refinement stagnates
 * (opts->gmres: -1 never, 0 automatic, 1 always).  NB must be a multiple of 256.
 * Returns PALIAL_ERR_NOT_CONVERGED (with the reached error in st) if the target is missed.
 * The refinement's full residuals are computed on the tensor cores from 48-bit digit
 * expansions of A and X (exact BF16 digit products, exact chunk sums, 64-bit integer
 * accumulation; palial_gpu_residual mode 3; opts->reserved[4] = 4 uses the compensated-FP32
 * residual of mode 1 instead), with errors below 1e-12 of the backward error's scale.  When the tolerance is below 1e-11 (or
 * opts->reserved[4] = 2) convergence is confirmed with an FP64 residual; opts->reserved[4] =
 * 1 computes every residual in FP64.  Once a correction d is small (2^-17 ||d|| <= tol/4 ||x||
 * per column) the next residual is r - A d with FP32 products (one HBM-bound pass over A);
 * their error bounds are summed and convergence requires backward error + bound <= tol (else
 * the residual is recomputed in full).  opts->reserved[4] = 3 computes every residual in
 * full instead.  The status message counts the update-form residuals.
 * With BF16x3 updates the row / column panels' block products also run as BF16x3 on the warp
 * tensor cores (opts->reserved[5] bit 3 keeps them in FP32 FMAs).
 * Opt-in stabilised LU (alg = PALIAL_ALG_LU, mixed precisions): opts->reserved[6] = 1 factors
 * the random-butterfly transform U^T A V (depth-2 recursive butterflies, Parker 1995) without
 * pivoting instead of A, refines against A (seed: opts->reserved[7], 0 = 1).  PALIAL_PREC_AUTO
 * runs a precision ladder: BF16x3 (at most 10 refinement steps and 36 GMRES iterations; a
 * Cholesky breakdown moves up at once), then TF32x3 (FP32-level factors; 20 steps, GMRES
 * restarts of 200 and 600 iterations in all), then the FP64 factorization;
 * status.precision_used reports the rung that produced the result (PALIAL_PREC_*, + 100 for the
 * butterfly transform). */
int palial_gpu_solve_ir(int alg, const double *dA, int n, int nb, const double *dB, double *dX,
                        int nrhs, const palial_opts *opts, palial_status *st, void *stream);
/* Same with host buffers: A in the reference's tile layout (descriptor), B and X n x nrhs
 * column-major in host memory; includes the host<->device copies.  Cholesky (N a multiple of
 * NB, NB a multiple of 32) reads only the upper triangle of A, as the factorization does: the
 * lower triangle is never copied, and the residuals use the symmetric matrix the upper
 * triangle defines (the device-buffer entry point reads all of A for its residuals). */
int palial_gpu_solve_ir_host(int alg, const palial_desc *A, const double *B, double *X, int nrhs,
                             const palial_opts *opts, palial_status *st);
/* R = B - A X (B may be NULL: R = A X) on device buffers, A an FP64 tile matrix, X, B, R
 * n x nrhs column-major (nrhs <= 16): mode 0 in FP64, mode 1 with the compensated FP32
 * arithmetic; mode 2 (B must be NULL) is the refinement's update form R <- R - A X with FP32
 * products (|error| <= 2^-17 |A| |X| per entry); mode 3 the digit residual on the tensor cores
 * (A and X as 48-bit integers in 8-bit BF16 digits, exact digit products and chunk sums, 64-bit
 * integer accumulation; the refinement's full residual). */
int palial_gpu_residual(const double *dA, int n, int nb, const double *dX, const double *dB, double *dR, int nrhs,
                        int mode, void *stream);
/* The low-precision factorization alone: dW (n*n floats, tile layout) receives the FP32
 * factors (Cholesky: U in the upper tiles; LU: L\U). */
int palial_gpu_mp_factor(int alg, const double *dA, float *dW, int n, int nb,
                         const palial_opts *opts, palial_status *st, void *stream);
/* One trailing update of step k on an FP32 tile matrix dW, as the mixed factorization does
 * it: pack the step's panel(s) from dW in the given precision (1 bf16, 2 fp8, 3 bf16x3) and
 * apply C -= A_op B_op^T with the tcgen05 kernel (Cholesky: upper tile pairs; LU: all). */
int palial_gpu_mp_update_step(int alg, int precision, float *dW, int n, int nb, int k);
/* Which tcgen05 update kernel the mixed path launches (no reference counterpart): 0 one
 * 128 x 256 output block per CTA (two CTAs per SM); 2 runs of consecutive blocks per CTA with
 * double-buffered TMEM accumulators and a 192 KB load ring (one CTA per SM); 1 (default) runs
 * for BF16x3 / TF32x3 (tensor-bound) and one block per CTA for BF16 / FP8 (bound by the FP32
 * C traffic).  Both give the same bits.
 * Returns the previous setting (PALIAL_ERR_ARG for an unknown kind). */
int palial_gpu_set_update_kernel(int kind);
/* The mixed path's FP32 working copy: W = float(A) rounded to nearest even (tile layout, n x n,
 * tile nb), the upper tiles only when upper_only (the conversion of a solve; no reference
 * counterpart).  Device buffers, synchronous. */
int palial_gpu_f64_to_f32(const double *dA, float *dW, int n, int nb, int upper_only);
/* Which kernel factors the mixed path's 256 x 256 Cholesky blocks (the halves of a 512 diagonal
 * tile, or 256 tiles): 1 (default) keeps the block's upper triangle in shared memory for the
 * whole factorization, 0 stages 64-column pieces from global memory.  Same bits.  Returns the
 * previous setting (PALIAL_ERR_ARG for an unknown kind). */
int palial_gpu_set_diag_kernel(int kind);
/* SMs (0..64) the mixed factorization's rest-of-trailing-update launches leave free for the
 * critical chain's kernels on the high-priority stream (the tile-run kernel then launches at
 * most SMs - sms CTAs with longer runs), in the steps whose trailing matrix has fewer than
 * below_rows tile rows (0: every step).  Default 24 SMs in every step.  Same bits for every
 * setting.  Returns the previous number of SMs (PALIAL_ERR_ARG for sms outside 0..64 or
 * below_rows < 0). */
int palial_gpu_set_update_reserve(int sms, int below_rows);

/* ---- linear solve and least squares through the tile QR (no reference counterpart) -------
 * A: rows x cols FP64 tile matrix on the device (rows >= cols, both multiples of nb, nb a
 * multiple of 64; tile (m,n) at element nb*nb*(m + (rows/nb)*n)), not modified.
 * B: rows x nrhs column-major (ld = rows), 1 <= nrhs <= nb.  X: cols x nrhs column-major
 * (ld = cols) receives the solution of A X = B (square) or the least-squares solution
 * min ||A X - B||_2 (tall).  resid (optional, nrhs doubles) receives ||A x_j - b_j||_2 for
 * the tall case (0 for square).  One persistent launch runs the flat-tree tile QR of [A | B]
 * (Q^T applied to B by the same UNMQR/TSMQR tasks as the reference's src/qr.h:57-188 applies
 * to the trailing tiles) followed by the blocked back-substitution with R. */
int palial_gpu_qr_solve(int rows, int cols, int nb, const double *dA, const double *dB, double *dX, int nrhs,
                        double *dResid, const palial_opts *opts, palial_status *st, void *stream);
/* Mixed-precision QR solve of a square system A X = B (n x n, nrhs <= 16; device buffers, A
 * not modified): the flat-tree TS QR of the reference (the same GEQRT/TSQRT/UNMQR/TSMQR task
 * DAG and R/V/T layout) computed in FP32 by the FP32 task scheduler, then FP64 refinement
 * X += |R| R_f^-1 Q_f^T (R / |R|) with R = B - A X in FP64, until every column's normwise
 * backward error |r_j|/(|A||x_j| + |b_j|) <= opts->ir_tol (0: 1e-14 * n).  NB: a multiple of
 * 64 up to 512.  opts->precision = PALIAL_PREC_BF16X3 runs TSMQR's two products with V on the
 * warp tensor cores (BF16x3 split operands, FP32 accumulation) instead of FP32 FMAs.  A refinement
 * that does not halve the error per step (or exceeds
 * opts->ir_max_iter, 0 = 30) hands the system to palial_gpu_qr_solve (FP64).  status:
 * ir_iters, backward_error, factor_seconds, precision_used = the precision that produced the
 * result (PALIAL_PREC_FP32, PALIAL_PREC_BF16X3 for the tensor-core form, or PALIAL_PREC_FP64). */
int palial_gpu_qr_solve_ir(int n, int nb, const double *dA, const double *dB, double *dX, int nrhs,
                           const palial_opts *opts, palial_status *st, void *stream);
/* Same with host buffers (A in tile layout, B and X column-major, resid optional). */
int palial_gpu_qr_solve_host(int rows, int cols, int nb, const double *A, const double *B, double *X, int nrhs,
                             double *resid, const palial_opts *opts, palial_status *st);

/* ---- layout bridges, any N, tiled-matrix files (no reference counterpart) ------------------
 * The reference requires N % NB == 0 and the tile layout (palial_src/main.c:101-105,
 * include/tile_address.h:9-17).  These convert LAPACK column-major matrices (device) to and
 * from the tile layout, padding to npad = the next multiple of nb: the padding is zero except
 * its diagonal (pad_diag; 1 for LU, the matrix' diagonal scale for Cholesky), so the leading
 * n x n block of the padded matrix' factors is the factor of the original. */
int palial_gpu_padded_size(int n, int nb);
int palial_gpu_colmajor_to_tiles(const double *dC, long long ldc, int n, double *dT, int npad, int nb,
                                 double pad_diag, void *stream);
int palial_gpu_tiles_to_colmajor(const double *dT, int npad, int nb, double *dC, long long ldc, int n, void *stream);
/* A X = B for a column-major A of any n (device buffers, lda/ldb/ldx leading dimensions):
 * padded internally, solved by palial_gpu_solve_ir (opts as there), X = the first n rows. */
int palial_gpu_solve_colmajor(int alg, int n, const double *dA, long long lda, const double *dB, long long ldb,
                              double *dX, long long ldx, int nrhs, int nb, const palial_opts *opts, palial_status *st,
                              void *stream);
/* Tiled-matrix file (host): 8-byte magic "PALTILE1", int64 n, int64 nb, int64 flags (0), then
 * the n*n doubles of the tile layout in memory order, little-endian.  palial_tiles_read fills
 * n and nb and, when dst is not NULL, reads the n*n doubles into it. */
int palial_tiles_write(const char *path, const palial_desc *A);
int palial_tiles_read(const char *path, int *n_out, int *nb_out, double *dst);

/* ---- single-tile kernels on device pointers (reference tile-kernel ABI, for unit tests) ----
 * Each runs one tile task on one CTA of the persistent scheduler's kernels.
 * Replace reference src/srclu/dgetrf.h:11 PALIAL_dgetrf, src/srcqr/dgeqrt.h:9 PALIAL_dgeqrt,
 * src/srcqr/dormqr.h:9 PALIAL_dormqr, src/srcqr/dtsqrt.h:11 PALIAL_dtsqrt,
 * src/srcqr/dtsmqr.h:11 PALIAL_dtsmqr, and the LAPACKE/CBLAS tile calls of src/cholesky.h:40,
 * :73, :115, :156 and src/lu.h:67, :109, :151.  lda = ld of every tile argument.      */
int palial_gpu_tile_dpotrf(int nb, double *dA, int lda);
int palial_gpu_tile_dgetrf(int nb, double *dA, int lda);
int palial_gpu_tile_dtrsm(int kind, int nb, const double *dT, double *dB, int lda);
int palial_gpu_tile_dsyrk(int nb, const double *dA, double *dC, int lda);
int palial_gpu_tile_dgemm(int kind, int nb, const double *dA, const double *dB, double *dC, int lda);
int palial_gpu_tile_dgeqrt(int nb, double *dA, double *dT, int lda);
int palial_gpu_tile_dormqr(int nb, const double *dV, const double *dT, double *dC, int lda);
int palial_gpu_tile_dtsqrt(int nb, double *dA1, double *dA2, double *dT, int lda);
int palial_gpu_tile_dtsmqr(int nb, double *dA1, double *dA2, const double *dV, const double *dT,
                           int lda);
/* The FP32 forms of the four QR tile kernels (the mixed-precision QR's routines), same
 * arguments on FP32 device tiles; nb a multiple of 64 up to 512. */
int palial_gpu_tile_sgeqrt(int nb, float *dA, float *dT, int lda);
int palial_gpu_tile_sormqr(int nb, const float *dV, const float *dT, float *dC, int lda);
int palial_gpu_tile_stsqrt(int nb, float *dA1, float *dA2, float *dT, int lda);
int palial_gpu_tile_stsmqr(int nb, float *dA1, float *dA2, const float *dV, const float *dT, int lda);
/* TSMQR without any device allocation.  No counterpart in the reference: it exists for
 * callers that may not allocate device memory themselves -- code inside an application that
 * owns all device memory (its own pool or allocator, a fixed budget), or latency-critical
 * code that must avoid cudaMalloc/cudaFree and the device-wide synchronization they can
 * cause.  Same arguments and result as palial_gpu_tile_dtsmqr, plus a stream (a
 * cudaStream_t as void*, NULL = default stream); the call only enqueues the kernel.
 * Limit: nb <= 512 (a multiple of 64); larger tiles return PALIAL_ERR_ARG.  Its scratch is a
 * fixed 512 KiB array inside the library, held by every GPU that loads it until the process
 * exits.  The first call on a device looks up that array's device address (thread-safe), so
 * make that first call before capturing a stream.  The address belongs to the device's context
 * at that call: after cudaDeviceReset, call palial_gpu_finalize() before calling this again (it
 * makes the next call look the address up anew).  All calls share the one array: calls whose
 * kernels overlap on the GPU (unordered streams, other host threads) race on it. */
int palial_gpu_tile_dtsmqr_noalloc(int nb, double *dA1, double *dA2, const double *dV,
                                   const double *dT, int lda, void *stream);
/* kind for dtrsm: 0 = left upper trans non-unit (Cholesky), 1 = right upper no-trans non-unit
 * (LU), 2 = left lower no-trans unit (LU), 3 = left upper no-trans non-unit (QR solve).  kind for dgemm: 0 = C -= A^T B (Cholesky),
 * 1 = C -= A B (LU). */

/* ---- batched factorizations (no reference counterpart) ------------------------
 * Factor `count` independent matrices (alg 0 Cholesky / 1 LU per matrix) in ONE persistent
 * launch: the DAGs of all matrices are merged into one dispatch list ordered by critical path.
 * Matrix i: device tile-layout buffer dA[i] of size ns[i] (multiple of nbs[i]), scheduled in
 * blocks of bss[i] (multiple of 64, divides nbs[i]).  Matrices whose true size is not a multiple
 * of 64 are embedded with identity (LU) or n*I (Cholesky) padding, which keeps the leading
 * factor exact (palial_gpu_gen_batch_matrix makes such inputs).  completion_s (optional, count
 * doubles) receives each matrix's completion time from the start of the launch (device trace).
 * opts->reserved[2] = 1 replays the launch from a CUDA graph (captured on first use for the
 * same DAG and matrix table). */
int palial_gpu_batched(int count, const int *algs, const int *ns, const int *nbs, const int *bss,
                       double *const *dA, const palial_opts *opts, palial_status *st,
                       double *completion_s, void *stream);
int palial_gpu_gen_batch_matrix(double *dA, int kind, int n_true, int n_pad, int nb, uint64_t seed,
                                void *stream);
/* The same batched launch with FP32 tasks on FP32 tile-layout buffers (16-byte aligned): the
 * FP32 factorizations of the batched mixed-precision solves.  A non-positive Cholesky pivot
 * or an exact zero LU pivot does not stop the launch: breakdown[i] (optional, count ints)
 * receives 0, or nonzero for matrix i (Cholesky: 1 + the first failing column). */
int palial_gpu_batched_f32(int count, const int *algs, const int *ns, const int *nbs, const int *bss,
                           float *const *dA, int *breakdown, const palial_opts *opts, palial_status *st,
                           double *completion_s, void *stream);

/* ---- batched solves (no reference counterpart) ------------------------------------------
 * A_i x_i = b_i for `count` independent matrices to FP64-level normwise backward error
 * |r|/(|A||x| + |b|) <= opts->ir_tol (0: 1e-14 * n_i), infinity norms.  Matrix i: device
 * tile-layout buffer dA[i] holding the full matrix (both triangles, also for Cholesky: the
 * residuals read all of it; n = ns[i] <= 4096, tile nbs[i] = scheduler block, a multiple of 64
 * dividing n; 16-byte aligned; not modified), right-hand side dB[i] and solution dX[i] (n
 * doubles each).  precs[i] (NULL: all FP32): PALIAL_PREC_FP32 = the matrix is rounded to FP32
 * and factored with the other FP32 matrices in ONE persistent launch, then refined with FP64
 * residuals; PALIAL_PREC_BF16X3 = the same FP32 storage and launch with the update tasks'
 * products (SYRK, GEMM) on the warp tensor cores as BF16x3 (split operands, three products, FP32
 * accumulation; the "BF16-update" form); PALIAL_PREC_FP64 = factored in FP64 (one launch for
 * those).  An FP32 or BF16x3 matrix whose
 * factorization breaks down or whose refinement stalls (less than 2x per step, at most
 * opts->ir_max_iter steps, 0 = 30) is refactored in FP64 and refined again.  iters[i]
 * (optional): refinement steps, or -(steps + 1) for a matrix that fell back to FP64; berr[i]
 * (optional): its final backward error.  st: seconds = wall time of the call, factor_seconds =
 * the factorization launches, backward_error = the worst, ir_iters = the most steps,
 * fallbacks = the number of FP64 fallbacks.  Returns PALIAL_ERR_NOT_CONVERGED if a matrix stays
 * above its tolerance; an FP64 Cholesky breakdown fails the call (PALIAL_ERR_NOT_SPD). */
int palial_gpu_batched_solve(int count, const int *algs, const int *ns, const int *nbs,
                             const double *const *dA, const double *const *dB, double *const *dX,
                             const int *precs, const palial_opts *opts, palial_status *st, int *iters,
                             double *berr, void *stream);

/* ---- the synthetic uneven batch, its autotuner and its rank partition -----------------------
 * Batch of `count` matrices: N_i = floor(32 * 64^u_i), u_i uniform in [0,1) (splitmix64 of
 * seed, stream 6, index i), capped at 2047; alg_i = i % 2 (0 Cholesky on B B^T + N I, 1 LU on
 * uniform [-1,1)).  Size classes [32,64) [64,128) [128,256) [256,512) [512,1024) [1024,2048). */
typedef struct palial_batch_report {
    int count;                /* matrices run by this rank                                   */
    int bs_of_class[6];       /* block size used per size class                              */
    int count_of_class[6];
    double seconds;           /* median device time of one batched launch                   */
    double matrices_per_s;
    double tflops;            /* algorithmic flops / seconds                                 */
    double p50_ms[6], p99_ms[6]; /* completion time from the launch, per size class        */
    double autotune_seconds;
    double autotune_s[18];    /* autotuner times [class][candidate 64,128,256], -1 = not run */
} palial_batch_report;
/* Host only: the sizes and algorithms of the synthetic batch. */
int palial_gpu_batch_sizes(int count, uint64_t seed, int *ns, int *algs);
/* Host only: size-balanced partition over `world` ranks (longest-processing-time first on the
 * flop counts, deterministic): rank_of[i] = the rank that factors matrix i.  No collective is
 * needed: every rank computes the same partition and factors its own matrices. */
int palial_gpu_batch_partition(int count, const int *ns, const int *algs, int world, int *rank_of);
/* Per size class, time the class's matrices alone with each candidate block size (64, 128,
 * 256 where it fits the class) in a batched launch and keep the fastest. */
int palial_gpu_batch_autotune(int count, const int *ns, const int *algs, uint64_t seed, int reps, int *bs_of_class,
                              double *timings, palial_status *st);
/* Generate this rank's share of the synthetic batch on the device, optionally autotune the
 * block size per class (else bs_of_class, NULL = 64 below N = 512 and 128 above), run one
 * warm-up and `reps` timed batched launches (CUDA graph replay), and fill the report. */
int palial_gpu_batch_synthetic(int count, uint64_t seed, int rank, int world, int autotune, const int *bs_of_class,
                               int reps, const palial_opts *opts, palial_status *st, palial_batch_report *rep);

/* Batched solves of the synthetic batch (right-hand sides uniform [-1,1)), block size and
 * factorization precision per (algorithm, size class), index alg * 6 + class. */
typedef struct palial_batch_solve_report {
    int count;                /* matrices solved by this rank                                */
    int bs_of_class[12];      /* block (= tile) size per [alg * 6 + size class]              */
    int prec_of_class[12];    /* 1 = FP32 factorization + FP64 refinement, 2 = the same with its
                                 updates as BF16x3 products on the tensor cores, 0 = FP64     */
    int fallbacks;            /* most matrices refactored in FP64 in one timed solve         */
    int butterflies;          /* most LU matrices solved on their butterfly transform         */
    int max_iters;            /* most refinement steps of one matrix                         */
    int not_converged;        /* 1 if a timed solve left a matrix above its tolerance        */
    double seconds;           /* median wall time of one batched solve (every phase)         */
    double matrices_per_s;
    double tflops;            /* factorization flops (N^3/3, 2N^3/3) / seconds               */
    double max_backward_error;
    double autotune_seconds;
    double autotune_s[108];   /* [alg*6 + class][precision 0,1,2][block 64,128,256] seconds;
                                 -1 = not run, -2 = did not reach the tolerance              */
    double phase_seconds[3];  /* median run: copies + first factorizations, refinement,
                                 FP64 fallback (copies, factorization, refinement)           */
} palial_batch_solve_report;
/* Per (algorithm, size class), time the class's matrices alone with every block size (64,
 * 128, 256 where it fits) and both precisions, and keep the fastest choice that reaches the
 * tolerance on every matrix. */
int palial_gpu_batch_solve_autotune(int count, const int *ns, const int *algs, uint64_t seed, int reps, int *bs12,
                                    int *prec12, double *timings, palial_status *st);
/* Generate this rank's share of the synthetic batch with right-hand sides, optionally autotune
 * (else bs12 / prec12, NULL = block 64 below N = 512 and 128 above / FP32 everywhere), run one
 * warm-up and `reps` timed batched solves, and fill the report. */
int palial_gpu_batch_solve_synthetic(int count, uint64_t seed, int rank, int world, int autotune, const int *bs12,
                                     const int *prec12, int reps, const palial_opts *opts, palial_status *st,
                                     palial_batch_solve_report *rep);

/* ---- generators (counter-based; the same bytes as the CPU oracle's generators) ------------ */
/* uniform [-1,1): entry (i,j) from splitmix64 of seed/stream and i + j*rows.  Tile layout. */
int palial_gpu_gen_uniform(double *dA, int n, int nb, uint64_t seed, void *stream);
/* Dense column-major rows x cols block uniform [-1,1) (right-hand sides): entry (i,j) from
 * splitmix64 of seed / stream_id (2 = right-hand sides) and index i + j*rows. */
int palial_gpu_gen_dense(double *dX, long long rows, int cols, uint64_t seed, int stream_id, void *stream);
/* A = B B^T + n I, B = K/128, K integer in [-128,127] (exact integer arithmetic). */
int palial_gpu_gen_spd(double *dA, int n, int nb, uint64_t seed, void *stream);

/* The reference generator's pattern (reference include/populate.h:36-67) made reproducible:
 * 0.5 everywhere, diagonal 173*u + 173 in [173, 346) with u = (x_i + 1)/2 and x_i the
 * uniform [-1,1) number of index i (seed, stream 0).  SPD and diagonally dominant. */
int palial_gpu_gen_refpattern(double *dA, int n, int nb, uint64_t seed, void *stream);
/* Generate into a HOST tile buffer (generated on the device, then copied):
 * kind 0 = uniform, 1 = SPD B B^T + n I, 2 = reference pattern. */
int palial_gpu_generate(int kind, uint64_t seed, const palial_desc *A);

/* A = U diag(s) V^T with s_i = kappa^(-i/(n-1)) and U, V products of 64 Householder
 * reflectors with random unit vectors (seeded; V = U when symmetric, then A is made exactly
 * symmetric).  Tile layout, FP64, on the device.  Condition number kappa by construction. */
int palial_gpu_gen_kappa(double *dA, int n, int nb, double kappa, int symmetric, uint64_t seed,
                         void *stream);

/* ---- checks on device buffers --------------------------------------------------------------- */
/* Normwise relative residual of the factorization against the original matrix dA0 using
 * `nprobe` random probe vectors: ||A0 X - F(X)||_F / (||A0||_F ||X||_F), F = U^T U X, L U X or
 * Q R X.  Exact for nprobe >= n (identity columns are not used; a probe estimates). */
int palial_gpu_residual_probe(int alg, const double *dA0, const double *dF, const double *dS, int n,
                              int nb, int nprobe, uint64_t seed, double *out);

/* Same from HOST tile buffers (original matrix a0_host, factors in F). */
int palial_gpu_residual_host(int alg, const double *a0_host, const palial_desc *F, int nprobe,
                             uint64_t seed, double *out);

/* ---- device trace (reference palial_trace/log.h:43-50 format) ------------------------------- */
/* Writes one "name, ms" line per task of the last traced factorization, in creation order,
 * with the reference's naming rule (type + k + m + n, stale loop variables,
 * src/cholesky.h:19-28).  path NULL = stdout.  A side-car CSV with
 * start/end ns, SM id and dispatch index is written to `csv_path` if not NULL. */
int palial_gpu_trace_dump(const char *path, const char *csv_path);
long long palial_gpu_trace_count(void);
/* Replay the last trace into the reference's trace hooks (reference include/common.h:9-11):
 * set_name(name) for every task in creation order, then per task in start order
 * cpu_node(SM id, device ordinal, name) and task_time(start_us, end_us, name), wall-clock
 * microseconds since the epoch.  NULL hooks are skipped.  palial_entry.h calls this with the
 * weak palial_set_task_name / palial_set_task_cpu_node / palial_get_task_time. */
int palial_gpu_trace_hooks(void (*set_name)(const char *), void (*cpu_node)(int, int, char *),
                           void (*task_time)(long long, long long, char *));
/* Host only: the task names of a DAG in creation order, newline separated (the same names the
 * trace prints).  Returns the bytes needed including the terminating zero, -1 on bad sizes. */
long long palial_dag_names(int alg, int n, int nb, int block, char *buf, long long buflen);

/* ---- GPU clock reporting (replaces the reference's palial_power CPU frequency control) ----- */
typedef struct palial_clock_report {
    double sm_mhz_start, sm_mhz_end, sm_mhz_max; /* via NVML when available, else -1     */
    double sm_mhz_device;                         /* clock64 / globaltimer during the run */
    int throttle_reasons;                         /* NVML bit mask, -1 if unavailable     */
} palial_clock_report;
/* Clocks around the last traced factorization (NVML samples just before and during the
 * launch, device clock64/globaltimer ratio of its tasks); without a traced run, the current
 * NVML values.  NVML is loaded at run time and only queried, never used to set anything. */
int palial_gpu_clock_report(palial_clock_report *out);
/* The current SM clock, its maximum (MHz) and the NVML clock-event reason mask (bit 0x4
 * software power cap, 0x8 hardware slowdown, 0x20 software thermal, 0x40 hardware thermal).
 * PALIAL_ERR_NO_DEVICE (values -1) when NVML is not available. */
int palial_gpu_clock_sample(double *sm_mhz, double *sm_max_mhz, long long *reasons);

/* ---- DAG builder (host only; exported for tests) -------------------------------------------- */
/* Build the task list the scheduler would run; returns the number of tasks, fills counts per
 * task type (array of 16) and the critical-path length estimate (seconds, model costs). */
long long palial_dag_info(int alg, int n, int nb, int block, int priority, int nworkers,
                          long long *type_counts, double *critical_path_s, double *makespan_s);
/* Host only: build, order and validate the QR solve DAG (rows x cols, nrhs right-hand
 * sides); returns its number of task records, or -1 with the reason in msg.  type_counts
 * (optional, 16 entries) receives the logical task count per type. */
long long palial_dag_qr_solve_validate(int rows, int cols, int nb, int nrhs, int nworkers, unsigned int seed,
                                       long long *type_counts, char *msg, int msglen);
/* The same for the apply-only QR solve DAG of the mixed-precision QR refinement (square n x n:
 * Q^T on the extra tile column and the back-substitution, the factors already in place). */
long long palial_dag_qr_apply_validate(int n, int nb, int nrhs, int nworkers, unsigned int seed,
                                       long long *type_counts, char *msg, int msglen);
/* Validate a built DAG on the host: every wait is satisfiable by earlier tasks in dispatch
 * order, updates to each object are totally ordered, no read/write race; then emulate the
 * dispatch with `nworkers` workers and random durations (seed).  Returns 0 if valid. */
int palial_dag_validate(int alg, int n, int nb, int block, int priority, int nworkers,
                        unsigned int seed, char *msg, int msglen);

/* ---- learned task-cost model (no reference counterpart) ------------------------
 * An MLP (nin -> hidden -> hidden -> 1, ReLU, FP32) trained on the device by this library's
 * own forward / backward / Adam kernels.  Inputs are task features (palial_dag_features_count()
 * floats per task); the target is log(task time in microseconds). */
int palial_mlp_init(int nin, int hidden, uint64_t seed);
long long palial_mlp_param_count(void);
int palial_mlp_get_params(float *out);
int palial_mlp_set_params(const float *in);
int palial_mlp_grad(const float *X, const float *y, int n, float *grads_out, float *loss_out);
int palial_mlp_train(const float *X, const float *y, int n, int epochs, int batch, float lr, uint64_t seed,
                     float *final_loss);
int palial_mlp_predict(const float *X, int n, float *out);
int palial_dag_features_count(void);
/* Training data from the last traced factorization: features and log(us) per task record. */
long long palial_gpu_trace_features(float *X, float *y, long long cap);
/* Planning: features of every logical task of the DAG (alg, n, nb, block). */
long long palial_dag_logical_features(int alg, int n, int nb, int block, int nworkers, float *X, long long cap);
/* Register per-logical-task costs (seconds) for a DAG shape; opts.priority = 2 (and
 * palial_dag_info with priority 2) then orders by the critical path of these costs.
 * cost_s = NULL removes them. */
int palial_gpu_set_task_costs(int alg, int n, int nb, int block, const double *cost_s, long long count);

/* Same validation for a merged batch DAG (and that no record crosses matrices). */
int palial_dag_batch_validate(int count, const int *algs, const int *ns, const int *nbs, const int *bss,
                              int nworkers, unsigned int seed, char *msg, int msglen);

/* ---- introspection of host-side schedules (host only, no GPU needed) ---------------------
 * palial_gpu_row_groups: the tile-row groups in which palial_gpu_solve_ir_host sends the upper
 * triangle of a mixed-precision Cholesky (gs/ge: rows [gs, ge); due: step by which the group's
 * data is expected; kg: step by which it joins the trailing updates); arrays of at least 64;
 * returns the number of groups or a negative error.
 * palial_gpu_check_solve_tasks: 0 when the refinement's triangular-solve task list for mt tile
 * rows, nbl 64-row blocks per tile and direction kind (0 U^T, 1 U, 2 unit L) is deadlock-free
 * under in-order dispatch and its counters are consistent; else 1 + the first bad record. */
int palial_gpu_row_groups(int n, int nb, int *gs, int *ge, int *due, int *kg, int max_groups);
/* 0 when the host-buffer Cholesky's catch-up plan for those groups (update mode 0 BF16, 1 FP8,
 * 2 BF16x3) waits for each group's data first, applies its skipped steps in order exactly once,
 * joins it in time and covers the rows each next step needs; else a positive code. */
int palial_gpu_check_arrival_plan(int n, int nb, int mode);
int palial_gpu_check_solve_tasks(int mt, int nbl, int kind);

#ifdef __cplusplus
}
#endif
#endif /* PALIAL_GPU_H */
