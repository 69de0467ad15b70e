/*
 * palial_entry.h -- drop-in replacements for the reference's per-algorithm entry points.
 *
 *   void cholesky(MATRIX_desc A)            replaces reference src/cholesky.h:12
 *   void lu(MATRIX_desc A)                  replaces reference src/lu.h:11
 *   void qr(MATRIX_desc A, MATRIX_desc S)   replaces reference src/qr.h:15
 *
 * Like the reference, these are defined in a header that exactly one translation unit
 * includes, take the descriptor by value and factor A.matrix (and S.matrix) in place, in the
 * reference's tile layout.  Unlike the reference they are synchronous (results are valid on
 * return), need no OpenMP region and no OMP_NUM_THREADS, and run on the GPU through
 * libpalial_gpu.so.  The reference returns nothing and ignores numerical failures; these keep
 * the void signature but report failures on stderr.  `palial_entry_opts` (precision, block
 * size, trace, ...) and `palial_entry_status` (time, TFLOP/s, error details) can be set/read
 * by the caller around the calls.
 *
 * Trace hooks: the reference's tasks call the weak hooks palial_set_task_name,
 * palial_set_task_cpu_node and palial_get_task_time (reference include/common.h:9-11) that a
 * tracing library may define.  When palial_entry_opts.trace is set, the wrappers replay the
 * device trace of the call into whichever of those hooks are linked: every name in creation
 * order, then per task the SM id as `cpu`, the GPU ordinal as `node`, and the task's start and
 * end wall times.
 *
 * MATRIX_desc must be defined before inclusion: by the reference's include/descriptor.h or
 * by palial_descriptor.h (identical layout).
 */
#ifndef PALIAL_ENTRY_H
#define PALIAL_ENTRY_H

#include <stdio.h>
#include <sys/time.h>

#include "palial_gpu.h"

palial_opts palial_entry_opts;
palial_status palial_entry_status;

void __attribute__((weak)) palial_set_task_name(const char *name);
void __attribute__((weak)) palial_set_task_cpu_node(int cpu, int node, char *name);
void __attribute__((weak)) palial_get_task_time(struct timeval start, struct timeval end, char *name);

static void palial_entry_task_time(long long start_us, long long end_us, char *name)
{
    struct timeval a, b;
    a.tv_sec = (time_t)(start_us / 1000000);
    a.tv_usec = (suseconds_t)(start_us % 1000000);
    b.tv_sec = (time_t)(end_us / 1000000);
    b.tv_usec = (suseconds_t)(end_us % 1000000);
    palial_get_task_time(a, b, name);
}

static void palial_entry_hooks(int rc)
{
    if (rc < 0 || !palial_entry_opts.trace) return;
    if (!palial_set_task_name && !palial_set_task_cpu_node && !palial_get_task_time) return;
    palial_gpu_trace_hooks(palial_set_task_name ? palial_set_task_name : NULL,
                           palial_set_task_cpu_node ? palial_set_task_cpu_node : NULL,
                           palial_get_task_time ? palial_entry_task_time : NULL);
}

static void palial_entry_report(const char *what, int rc)
{
    palial_entry_hooks(rc);
    if (rc < 0)
        fprintf(stderr, "palial: %s failed: %s (%s)\n", what, palial_gpu_error_string(rc),
                palial_entry_status.message);
    else if (rc > 0)
        fprintf(stderr, "palial: %s: %s\n", what, palial_gpu_error_string(rc));
}

void cholesky(MATRIX_desc A)
{
    palial_entry_report("cholesky", palial_gpu_cholesky((const palial_desc *)&A, &palial_entry_opts,
                                                        &palial_entry_status));
}

void lu(MATRIX_desc A)
{
    palial_entry_report("lu", palial_gpu_lu((const palial_desc *)&A, NULL, &palial_entry_opts,
                                            &palial_entry_status));
}

void qr(MATRIX_desc A, MATRIX_desc S)
{
    palial_entry_report("qr", palial_gpu_qr((const palial_desc *)&A, (const palial_desc *)&S,
                                            &palial_entry_opts, &palial_entry_status));
}

#endif
