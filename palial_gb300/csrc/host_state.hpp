// host_state.hpp -- host-side state shared by the runtime translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdarg>
#include <map>
#include <string>
#include <memory>
#include <tuple>
#include <vector>

#include "../../include/palial_gpu.h"
#include "common.cuh"
#include "dag.hpp"

namespace palial {

// grow-only device buffer
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t want) {
        if (want <= bytes) return cudaSuccess;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&ptr, want);
        if (e == cudaSuccess) bytes = want;
        return e;
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    template <class T>
    T *as() const {
        return static_cast<T *>(ptr);
    }
};

// Device state of one persistent-scheduler instance (records, counters, status, ticket,
// trace, scratch).  The main factorizations use one; the mixed-precision driver uses a
// second one for its FP64 diagonal-tile factorizations.
struct SchedCtx {
    DevBuf tasks, counters, status, ticket, trace, scratch;
    unsigned long long uploaded = 0;  // uid of the DAG whose records are on the device
    void release() {
        for (DevBuf *b : {&tasks, &counters, &status, &ticket, &trace, &scratch}) b->release();
        uploaded = 0;
    }
};

// One lane of batched launches (FP64 or FP32 tasks): scheduler buffers, the device matrix
// table and the CUDA graph captured for the last (DAG, table, trace) combination.
struct BatchLane {
    SchedCtx ctx;
    DevBuf mats, flags;
    cudaGraphExec_t graph = nullptr;
    unsigned long long graph_uid = 0;
    const void *graph_mats = nullptr;
    const void *graph_trace = nullptr;
    void release() {
        ctx.release();
        mats.release();
        flags.release();
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
        graph_uid = 0;
        graph_mats = graph_trace = nullptr;
    }
};

struct TraceState {
    Dag dag;
    std::vector<TraceRec> recs;
    bool valid = false;
};

struct State {
    bool init = false;
    int device = -1;
    int sms = 0;
    int occupancy = 1;
    int occupancy32 = 1;     // resident CTAs per SM of the FP32 batched scheduler
    int occupancy32_qr = 1;  // of the FP32 scheduler's one-matrix QR instance
    SchedCtx main, diag;
    BatchLane lane64, lane32;  // batched launches with FP64 / FP32 tasks
    std::map<std::string, std::shared_ptr<Dag>> batch_dags;
    DevBuf mat, smat, kbuf, probe;
    std::map<std::tuple<int, int, int, int, int, int, unsigned>, std::shared_ptr<Dag>> dags;
    unsigned long long next_uid = 1;
    TraceState last_trace;
    int last_trace_workers = 0;
    long long last_trace_host_ns = 0;  // host CLOCK_REALTIME just before the traced launch
    // NVML clock samples around the last traced factorization (-1: not available)
    double clk_start = -1, clk_end = -1, clk_max = -1;
    long long clk_reasons = -1;
    // learned per-task costs (seconds, per logical task) keyed by "alg,n,nb,bs"
    std::map<std::string, std::vector<double>> task_costs;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};
extern State g;

// Free the QR solve's cached device buffers and DAG (palial_gpu_finalize).
void qr_solve_release();
// z = F^-1 v in FP64 for Cholesky / LU factors F in an n x (n + nb) tile matrix (qr_solve.cu).
int fp64_trsolve(int alg, double *W, int n, int nb, const double *v, double *z, int nrhs, cudaStream_t s,
                 palial_status *st);
// Free the layout bridges' padded buffers (palial_gpu_finalize).
void layout_release();
// Free the batched solves' workspaces (palial_gpu_finalize).
void batch_solve_release();
// Free the mixed-precision QR solve's buffers and DAGs (palial_gpu_finalize).
void mp_qr_release();
// palial_gpu_batched_solve with the wall time of its phases (phases[3], optional): copies and
// first factorizations, refinement, FP64 fallback (copies, factorization, refinement).
int batched_solve_run(int count, const int *algs, const int *ns, const int *nbs, const double *const *dA,
                      const double *const *dB, double *const *dX, const int *precs, const palial_opts *opts,
                      palial_status *st, int *iters, double *berr, double *phases, void *stream);
// Free the random butterflies (palial_gpu_finalize).
void rbt_release();

// Read-only NVML query of the library's device (false and -1 values without NVML).
bool nvml_sample(double *sm_mhz, double *sm_max_mhz, long long *reasons);

int set_status(palial_status *st, int code, const char *fmt = nullptr, ...);
int cuda_fail(palial_status *st, cudaError_t e, const char *what);
int ensure_init(palial_status *st);
int auto_block(int alg, int n, int nb);
std::shared_ptr<Dag> get_dag(int alg, int n, int nb, int bs, int priority, int workers, unsigned seed);

// Prepare a scheduler run (host: DAG upload, buffers) and return its launch parameters.
int sched_prepare(SchedCtx &c, const std::shared_ptr<Dag> &dag, double *dA, double *dS, int workers, int trace,
                  double timeout_s, SchedParams &p, palial_status *st);
// Enqueue it (asynchronous): clear counters and ticket (and status if clear_status), launch
// the FP64 scheduler (or the FP32 one of the batched mixed-precision solves when f32).
cudaError_t sched_enqueue(SchedCtx &c, const SchedParams &p, int nobj, int workers, bool clear_status, cudaStream_t s,
                          bool f32 = false);
// One batched persistent launch over `count` matrices, synchronous.  bufs[i]: the matrix's
// tile-layout buffer, double (FP64 tasks) or float (FP32 tasks: f32 = true).  FP32 runs
// report breakdowns per matrix in flags (count ints, host; 0 = none) instead of failing.
int batched_run(int count, const int *algs, const int *ns, const int *nbs, const int *bss, void *const *bufs, bool f32,
                int *flags, const palial_opts *opts, palial_status *st, double *completion_s, cudaStream_t s,
                const int *tcs = nullptr);  // tcs[i] = 1: FP32 updates of matrix i on the tensor cores

#define PALIAL_CK(call, what)                                  \
    do {                                                       \
        cudaError_t _e = (call);                               \
        if (_e != cudaSuccess) return cuda_fail(st, _e, what); \
    } while (0)

}  // namespace palial
