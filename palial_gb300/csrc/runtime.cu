// runtime.cu -- host side of libpalial_gpu.so: the C ABI of include/palial_gpu.h.
//
// Owns the device state (one device per process), caches DAGs and device buffers, launches
// the persistent scheduler and reports status.  No CPU fallback exists: every entry point
// fails with PALIAL_ERR_NO_DEVICE / PALIAL_ERR_CUDA when the GPU path cannot run.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/palial_gpu.h"
#include "common.cuh"
#include "dag.hpp"
#include "host_state.hpp"

namespace palial {
// sched_f64.cu
int sched_smem_bytes();
cudaError_t sched_configure();
int sched_occupancy();
cudaError_t sched_launch(const SchedParams &p, int grid, cudaStream_t s);
long long sched_scratch_doubles(int alg, int n, int nb, int bs, int workers, long long *per_worker);
cudaError_t tile_task_launch(int type, int nb, int ld, double *p0, double *p1, double *p2, double *p3, double *scratch,
                             int *status, cudaStream_t s);
// sched_f32.cu
cudaError_t sched32_configure();
int sched32_occupancy(bool qr);
cudaError_t sched32_launch(const SchedParams &p, int grid, cudaStream_t s);
cudaError_t tile_qr_f32_launch(int type, int nb, int ld, float *p0, float *p1, float *p2, float *p3, float *scratch,
                               cudaStream_t s);
// gen_check.cu
cudaError_t launch_gen_uniform(double *A, int n, int nb, uint64_t seed, cudaStream_t s);
cudaError_t launch_gen_refpattern(double *A, int n, int nb, uint64_t seed, cudaStream_t s);
cudaError_t launch_gen_dense(double *X, long long rows, int cols, uint64_t seed, int stream, cudaStream_t s);
cudaError_t launch_gen_spd(double *A, int n, int nb, uint64_t seed, int8_t *kbuf, cudaStream_t s);
cudaError_t launch_gen_batch(double *A, int kind, int nt, int np, int nb, uint64_t seed, int8_t *kbuf,
                             cudaStream_t s);
cudaError_t launch_tiled_mm(const double *A, const double *X, double *Y, int n, int nb, int r, int mode, int trans,
                            cudaStream_t s);
cudaError_t launch_sumsq(const double *X, long long len, double *partial, int blocks, cudaStream_t s);
cudaError_t launch_sub(const double *X, const double *Y, double *Z, long long len, cudaStream_t s);
cudaError_t mps_configure();
cudaError_t mpd_configure();
cudaError_t mpr_configure();
void mpr_release();
void mp_release();

State g;
static long long g_launches = 0;
void note_launch() { g_launches++; }

int set_status(palial_status *st, int code, const char *fmt, ...) {
    if (st) {
        st->code = code;
        if (fmt) {
            va_list ap;
            va_start(ap, fmt);
            vsnprintf(st->message, sizeof st->message, fmt, ap);
            va_end(ap);
        }
    }
    return code;
}

int cuda_fail(palial_status *st, cudaError_t e, const char *what) {
    if (st) st->cuda_error = (int)e;
    return set_status(st, PALIAL_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int ensure_init(palial_status *st) {
    if (g.init) {
        cudaSetDevice(g.device);
        return PALIAL_OK;
    }
    int rc = palial_gpu_init(0);
    if (rc != PALIAL_OK) return set_status(st, rc, "no CUDA device available");
    return PALIAL_OK;
}

int auto_block(int alg, int n, int nb) {
    if (alg == 2) return nb;
    // blocks of 256 keep the FP64 critical path short at the reference's NB = 512
    int bs = std::min(nb, 256);
    while (nb % bs) bs -= 64;
    (void)n;
    return std::max(64, bs);
}

static std::string cost_key(int alg, int n, int nb, int bs) {
    return std::to_string(alg) + "," + std::to_string(n) + "," + std::to_string(nb) + "," + std::to_string(bs);
}

// priority 2: critical-path order from the learned per-task costs registered with
// palial_gpu_set_task_costs (falls back to the flop model when none are registered).
static void apply_learned_costs(Dag &d) {
    auto it = g.task_costs.find(cost_key(d.alg, d.n, d.nb, d.bs));
    if (it == g.task_costs.end() || it->second.size() != d.logical.size()) return;
    for (size_t i = 0; i < d.logical.size(); i++) d.logical[i].cost = it->second[i];
    recompute_bottom_levels(d);
}

std::shared_ptr<Dag> get_dag(int alg, int n, int nb, int bs, int priority, int workers, unsigned seed) {
    auto key = std::make_tuple(alg, n, nb, bs, priority, workers, seed);
    auto it = g.dags.find(key);
    if (it != g.dags.end()) return it->second;
    auto d = std::make_shared<Dag>(build_dag(alg, n, nb, bs));
    if (priority == 2) apply_learned_costs(*d);
    order_dag(*d, priority == 2 ? 0 : priority, workers, seed);
    d->uid = g.next_uid++;
    if (g.dags.size() > 16) g.dags.clear();
    g.dags[key] = d;
    return d;
}

int sched_prepare(SchedCtx &c, const std::shared_ptr<Dag> &dag, double *dA, double *dS, int workers, int trace,
                  double timeout_s, SchedParams &p, palial_status *st) {
    const int ntasks = (int)dag->records.size();
    void *old_tasks = c.tasks.ptr;
    PALIAL_CK(c.tasks.ensure(sizeof(Task) * (size_t)std::max(1, ntasks)), "alloc tasks");
    if (c.tasks.ptr != old_tasks) c.uploaded = 0;  // reallocated: contents gone
    if (c.uploaded != dag->uid) {
        c.uploaded = 0;
        PALIAL_CK(cudaMemcpy(c.tasks.ptr, dag->records.data(), sizeof(Task) * ntasks, cudaMemcpyHostToDevice),
                  "upload tasks");
        c.uploaded = dag->uid;
    }
    // one spare counter past the objects: nothing ever signals it (used by the stall test)
    PALIAL_CK(c.counters.ensure(sizeof(unsigned) * (size_t)(dag->nobj + 1)), "alloc counters");
    PALIAL_CK(c.status.ensure(sizeof(int) * ST_NSLOTS + 64), "alloc status");
    PALIAL_CK(c.ticket.ensure(64), "alloc ticket");
    long long per_worker = 0;
    const long long scr = sched_scratch_doubles(dag->alg, dag->n, dag->nb, dag->bs, workers, &per_worker);
    PALIAL_CK(c.scratch.ensure(sizeof(double) * (size_t)std::max<long long>(1, scr)), "alloc scratch");
    if (trace) PALIAL_CK(c.trace.ensure(sizeof(TraceRec) * (size_t)ntasks), "alloc trace");
    p = SchedParams{};
    p.tasks = c.tasks.as<Task>();
    p.ntasks = ntasks;
    p.ticket = c.ticket.as<unsigned>();
    p.counters = c.counters.as<unsigned>();
    p.status = c.status.as<int>();
    p.trace = trace ? c.trace.as<TraceRec>() : nullptr;
    p.A = dA;
    p.S = dS;
    p.scratch = c.scratch.as<double>();
    p.scratch_per_worker = per_worker;
    p.n = dag->n;
    p.nb = dag->nb;
    p.bs = dag->bs;
    p.timeout_ns = (unsigned long long)((timeout_s > 0 ? timeout_s : 120.0) * 1e9);
    return PALIAL_OK;
}

cudaError_t sched_enqueue(SchedCtx &c, const SchedParams &p, int nobj, int workers, bool clear_status, cudaStream_t s,
                          bool f32) {
    cudaError_t e = cudaMemsetAsync(c.counters.ptr, 0, sizeof(unsigned) * (size_t)(nobj + 1), s);
    if (e == cudaSuccess && clear_status) e = cudaMemsetAsync(c.status.ptr, 0, sizeof(int) * ST_NSLOTS, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(c.ticket.ptr, 0, 64, s);
    if (e == cudaSuccess) e = f32 ? sched32_launch(p, workers, s) : sched_launch(p, workers, s);
    return e;
}

int batched_run(int count, const int *algs, const int *ns, const int *nbs, const int *bss, void *const *bufs, bool f32,
                int *flags, const palial_opts *opts, palial_status *st, double *completion_s, cudaStream_t s,
                const int *tcs) {
    palial_opts o;
    palial_opts_default(&o);
    if (opts) o = *opts;
    if (count <= 0 || !algs || !ns || !nbs || !bss || !bufs) return set_status(st, PALIAL_ERR_ARG, "empty batch");
    int rc = ensure_init(st);
    if (rc) return rc;
    std::vector<BatchSpec> specs(count);
    std::string key = std::to_string(o.priority) + ":";
    double flops = 0;
    for (int i = 0; i < count; i++) {
        const int a = algs[i], n = ns[i], nb = nbs[i], bs = bss[i];
        if ((a != 0 && a != 1) || n <= 0 || nb <= 0 || n % nb || nb % bs || bs % 64 || !bufs[i] ||
            (f32 && (reinterpret_cast<uintptr_t>(bufs[i]) & 15)))
            return set_status(st, PALIAL_ERR_ARG, "matrix %d: alg %d n %d nb %d bs %d", i, a, n, nb, bs);
        specs[i] = BatchSpec{a, n, nb, bs};
        key += std::to_string(a) + "," + std::to_string(n) + "," + std::to_string(nb) + "," + std::to_string(bs) + ";";
        flops += algorithmic_flops(a, n);
    }
    BatchLane &lane = f32 ? g.lane32 : g.lane64;
    const int workers = f32 ? g.sms * g.occupancy32 : g.sms;
    std::shared_ptr<Dag> dag;
    auto it = g.batch_dags.find(key);
    if (it != g.batch_dags.end()) {
        dag = it->second;
    } else {
        try {
            dag = std::make_shared<Dag>(build_batch_dag(specs));
            order_dag(*dag, o.priority, g.sms, 0);
        } catch (const std::exception &ex) {
            return set_status(st, PALIAL_ERR_ARG, "%s", ex.what());
        }
        dag->uid = g.next_uid++;
        if (g.batch_dags.size() > 8) g.batch_dags.clear();
        g.batch_dags[key] = dag;
    }
    std::vector<MatInfo> mats(count);
    for (int i = 0; i < count; i++) {
        mats[i] = MatInfo{};
        if (f32) mats[i].Af = static_cast<float *>(bufs[i]);
        else mats[i].A = static_cast<double *>(bufs[i]);
        mats[i].n = ns[i];
        mats[i].nb = nbs[i];
        mats[i].bs = bss[i];
        mats[i].tc = (f32 && tcs) ? tcs[i] : 0;
    }
    PALIAL_CK(lane.mats.ensure(sizeof(MatInfo) * count), "alloc matrix table");
    PALIAL_CK(cudaMemcpyAsync(lane.mats.ptr, mats.data(), sizeof(MatInfo) * count, cudaMemcpyHostToDevice, s), "upload");
    if (f32) {
        PALIAL_CK(lane.flags.ensure(sizeof(int) * (size_t)count), "alloc breakdown flags");
        PALIAL_CK(cudaMemsetAsync(lane.flags.ptr, 0, sizeof(int) * (size_t)count, s), "clear breakdown flags");
    }
    const bool want_trace = o.trace || completion_s;
    SchedParams p;
    rc = sched_prepare(lane.ctx, dag, nullptr, nullptr, workers, want_trace, o.timeout_s, p, st);
    if (rc) return rc;
    p.mats = lane.mats.as<MatInfo>();
    p.mat_status = f32 ? lane.flags.as<int>() : nullptr;
    const bool use_graph = o.reserved[2] == 1;
    PALIAL_CK(cudaEventRecord(g.ev0, s), "event");
    if (use_graph) {
        // one CUDA graph per (DAG, matrix table): counter/ticket/status clears + the launch
        const void *gkey = want_trace ? (const void *)lane.ctx.trace.ptr : nullptr;
        if (!lane.graph || lane.graph_uid != dag->uid || lane.graph_mats != lane.mats.ptr || lane.graph_trace != gkey) {
            if (lane.graph) cudaGraphExecDestroy(lane.graph);
            lane.graph = nullptr;
            cudaStream_t cs;
            PALIAL_CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "stream");
            cudaGraph_t graph;
            PALIAL_CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "capture");
            cudaError_t e = sched_enqueue(lane.ctx, p, dag->nobj, workers, true, cs, f32);
            cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
            cudaStreamDestroy(cs);
            PALIAL_CK(e, "capture enqueue");
            PALIAL_CK(e2, "end capture");
            PALIAL_CK(cudaGraphInstantiate(&lane.graph, graph, 0), "instantiate");
            cudaGraphDestroy(graph);
            lane.graph_uid = dag->uid;
            lane.graph_mats = lane.mats.ptr;
            lane.graph_trace = gkey;
        }
        PALIAL_CK(cudaGraphLaunch(lane.graph, s), "graph launch");
        note_launch();
    } else {
        PALIAL_CK(sched_enqueue(lane.ctx, p, dag->nobj, workers, true, s, f32), "launch");
    }
    PALIAL_CK(cudaEventRecord(g.ev1, s), "event");
    PALIAL_CK(cudaEventSynchronize(g.ev1), "batched run");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, g.ev0, g.ev1);
    int hs[ST_NSLOTS];
    PALIAL_CK(cudaMemcpy(hs, lane.ctx.status.ptr, sizeof hs, cudaMemcpyDeviceToHost), "status");
    if (f32 && flags)
        PALIAL_CK(cudaMemcpy(flags, lane.flags.ptr, sizeof(int) * (size_t)count, cudaMemcpyDeviceToHost), "flags");
    if (st) {
        st->seconds = ms * 1e-3;
        st->tflops = flops / std::max(1e-12, st->seconds) * 1e-12;
        st->ntasks = (long long)dag->records.size();
    }
    if (want_trace && hs[ST_CODE] == 0) {
        std::vector<TraceRec> recs(dag->records.size());
        PALIAL_CK(cudaMemcpy(recs.data(), lane.ctx.trace.ptr, sizeof(TraceRec) * recs.size(), cudaMemcpyDeviceToHost),
                  "trace");
        unsigned long long t0 = ~0ull;
        for (const auto &r : recs) t0 = std::min(t0, r.t0);
        if (completion_s) {
            for (int i = 0; i < count; i++) completion_s[i] = 0;
            for (size_t r = 0; r < recs.size(); r++) {
                const uint32_t m = dag->records[r].mat;
                completion_s[m] = std::max(completion_s[m], (double)(recs[r].t1 - t0) * 1e-9);
            }
        }
    }
    if (hs[ST_CODE] == PALIAL_ERR_NOT_SPD)
        return set_status(st, PALIAL_ERR_NOT_SPD, "non-positive pivot in a batched Cholesky");
    if (hs[ST_CODE] != 0) return set_status(st, hs[ST_CODE], "device error %d", hs[ST_CODE]);
    if (hs[ST_ZEROPIV]) return set_status(st, PALIAL_WARN_ZERO_PIVOT, "exact zero pivot skipped");
    return set_status(st, PALIAL_OK);
}
void noalloc_reset();  // noalloc.cu: forget the fixed scratch's per-device address
}  // namespace palial

using namespace palial;

#define CK(call, what) PALIAL_CK(call, what)

extern "C" {

void palial_opts_default(palial_opts *o) {
    if (!o) return;
    memset(o, 0, sizeof *o);
}

const char *palial_gpu_error_string(int code) {
    switch (code) {
        case PALIAL_OK: return "ok";
        case PALIAL_ERR_ARG: return "bad argument";
        case PALIAL_ERR_CUDA: return "CUDA error";
        case PALIAL_ERR_NOT_SPD: return "matrix is not positive definite";
        case PALIAL_ERR_TIMEOUT: return "device dependency wait timed out";
        case PALIAL_ERR_NO_DEVICE: return "no CUDA device";
        case PALIAL_ERR_NOT_CONVERGED: return "iterative refinement did not converge";
        case PALIAL_ERR_NOMEM: return "device allocation failed";
        case PALIAL_WARN_ZERO_PIVOT: return "exact zero pivot met and skipped";
        default: return "unknown";
    }
}

int palial_gpu_init(int device) {
    if (g.init && g.device == device) return PALIAL_OK;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= device || device < 0) {
        cudaGetLastError();
        return PALIAL_ERR_NO_DEVICE;
    }
    if (cudaSetDevice(device) != cudaSuccess) return PALIAL_ERR_NO_DEVICE;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return PALIAL_ERR_NO_DEVICE;
    g.device = device;
    g.sms = prop.multiProcessorCount;
    if (sched_configure() != cudaSuccess) return PALIAL_ERR_CUDA;
    if (mps_configure() != cudaSuccess) return PALIAL_ERR_CUDA;
    if (mpd_configure() != cudaSuccess) return PALIAL_ERR_CUDA;
    if (mpr_configure() != cudaSuccess) return PALIAL_ERR_CUDA;
    if (sched32_configure() != cudaSuccess) return PALIAL_ERR_CUDA;
    g.occupancy = std::max(1, sched_occupancy());
    g.occupancy32 = std::max(1, sched32_occupancy(false));
    g.occupancy32_qr = std::max(1, sched32_occupancy(true));
    if (!g.ev0) cudaEventCreate(&g.ev0);
    if (!g.ev1) cudaEventCreate(&g.ev1);
    g.init = true;
    return PALIAL_OK;
}

int palial_gpu_finalize(void) {
    noalloc_reset();
    if (!g.init) return PALIAL_OK;
    g.main.release();
    g.diag.release();
    g.lane64.release();
    g.lane32.release();
    g.batch_dags.clear();
    batch_solve_release();
    mp_qr_release();
    for (DevBuf *b : {&g.mat, &g.smat, &g.kbuf, &g.probe}) b->release();
    qr_solve_release();
    mpr_release();
    mp_release();
    layout_release();
    rbt_release();
    g.dags.clear();
    return PALIAL_OK;
}

int palial_gpu_sm_count(void) { return g.init ? g.sms : 0; }

long long palial_gpu_kernel_launches(void) { return palial::g_launches; }

int palial_gpu_factor_dev(int alg, double *dA, double *dS, int n, int nb, const palial_opts *opts,
                          palial_status *st, void *stream) {
    palial_opts o;
    palial_opts_default(&o);
    if (opts) o = *opts;
    if (st) {
        memset(st, 0, sizeof *st);
    }
    if (alg < 0 || alg > 2) return set_status(st, PALIAL_ERR_ARG, "unknown algorithm %d", alg);
    if (n <= 0 || nb <= 0 || n % nb) return set_status(st, PALIAL_ERR_ARG, "N %% NB != 0 (N=%d, NB=%d)", n, nb);
    if (nb % 64) return set_status(st, PALIAL_ERR_ARG, "NB must be a multiple of 64 (NB=%d)", nb);
    if (n / nb > 65535) return set_status(st, PALIAL_ERR_ARG, "too many tiles");
    if (!dA || (alg == 2 && !dS)) return set_status(st, PALIAL_ERR_ARG, "NULL matrix");
    int rc = ensure_init(st);
    if (rc) return rc;
    const int bs = o.block > 0 ? o.block : auto_block(alg, n, nb);
    if (alg != 2 && (bs % 64 || nb % bs)) return set_status(st, PALIAL_ERR_ARG, "block %d must divide NB and be a multiple of 64", bs);
    int sms = g.sms;
    if (o.max_sms > 0) sms = std::min(sms, o.max_sms);
    int wps = o.workers_per_sm > 0 ? std::min(o.workers_per_sm, g.occupancy) : 1;
    const int workers = sms * wps;
    std::shared_ptr<Dag> dag;
    try {
        dag = get_dag(alg, n, nb, bs, o.priority, workers, o.shuffle_seed);
    } catch (const std::exception &ex) {
        return set_status(st, PALIAL_ERR_ARG, "%s", ex.what());
    }
    const int ntasks = (int)dag->records.size();
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    SchedParams p;
    rc = sched_prepare(g.main, dag, dA, dS, workers, o.trace, o.timeout_s, p, st);
    if (rc) return rc;
    // Fault injection for tests (opts.reserved[0] = r + 1): record r additionally waits on the
    // spare counter, which nothing signals, so its wait must end by deadline with
    // PALIAL_ERR_TIMEOUT.  The uploaded copy is patched and restored afterwards.
    const int stall = o.reserved[0] - 1;
    Task saved{};
    if (stall >= 0 && stall < ntasks) {
        saved = dag->records[stall];
        Task t = saved;
        if (t.nwait < 3) {
            t.wait_obj[t.nwait] = (uint32_t)dag->nobj;
            t.wait_cnt[t.nwait] = 1;
            t.nwait++;
        } else {
            t.wait_obj[2] = (uint32_t)dag->nobj;
            t.wait_cnt[2] = 1;
        }
        CK(cudaMemcpy(g.main.tasks.as<Task>() + stall, &t, sizeof(Task), cudaMemcpyHostToDevice), "inject stall");
    }
    double clk0 = -1, clk_max = -1;
    long long reasons = -1;
    if (o.trace) {
        nvml_sample(&clk0, &clk_max, &reasons);
        timespec ts;
        clock_gettime(CLOCK_REALTIME, &ts);
        g.last_trace_host_ns = (long long)ts.tv_sec * 1000000000ll + ts.tv_nsec;
    }
    const auto w0 = std::chrono::steady_clock::now();
    CK(cudaEventRecord(g.ev0, s), "event");
    CK(sched_enqueue(g.main, p, dag->nobj, workers, true, s), "launch scheduler");
    CK(cudaEventRecord(g.ev1, s), "event");
    if (o.trace) {
        // sample while the scheduler runs (the launch is asynchronous)
        double c1, m1;
        nvml_sample(&c1, &m1, &reasons);
        g.clk_start = clk0;
        g.clk_end = c1;
        g.clk_max = m1;
        g.clk_reasons = reasons;
    }
    CK(cudaEventSynchronize(g.ev1), "scheduler run");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, g.ev0, g.ev1);
    int hs[ST_NSLOTS];
    CK(cudaMemcpy(hs, g.main.status.ptr, sizeof hs, cudaMemcpyDeviceToHost), "read status");
    unsigned tick = 0;
    CK(cudaMemcpy(&tick, g.main.ticket.ptr, sizeof tick, cudaMemcpyDeviceToHost), "read ticket");
    if (stall >= 0 && stall < ntasks)
        CK(cudaMemcpy(g.main.tasks.as<Task>() + stall, &saved, sizeof(Task), cudaMemcpyHostToDevice), "restore record");
    const auto w1 = std::chrono::steady_clock::now();
    if (st) {
        st->ntasks = std::min<long long>(tick, ntasks);
        st->seconds = ms * 1e-3;
        st->total_seconds = std::chrono::duration<double>(w1 - w0).count();
        st->tflops = algorithmic_flops(alg, n) / std::max(1e-12, st->seconds) * 1e-12;
        st->task = hs[ST_TASK];
        st->tile_m = hs[ST_M];
        st->tile_n = hs[ST_N];
        st->column = hs[ST_COL];
    }
    if (o.trace && hs[ST_CODE] == 0) {
        g.last_trace.dag = *dag;
        g.last_trace_workers = workers;
        g.last_trace.recs.resize(ntasks);
        CK(cudaMemcpy(g.last_trace.recs.data(), g.main.trace.ptr, sizeof(TraceRec) * ntasks, cudaMemcpyDeviceToHost),
           "read trace");
        g.last_trace.valid = true;
    }
    if (hs[ST_CODE] == PALIAL_ERR_NOT_SPD)
        return set_status(st, PALIAL_ERR_NOT_SPD, "non-positive pivot in tile (%d,%d) column %d", hs[ST_M], hs[ST_N],
                          hs[ST_COL]);
    if (hs[ST_CODE] == PALIAL_ERR_TIMEOUT)
        return set_status(st, PALIAL_ERR_TIMEOUT, "dependency wait timed out in task %d (object %d)", hs[ST_TASK],
                          hs[ST_COL]);
    if (hs[ST_CODE] != 0) return set_status(st, hs[ST_CODE], "device error %d", hs[ST_CODE]);
    if (hs[ST_ZEROPIV]) return set_status(st, PALIAL_WARN_ZERO_PIVOT, "exact zero pivot skipped");
    return set_status(st, PALIAL_OK);
}

static int factor_host(int alg, const palial_desc *A, const palial_desc *S, int *ipiv, const palial_opts *opts,
                       palial_status *st) {
    if (st) memset(st, 0, sizeof *st);
    if (!A || !A->matrix) return set_status(st, PALIAL_ERR_ARG, "NULL descriptor");
    if (alg == 2 && (!S || !S->matrix)) return set_status(st, PALIAL_ERR_ARG, "QR needs the S workspace");
    const int n = A->matrix_size, nb = A->tile_size;
    if (n <= 0 || nb <= 0 || n % nb) return set_status(st, PALIAL_ERR_ARG, "N %% NB != 0 (N=%d, NB=%d)", n, nb);
    if (alg == 2 && (S->matrix_size != n || S->tile_size != nb))
        return set_status(st, PALIAL_ERR_ARG, "S must have the same N and NB as A");
    int rc = ensure_init(st);
    if (rc) return rc;
    const auto w0 = std::chrono::steady_clock::now();
    const size_t bytes = sizeof(double) * (size_t)n * n;
    CK(g.mat.ensure(bytes), "alloc matrix");
    CK(cudaMemcpy(g.mat.ptr, A->matrix, bytes, cudaMemcpyHostToDevice), "copy A to device");
    double *dS = nullptr;
    if (alg == 2) {
        CK(g.smat.ensure(bytes), "alloc S");
        CK(cudaMemcpy(g.smat.ptr, S->matrix, bytes, cudaMemcpyHostToDevice), "copy S to device");
        dS = g.smat.as<double>();
    }
    rc = palial_gpu_factor_dev(alg, g.mat.as<double>(), dS, n, nb, opts, st, nullptr);
    if (rc < 0 && rc != PALIAL_ERR_NOT_SPD) return rc;
    CK(cudaMemcpy(A->matrix, g.mat.ptr, bytes, cudaMemcpyDeviceToHost), "copy A to host");
    if (alg == 2) CK(cudaMemcpy(S->matrix, g.smat.ptr, bytes, cudaMemcpyDeviceToHost), "copy S to host");
    if (ipiv)
        for (int i = 0; i < n; i++) ipiv[i] = i + 1;
    if (st) st->total_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - w0).count();
    return rc;
}

int palial_gpu_cholesky(const palial_desc *A, const palial_opts *opts, palial_status *st) {
    return factor_host(0, A, nullptr, nullptr, opts, st);
}
int palial_gpu_lu(const palial_desc *A, int *ipiv, const palial_opts *opts, palial_status *st) {
    return factor_host(1, A, nullptr, ipiv, opts, st);
}
int palial_gpu_qr(const palial_desc *A, const palial_desc *S, const palial_opts *opts, palial_status *st) {
    return factor_host(2, A, S, nullptr, opts, st);
}

// ---- single-tile kernels ----------------------------------------------------------------
static int tile_call(int type, int nb, int ld, double *p0, double *p1, double *p2, double *p3) {
    palial_status *st = nullptr;
    int rc = ensure_init(nullptr);
    if (rc) return rc;
    if (nb <= 0 || nb % 64 || ld < nb) return PALIAL_ERR_ARG;
    // scratch: 2 strips of nb x 64 (QR update kernels)
    const size_t need = sizeof(double) * ((size_t)2 * nb * 64);
    CK(g.main.scratch.ensure(need), "alloc scratch");
    CK(g.main.status.ensure(sizeof(int) * ST_NSLOTS + 64), "alloc status");
    CK(cudaMemset(g.main.status.ptr, 0, sizeof(int) * ST_NSLOTS), "clear status");
    CK(tile_task_launch(type, nb, ld, p0, p1, p2, p3, g.main.scratch.as<double>(), g.main.status.as<int>(), nullptr),
       "launch");
    CK(cudaDeviceSynchronize(), "tile kernel");
    int hs[ST_NSLOTS];
    CK(cudaMemcpy(hs, g.main.status.ptr, sizeof hs, cudaMemcpyDeviceToHost), "status");
    if (hs[ST_CODE]) return hs[ST_CODE];
    if (hs[ST_ZEROPIV]) return PALIAL_WARN_ZERO_PIVOT;
    return PALIAL_OK;
}

int palial_gpu_tile_dpotrf(int nb, double *dA, int lda) { return tile_call(T_POTRF, nb, lda, dA, 0, 0, 0); }
int palial_gpu_tile_dgetrf(int nb, double *dA, int lda) { return tile_call(T_GETRF, nb, lda, dA, 0, 0, 0); }
int palial_gpu_tile_dtrsm(int kind, int nb, const double *dT, double *dB, int lda) {
    const int ty = kind == 0 ? T_TRSM_LUT : kind == 1 ? T_TRSM_RUN : kind == 2 ? T_TRSM_LLU : kind == 3 ? T_TRSM_LUN : -1;
    if (ty < 0) return PALIAL_ERR_ARG;
    return tile_call(ty, nb, lda, const_cast<double *>(dT), dB, 0, 0);
}
int palial_gpu_tile_dsyrk(int nb, const double *dA, double *dC, int lda) {
    return tile_call(T_SYRK, nb, lda, const_cast<double *>(dA), dC, 0, 0);
}
int palial_gpu_tile_dgemm(int kind, int nb, const double *dA, const double *dB, double *dC, int lda) {
    if (kind != 0 && kind != 1) return PALIAL_ERR_ARG;
    return tile_call(kind == 0 ? T_GEMM_TN : T_GEMM_NN, nb, lda, const_cast<double *>(dA), const_cast<double *>(dB),
                     dC, 0);
}
int palial_gpu_tile_dgeqrt(int nb, double *dA, double *dT, int lda) {
    return tile_call(T_GEQRT, nb, lda, dA, dT, 0, 0);
}
int palial_gpu_tile_dormqr(int nb, const double *dV, const double *dT, double *dC, int lda) {
    return tile_call(T_UNMQR, nb, lda, const_cast<double *>(dV), const_cast<double *>(dT), dC, 0);
}
int palial_gpu_tile_dtsqrt(int nb, double *dA1, double *dA2, double *dT, int lda) {
    return tile_call(T_TSQRT, nb, lda, dA1, dA2, dT, 0);
}
int palial_gpu_tile_dtsmqr(int nb, double *dA1, double *dA2, const double *dV, const double *dT, int lda) {
    return tile_call(T_TSMQR, nb, lda, dA1, dA2, const_cast<double *>(dV), const_cast<double *>(dT));
}

// FP32 QR tile tasks (the mixed-precision QR's tile routines), one CTA, synchronous
static int tile_qr_call(int type, int nb, int ld, float *p0, float *p1, float *p2, float *p3) {
    palial_status *st = nullptr;
    int rc = ensure_init(nullptr);
    if (rc) return rc;
    if (nb <= 0 || nb % 64 || nb > 512 || ld < nb || !p0 || !p1 || (type != T_GEQRT && !p2) ||
        (type == T_TSMQR && !p3))
        return PALIAL_ERR_ARG;
    CK(g.main.scratch.ensure(sizeof(float) * ((size_t)2 * nb * 64)), "alloc scratch");
    CK(tile_qr_f32_launch(type, nb, ld, p0, p1, p2, p3, static_cast<float *>(g.main.scratch.ptr), nullptr), "launch");
    CK(cudaDeviceSynchronize(), "tile kernel");
    return PALIAL_OK;
}

int palial_gpu_tile_sgeqrt(int nb, float *dA, float *dT, int lda) { return tile_qr_call(T_GEQRT, nb, lda, dA, dT, 0, 0); }
int palial_gpu_tile_sormqr(int nb, const float *dV, const float *dT, float *dC, int lda) {
    return tile_qr_call(T_UNMQR, nb, lda, const_cast<float *>(dV), const_cast<float *>(dT), dC, 0);
}
int palial_gpu_tile_stsqrt(int nb, float *dA1, float *dA2, float *dT, int lda) {
    return tile_qr_call(T_TSQRT, nb, lda, dA1, dA2, dT, 0);
}
int palial_gpu_tile_stsmqr(int nb, float *dA1, float *dA2, const float *dV, const float *dT, int lda) {
    return tile_qr_call(T_TSMQR, nb, lda, dA1, dA2, const_cast<float *>(dV), const_cast<float *>(dT));
}

// ---- generators --------------------------------------------------------------------------
int palial_gpu_gen_uniform(double *dA, int n, int nb, uint64_t seed, void *stream) {
    palial_status *st = nullptr;
    int rc = ensure_init(nullptr);
    if (rc) return rc;
    if (!dA || n <= 0 || nb <= 0 || n % nb) return PALIAL_ERR_ARG;
    CK(launch_gen_uniform(dA, n, nb, seed, static_cast<cudaStream_t>(stream)), "gen uniform");
    return PALIAL_OK;
}

int palial_gpu_gen_dense(double *dX, long long rows, int cols, uint64_t seed, int stream_id, void *stream) {
    palial_status *st = nullptr;
    int rc = ensure_init(nullptr);
    if (rc) return rc;
    if (!dX || rows <= 0 || cols <= 0 || stream_id < 0) return PALIAL_ERR_ARG;
    CK(launch_gen_dense(dX, rows, cols, seed, stream_id, static_cast<cudaStream_t>(stream)), "gen dense");
    return PALIAL_OK;
}

int palial_gpu_gen_spd(double *dA, int n, int nb, uint64_t seed, void *stream) {
    palial_status *st = nullptr;
    int rc = ensure_init(nullptr);
    if (rc) return rc;
    if (!dA || n <= 0 || nb <= 0 || n % nb || n % 64) return PALIAL_ERR_ARG;
    CK(g.kbuf.ensure((size_t)n * n), "alloc K");
    CK(launch_gen_spd(dA, n, nb, seed, g.kbuf.as<int8_t>(), static_cast<cudaStream_t>(stream)), "gen spd");
    return PALIAL_OK;
}

int palial_gpu_gen_refpattern(double *dA, int n, int nb, uint64_t seed, void *stream) {
    palial_status *st = nullptr;
    int rc = ensure_init(nullptr);
    if (rc) return rc;
    if (!dA || n <= 0 || nb <= 0 || n % nb) return PALIAL_ERR_ARG;
    CK(launch_gen_refpattern(dA, n, nb, seed, static_cast<cudaStream_t>(stream)), "gen pattern");
    return PALIAL_OK;
}

int palial_gpu_generate(int kind, uint64_t seed, const palial_desc *A) {
    palial_status *st = nullptr;
    if (!A || !A->matrix) return PALIAL_ERR_ARG;
    const int n = A->matrix_size, nb = A->tile_size;
    if (n <= 0 || nb <= 0 || n % nb) return PALIAL_ERR_ARG;
    int rc = ensure_init(nullptr);
    if (rc) return rc;
    const size_t bytes = sizeof(double) * (size_t)n * n;
    CK(g.mat.ensure(bytes), "alloc matrix");
    if (kind == 0) rc = palial_gpu_gen_uniform(g.mat.as<double>(), n, nb, seed, nullptr);
    else if (kind == 1) rc = palial_gpu_gen_spd(g.mat.as<double>(), n, nb, seed, nullptr);
    else if (kind == 2) rc = palial_gpu_gen_refpattern(g.mat.as<double>(), n, nb, seed, nullptr);
    else return PALIAL_ERR_ARG;
    if (rc) return rc;
    CK(cudaMemcpy(A->matrix, g.mat.ptr, bytes, cudaMemcpyDeviceToHost), "copy to host");
    return PALIAL_OK;
}

// ---- residual probe ------------------------------------------------------------------------
int palial_gpu_residual_probe(int alg, const double *dA0, const double *dF, const double *dS, int n, int nb,
                              int nprobe, uint64_t seed, double *out) {
    palial_status *st = nullptr;
    (void)dS;
    int rc = ensure_init(nullptr);
    if (rc) return rc;
    if (!dA0 || !dF || !out || n % 64 || nprobe <= 0 || nprobe > 64) return PALIAL_ERR_ARG;
    const size_t v = (size_t)n * nprobe;
    CK(g.probe.ensure(sizeof(double) * (4 * v + 4096)), "alloc probe");
    double *X = g.probe.as<double>(), *Y = X + v, *Z = Y + v, *W = Z + v, *part = W + v;
    CK(launch_gen_dense(X, n, nprobe, seed, 5, nullptr), "probe gen");
    // Y = A0 X (or A0^T A0 X for QR), Z = F(X)
    if (alg == 0) {
        CK(launch_tiled_mm(dA0, X, Y, n, nb, nprobe, 0, 0, nullptr), "A X");
        CK(launch_tiled_mm(dF, X, W, n, nb, nprobe, 1, 0, nullptr), "U X");
        CK(launch_tiled_mm(dF, W, Z, n, nb, nprobe, 1, 1, nullptr), "U^T U X");
    } else if (alg == 1) {
        CK(launch_tiled_mm(dA0, X, Y, n, nb, nprobe, 0, 0, nullptr), "A X");
        CK(launch_tiled_mm(dF, X, W, n, nb, nprobe, 1, 0, nullptr), "U X");
        CK(launch_tiled_mm(dF, W, Z, n, nb, nprobe, 2, 0, nullptr), "L U X");
    } else {
        // R^T R = A^T A: compare A^T (A X) with R^T (R X)
        CK(launch_tiled_mm(dA0, X, W, n, nb, nprobe, 0, 0, nullptr), "A X");
        CK(launch_tiled_mm(dA0, W, Y, n, nb, nprobe, 0, 1, nullptr), "A^T A X");
        CK(launch_tiled_mm(dF, X, W, n, nb, nprobe, 1, 0, nullptr), "R X");
        CK(launch_tiled_mm(dF, W, Z, n, nb, nprobe, 1, 1, nullptr), "R^T R X");
    }
    CK(launch_sub(Y, Z, W, (long long)v, nullptr), "diff");
    const int blocks = 512;
    std::vector<double> hp(blocks);
    auto sumsq = [&](const double *p, long long len) -> double {
        if (launch_sumsq(p, len, part, blocks, nullptr) != cudaSuccess) return NAN;
        cudaMemcpy(hp.data(), part, sizeof(double) * blocks, cudaMemcpyDeviceToHost);
        double s = 0;
        for (double x : hp) s += x;
        return s;
    };
    const double dn = sqrt(sumsq(W, (long long)v));
    const double yn = sqrt(sumsq(Y, (long long)v));
    CK(cudaGetLastError(), "probe");
    *out = dn / yn;
    return PALIAL_OK;
}

int palial_gpu_residual_host(int alg, const double *a0_host, const palial_desc *F, int nprobe, uint64_t seed,
                             double *out) {
    palial_status *st = nullptr;
    if (!a0_host || !F || !F->matrix || !out) return PALIAL_ERR_ARG;
    const int n = F->matrix_size, nb = F->tile_size;
    int rc = ensure_init(nullptr);
    if (rc) return rc;
    const size_t bytes = sizeof(double) * (size_t)n * n;
    DevBuf a0, f;
    CK(a0.ensure(bytes), "alloc");
    CK(f.ensure(bytes), "alloc");
    CK(cudaMemcpy(a0.ptr, a0_host, bytes, cudaMemcpyHostToDevice), "copy");
    CK(cudaMemcpy(f.ptr, F->matrix, bytes, cudaMemcpyHostToDevice), "copy");
    rc = palial_gpu_residual_probe(alg, a0.as<double>(), f.as<double>(), nullptr, n, nb, nprobe, seed, out);
    a0.release();
    f.release();
    return rc;
}

// ---- batched factorizations ---------------------------------------------------------------
int palial_gpu_gen_batch_matrix(double *dA, int kind, int n_true, int n_pad, int nb, uint64_t seed, void *stream) {
    palial_status *st = nullptr;
    int rc = ensure_init(nullptr);
    if (rc) return rc;
    if (!dA || n_true <= 0 || n_pad < n_true || nb <= 0 || n_pad % nb || n_pad % 64 || (kind != 0 && kind != 1))
        return PALIAL_ERR_ARG;
    CK(g.kbuf.ensure((size_t)n_pad * n_pad), "alloc K");
    CK(launch_gen_batch(dA, kind, n_true, n_pad, nb, seed, g.kbuf.as<int8_t>(), static_cast<cudaStream_t>(stream)),
       "gen batch");
    return PALIAL_OK;
}

int palial_gpu_batched(int count, const int *algs, const int *ns, const int *nbs, const int *bss, double *const *dA,
                       const palial_opts *opts, palial_status *st, double *completion_s, void *stream) {
    if (st) memset(st, 0, sizeof *st);
    if (count <= 0 || !algs || !ns || !nbs || !bss || !dA) return set_status(st, PALIAL_ERR_ARG, "empty batch");
    return batched_run(count, algs, ns, nbs, bss, reinterpret_cast<void *const *>(dA), false, nullptr, opts, st,
                       completion_s, static_cast<cudaStream_t>(stream));
}

int palial_gpu_batched_f32(int count, const int *algs, const int *ns, const int *nbs, const int *bss, float *const *dA,
                           int *breakdown, const palial_opts *opts, palial_status *st, double *completion_s,
                           void *stream) {
    if (st) memset(st, 0, sizeof *st);
    if (count <= 0 || !algs || !ns || !nbs || !bss || !dA) return set_status(st, PALIAL_ERR_ARG, "empty batch");
    std::vector<int> flags(count, 0);
    const int rc = batched_run(count, algs, ns, nbs, bss, reinterpret_cast<void *const *>(dA), true, flags.data(), opts,
                               st, completion_s, static_cast<cudaStream_t>(stream));
    if (breakdown) std::copy(flags.begin(), flags.end(), breakdown);
    return rc;
}

// ---- trace ----------------------------------------------------------------------------------
long long palial_gpu_trace_count(void) {
    return g.last_trace.valid ? (long long)g.last_trace.dag.logical.size() : 0;
}

int palial_gpu_trace_dump(const char *path, const char *csv_path) {
    if (!g.last_trace.valid) return PALIAL_ERR_ARG;
    const Dag &d = g.last_trace.dag;
    const auto names = reference_names(d);
    const size_t nl = d.logical.size();
    std::vector<unsigned long long> t0(nl, ~0ull), t1(nl, 0);
    for (size_t r = 0; r < d.records.size(); r++) {
        const TraceRec &x = g.last_trace.recs[r];
        const uint32_t l = d.rec_logical[r];
        t0[l] = std::min(t0[l], x.t0);
        t1[l] = std::max(t1[l], x.t1);
    }
    FILE *f = path ? fopen(path, "w") : stdout;
    if (!f) return PALIAL_ERR_ARG;
    for (size_t l = 0; l < nl; l++) fprintf(f, "%s, %f\n", names[l].c_str(), (double)(t1[l] - t0[l]) * 1e-6);
    if (path) fclose(f);
    if (csv_path) {
        FILE *c = fopen(csv_path, "w");
        if (!c) return PALIAL_ERR_ARG;
        static const char *tn[] = {"potrf", "trsm", "syrk", "gemm", "getrf", "trsm", "trsm", "gemm",
                                   "geqrt", "ormqr", "tsqrt", "tsmqr", "trsm"};
        fprintf(c, "dispatch,logical,name,type,k,m,n,part,nparts,t0_ns,t1_ns,smid,clk\n");
        for (size_t r = 0; r < d.records.size(); r++) {
            const TraceRec &x = g.last_trace.recs[r];
            const Task &t = d.records[r];
            fprintf(c, "%zu,%u,%s,%s,%d,%d,%d,%d,%d,%llu,%llu,%u,%lld\n", r, d.rec_logical[r],
                    names[d.rec_logical[r]].c_str(), tn[t.type], t.k, t.m, t.n, t.part, t.nparts, x.t0, x.t1, x.smid,
                    x.clk);
        }
        fclose(c);
    }
    return PALIAL_OK;
}

// ---- DAG (host only) ------------------------------------------------------------------------
// ---- learned cost model plumbing ----------------------------------------------------------
// Features and log-durations (log of microseconds) of every task record of the last traced
// factorization; returns the number of records (or the count needed when cap is too small).
long long palial_gpu_trace_features(float *X, float *y, long long cap) {
    if (!g.last_trace.valid) return -1;
    const Dag &d = g.last_trace.dag;
    const long long nrec = (long long)d.records.size();
    if (!X || !y || cap < nrec) return nrec;
    const auto widths = step_widths(d);
    for (long long r = 0; r < nrec; r++) {
        const LogicalTask &t = d.logical[d.rec_logical[r]];
        task_features(d, t, d.records[r].part, g.last_trace_workers, 0, widths, X + r * kFeatures);
        const double us = std::max(1.0, (double)(g.last_trace.recs[r].t1 - g.last_trace.recs[r].t0) * 1e-3);
        y[r] = (float)std::log(us);
    }
    return nrec;
}

// Features of every logical task (part 0) of a DAG, for planning with the model.
long long palial_dag_logical_features(int alg, int n, int nb, int block, int nworkers, float *X, long long cap) {
    try {
        const int bs = block > 0 ? block : auto_block(alg, n, nb);
        Dag d = build_dag(alg, n, nb, bs);
        const long long nl = (long long)d.logical.size();
        if (!X || cap < nl) return nl;
        const auto widths = step_widths(d);
        for (long long i = 0; i < nl; i++) task_features(d, d.logical[i], 0, nworkers, 0, widths, X + i * kFeatures);
        return nl;
    } catch (const std::exception &) {
        return -1;
    }
}

int palial_gpu_set_task_costs(int alg, int n, int nb, int block, const double *cost_s, long long count) {
    const int bs = block > 0 ? block : auto_block(alg, n, nb);
    if (!cost_s || count <= 0) {
        g.task_costs.erase(cost_key(alg, n, nb, bs));
    } else {
        g.task_costs[cost_key(alg, n, nb, bs)] = std::vector<double>(cost_s, cost_s + count);
    }
    // invalidate cached learned-priority DAGs of this shape
    for (auto it = g.dags.begin(); it != g.dags.end();) {
        if (std::get<4>(it->first) == 2) it = g.dags.erase(it);
        else ++it;
    }
    return PALIAL_OK;
}

int palial_dag_features_count(void) { return kFeatures; }

// The reference-rule task names of a DAG (creation order), newline separated.  Returns the
// number of bytes needed (including the terminating zero).
long long palial_dag_names(int alg, int n, int nb, int block, char *buf, long long buflen) {
    try {
        const int bs = block > 0 ? block : auto_block(alg, n, nb);
        Dag d = build_dag(alg, n, nb, bs);
        std::string all;
        for (const auto &s : reference_names(d)) {
            all += s;
            all += '\n';
        }
        if (buf && buflen > (long long)all.size()) memcpy(buf, all.c_str(), all.size() + 1);
        return (long long)all.size() + 1;
    } catch (const std::exception &) {
        return -1;
    }
}

long long palial_dag_info(int alg, int n, int nb, int block, int priority, int nworkers, long long *type_counts,
                          double *critical_path_s, double *makespan_s) {
    try {
        const int bs = block > 0 ? block : auto_block(alg, n, nb);
        Dag d = build_dag(alg, n, nb, bs);
        if (priority == 2) apply_learned_costs(d);
        order_dag(d, priority == 2 ? 0 : priority, nworkers, 0);
        if (type_counts) {
            for (int i = 0; i < 16; i++) type_counts[i] = 0;
            for (const auto &t : d.logical) type_counts[t.type]++;
        }
        if (critical_path_s) *critical_path_s = d.critical_path;
        if (makespan_s) *makespan_s = d.sim_makespan;
        return (long long)d.records.size();
    } catch (const std::exception &) {
        return -1;
    }
}

int palial_dag_validate(int alg, int n, int nb, int block, int priority, int nworkers, unsigned int seed, char *msg,
                        int msglen) {
    try {
        const int bs = block > 0 ? block : auto_block(alg, n, nb);
        Dag d = build_dag(alg, n, nb, bs);
        order_dag(d, priority, nworkers, seed);
        const std::string r = validate_dag(d, nworkers, seed);
        if (msg && msglen > 0) snprintf(msg, msglen, "%s", r.c_str());
        return r.empty() ? 0 : 1;
    } catch (const std::exception &ex) {
        if (msg && msglen > 0) snprintf(msg, msglen, "%s", ex.what());
        return -1;
    }
}

long long palial_dag_qr_apply_validate(int n, int nb, int nrhs, int nworkers, unsigned int seed,
                                       long long *type_counts, char *msg, int msglen) {
    try {
        Dag d = build_qr_solve_dag(n, n, nb, nrhs, true);
        order_dag(d, 0, nworkers, seed);
        if (type_counts) {
            for (int i = 0; i < 16; i++) type_counts[i] = 0;
            for (const auto &t : d.logical) type_counts[t.type]++;
        }
        const std::string r = validate_dag(d, nworkers, seed);
        if (msg && msglen > 0) snprintf(msg, msglen, "%s", r.c_str());
        return r.empty() ? (long long)d.records.size() : -1;
    } catch (const std::exception &ex) {
        if (msg && msglen > 0) snprintf(msg, msglen, "%s", ex.what());
        return -1;
    }
}

long long palial_dag_qr_solve_validate(int rows, int cols, int nb, int nrhs, int nworkers, unsigned int seed,
                                       long long *type_counts, char *msg, int msglen) {
    try {
        Dag d = build_qr_solve_dag(rows, cols, nb, nrhs);
        order_dag(d, 0, nworkers, seed);
        if (type_counts) {
            for (int i = 0; i < 16; i++) type_counts[i] = 0;
            for (const auto &t : d.logical) type_counts[t.type]++;
        }
        const std::string r = validate_dag(d, nworkers, seed);
        if (msg && msglen > 0) snprintf(msg, msglen, "%s", r.c_str());
        return r.empty() ? (long long)d.records.size() : -1;
    } catch (const std::exception &ex) {
        if (msg && msglen > 0) snprintf(msg, msglen, "%s", ex.what());
        return -1;
    }
}

int palial_dag_batch_validate(int count, const int *algs, const int *ns, const int *nbs, const int *bss, int nworkers,
                              unsigned int seed, char *msg, int msglen) {
    try {
        std::vector<BatchSpec> specs(count);
        for (int i = 0; i < count; i++) specs[i] = BatchSpec{algs[i], ns[i], nbs[i], bss[i]};
        Dag d = build_batch_dag(specs);
        order_dag(d, 0, nworkers, seed);
        std::string r = validate_dag(d, nworkers, seed);
        // every record of matrix i touches only matrix i's objects
        std::vector<uint32_t> lo(count, ~0u), hi(count, 0);
        uint32_t base = 0;
        for (int i = 0; i < count; i++) {
            const int mb = ns[i] / bss[i];
            lo[i] = base;
            hi[i] = base + (uint32_t)(mb * mb);
            base = hi[i];
        }
        for (size_t q = 0; q < d.records.size() && r.empty(); q++) {
            const Task &t = d.records[q];
            for (int w = 0; w < t.nwait; w++)
                if (t.wait_obj[w] < lo[t.mat] || t.wait_obj[w] >= hi[t.mat]) r = "record waits on another matrix";
            for (int s2 = 0; s2 < t.nsig; s2++)
                if (t.sig_obj[s2] < lo[t.mat] || t.sig_obj[s2] >= hi[t.mat]) r = "record signals another matrix";
        }
        if (msg && msglen > 0) snprintf(msg, msglen, "%s", r.c_str());
        return r.empty() ? 0 : 1;
    } catch (const std::exception &ex) {
        if (msg && msglen > 0) snprintf(msg, msglen, "%s", ex.what());
        return -1;
    }
}

int palial_gpu_clock_report(palial_clock_report *out) {
    if (!out) return PALIAL_ERR_ARG;
    out->sm_mhz_start = out->sm_mhz_end = out->sm_mhz_max = -1;
    out->throttle_reasons = -1;
    out->sm_mhz_device = -1;
    if (g.last_trace.valid) {
        double cyc = 0, ns = 0;
        for (const auto &r : g.last_trace.recs) {
            cyc += (double)r.clk;
            ns += (double)(r.t1 - r.t0);
        }
        if (ns > 0) out->sm_mhz_device = cyc / ns * 1e3;
        out->sm_mhz_start = g.clk_start;
        out->sm_mhz_end = g.clk_end;
        out->sm_mhz_max = g.clk_max;
        out->throttle_reasons = (int)g.clk_reasons;
    } else {
        // no traced run yet: the current clocks
        long long r;
        nvml_sample(&out->sm_mhz_end, &out->sm_mhz_max, &r);
        out->throttle_reasons = (int)r;
    }
    return PALIAL_OK;
}

// Replays the last trace into the reference's hook interface (include/common.h:9-11 of the
// reference): every task name in creation order (set_task_name, called by the reference at
// task creation), then per task in start order the executing SM and GPU ordinal
// (set_task_cpu_node: cpu -> SM id, node -> device) and the start/end wall times in
// microseconds since the epoch (get_task_time; the host clock at launch plus the device
// %globaltimer offsets).  A NULL hook is skipped.
int palial_gpu_trace_hooks(void (*set_name)(const char *), void (*cpu_node)(int, int, char *),
                           void (*task_time)(long long, long long, char *)) {
    if (!g.last_trace.valid) return PALIAL_ERR_ARG;
    const Dag &d = g.last_trace.dag;
    const auto names = reference_names(d);
    const size_t nl = d.logical.size();
    std::vector<unsigned long long> t0(nl, ~0ull), t1(nl, 0);
    std::vector<unsigned> sm(nl, 0);
    unsigned long long tmin = ~0ull;
    for (size_t r = 0; r < d.records.size(); r++) {
        const TraceRec &x = g.last_trace.recs[r];
        const uint32_t l = d.rec_logical[r];
        if (x.t0 < t0[l]) {
            t0[l] = x.t0;
            sm[l] = x.smid;
        }
        t1[l] = std::max(t1[l], x.t1);
        tmin = std::min(tmin, x.t0);
    }
    std::vector<std::vector<char>> buf(nl);
    for (size_t l = 0; l < nl; l++) {
        buf[l].assign(names[l].begin(), names[l].end());
        buf[l].push_back(0);
        if (set_name) set_name(buf[l].data());
    }
    std::vector<size_t> order(nl);
    for (size_t l = 0; l < nl; l++) order[l] = l;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return t0[a] < t0[b]; });
    for (size_t l : order) {
        if (cpu_node) cpu_node((int)sm[l], g.device, buf[l].data());
        if (task_time) {
            const long long s = (g.last_trace_host_ns + (long long)(t0[l] - tmin)) / 1000;
            const long long e = (g.last_trace_host_ns + (long long)(t1[l] - tmin)) / 1000;
            task_time(s, e, buf[l].data());
        }
    }
    return PALIAL_OK;
}

}  // extern "C"
