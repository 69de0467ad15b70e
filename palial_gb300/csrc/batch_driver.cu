// batch_driver.cu -- the synthetic uneven batch (2000 matrices, N log-uniform in [32, 2048)),
// its per-size-class block autotuner, and the size-balanced partition of a batch over ranks.
//
// The batch: matrix i has N_i = floor(32 * 64^u_i), u_i uniform in [0, 1) from splitmix64 of
// (seed, stream 6, index i); even i are SPD (Cholesky), odd i uniform [-1, 1) (no-pivot LU).
// Each matrix sits in its own tile buffer padded to a multiple of its block size (identity
// padding for LU, N I for Cholesky) and all of them run in one persistent launch
// (palial_gpu_batched).  The autotuner times every size class alone with each candidate block
// size and keeps the fastest.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <queue>
#include <vector>

#include "host_state.hpp"

namespace palial {
cudaError_t launch_gen_dense(double *X, long long rows, int cols, uint64_t seed, int stream, cudaStream_t s);
namespace {

constexpr int kClassEdges[7] = {32, 64, 128, 256, 512, 1024, 2048};
constexpr int kCandidates[3] = {64, 128, 256};

uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int size_class(int n) {
    for (int c = 0; c < 5; c++)
        if (n < kClassEdges[c + 1]) return c;
    return 5;
}

int padded(int n, int bs) { return (n + bs - 1) / bs * bs; }

// Device copy of one (sub)batch: matrices generated once, a pristine copy for resets.
struct BatchBufs {
    std::vector<int> ns, algs, np, bs, idx;
    std::vector<double *> ptrs;
    double *buf = nullptr, *pristine = nullptr;
    size_t elems = 0;
    double flops = 0;
    ~BatchBufs() {
        if (buf) cudaFree(buf);
        if (pristine) cudaFree(pristine);
    }
};

int make_batch(BatchBufs &b, const std::vector<int> &idx, const std::vector<int> &ns, const std::vector<int> &algs,
               const int *bs_of_class, uint64_t seed, palial_status *st) {
    b.idx = idx;
    std::vector<size_t> off;
    for (int i : idx) {
        const int n = ns[i], bs = bs_of_class[size_class(n)];
        b.ns.push_back(n);
        b.algs.push_back(algs[i]);
        b.bs.push_back(bs);
        b.np.push_back(padded(n, bs));
        off.push_back(b.elems);
        b.elems += (size_t)b.np.back() * b.np.back();
        b.flops += algorithmic_flops(algs[i], n);
    }
    PALIAL_CK(cudaMalloc(&b.buf, sizeof(double) * std::max<size_t>(1, b.elems)), "alloc batch");
    PALIAL_CK(cudaMalloc(&b.pristine, sizeof(double) * std::max<size_t>(1, b.elems)), "alloc batch copy");
    for (size_t j = 0; j < idx.size(); j++) {
        b.ptrs.push_back(b.buf + off[j]);
        const int rc = palial_gpu_gen_batch_matrix(b.ptrs[j], b.algs[j] == 0 ? 1 : 0, b.ns[j], b.np[j], b.bs[j],
                                                   seed * 100000ull + (uint64_t)idx[j], nullptr);
        if (rc) return set_status(st, rc, "generating batch matrix %d", idx[j]);
    }
    PALIAL_CK(cudaMemcpy(b.pristine, b.buf, sizeof(double) * b.elems, cudaMemcpyDeviceToDevice), "copy batch");
    return PALIAL_OK;
}

// Reset to the pristine inputs and run one batched launch (graph replay).
int run_batch(BatchBufs &b, const palial_opts &o, palial_status *st, double *completion) {
    PALIAL_CK(cudaMemcpy(b.buf, b.pristine, sizeof(double) * b.elems, cudaMemcpyDeviceToDevice), "reset batch");
    palial_opts ro = o;
    ro.reserved[2] = 1;
    return palial_gpu_batched((int)b.ns.size(), b.algs.data(), b.np.data(), b.bs.data(), b.bs.data(), b.ptrs.data(),
                              &ro, st, completion, nullptr);
}

// Device copy of a (sub)batch for the batched solves: per matrix A (padded, tile = block
// size of its (algorithm, size class)), b (uniform [-1, 1), stream 7 of the matrix's seed)
// and x.  A and b are read only, so repeated solves need no reset.
struct SolveBatch {
    std::vector<int> ns, algs, np, bs, prec;
    std::vector<const double *> A, B;
    std::vector<double *> X;
    double *buf = nullptr;
    double flops = 0;
    ~SolveBatch() {
        if (buf) cudaFree(buf);
    }
};

int make_solve_batch(SolveBatch &b, const std::vector<int> &idx, const std::vector<int> &ns,
                     const std::vector<int> &algs, const int *bs12, const int *prec12, uint64_t seed,
                     palial_status *st) {
    std::vector<size_t> offa, offb, offx;
    size_t elems = 0;
    for (int i : idx) {
        const int k = algs[i] * 6 + size_class(ns[i]);
        b.ns.push_back(ns[i]);
        b.algs.push_back(algs[i]);
        b.bs.push_back(bs12[k]);
        b.prec.push_back(prec12[k]);
        b.np.push_back(padded(ns[i], bs12[k]));
        const size_t np = (size_t)b.np.back();
        offa.push_back(elems);
        elems += (np * np + 3) / 4 * 4;
        b.flops += algorithmic_flops(algs[i], ns[i]);
    }
    for (size_t j = 0; j < idx.size(); j++) {
        offb.push_back(elems);
        elems += ((size_t)b.np[j] + 3) / 4 * 4;
        offx.push_back(elems);
        elems += ((size_t)b.np[j] + 3) / 4 * 4;
    }
    PALIAL_CK(cudaMalloc(&b.buf, sizeof(double) * std::max<size_t>(4, elems)), "alloc solve batch");
    for (size_t j = 0; j < idx.size(); j++) {
        b.A.push_back(b.buf + offa[j]);
        b.B.push_back(b.buf + offb[j]);
        b.X.push_back(b.buf + offx[j]);
        const uint64_t ms = seed * 100000ull + (uint64_t)idx[j];
        const int rc = palial_gpu_gen_batch_matrix(b.buf + offa[j], b.algs[j] == 0 ? 1 : 0, b.ns[j], b.np[j], b.bs[j],
                                                   ms, nullptr);
        if (rc) return set_status(st, rc, "generating batch matrix %d", idx[j]);
        PALIAL_CK(launch_gen_dense(b.buf + offb[j], b.np[j], 1, ms, 7, nullptr), "generating right-hand side");
    }
    PALIAL_CK(cudaDeviceSynchronize(), "generate solve batch");
    return PALIAL_OK;
}

struct SolveResult {
    double seconds = 0, worst = 0, phases[3] = {0, 0, 0};
    int fallbacks = 0, butterflies = 0, max_iters = 0, rc = 0;
};

int run_solve_batch(SolveBatch &b, const palial_opts &o, SolveResult &res, palial_status *st) {
    const int count = (int)b.ns.size();
    std::vector<int> prec(count), iters(count);
    std::vector<double> berr(count);
    // precision choice per matrix: 0 FP64, 1 FP32, 2 FP32 storage with BF16x3 tensor-core updates
    for (int j = 0; j < count; j++)
        prec[j] = b.prec[j] == 2 ? PALIAL_PREC_BF16X3 : b.prec[j] ? PALIAL_PREC_FP32 : PALIAL_PREC_FP64;
    palial_status s2;
    const int rc = batched_solve_run(count, b.algs.data(), b.np.data(), b.bs.data(), b.A.data(), b.B.data(),
                                     b.X.data(), prec.data(), &o, &s2, iters.data(), berr.data(), res.phases, nullptr);
    if (rc < 0 && rc != PALIAL_ERR_NOT_CONVERGED) return set_status(st, rc, "batched solve: %s", s2.message);
    res.rc = rc;
    res.seconds = s2.seconds;
    res.worst = s2.backward_error;
    res.fallbacks = s2.fallbacks;
    res.butterflies = s2.butterflies;
    res.max_iters = s2.ir_iters;
    return PALIAL_OK;
}

double percentile(std::vector<double> v, double q) {
    if (v.empty()) return 0;
    std::sort(v.begin(), v.end());
    // linear interpolation between closest ranks (numpy's default)
    const double pos = q / 100.0 * (double)(v.size() - 1);
    const size_t lo = (size_t)std::floor(pos), hi = std::min(v.size() - 1, lo + 1);
    return v[lo] + (v[hi] - v[lo]) * (pos - (double)lo);
}

}  // namespace
}  // namespace palial

using namespace palial;

extern "C" {

int palial_gpu_batch_sizes(int count, uint64_t seed, int *ns, int *algs) {
    if (count < 0 || (count > 0 && (!ns || !algs))) return PALIAL_ERR_ARG;
    const uint64_t key = mix64(seed * 0xD1B54A32D192ED03ull + 6ull);
    for (int i = 0; i < count; i++) {
        const double u = (double)(mix64(key + (uint64_t)i) >> 11) * 0x1.0p-53;
        ns[i] = std::min(2047, (int)std::floor(32.0 * std::pow(64.0, u)));
        algs[i] = i % 2;
    }
    return PALIAL_OK;
}

int palial_gpu_batch_partition(int count, const int *ns, const int *algs, int world, int *rank_of) {
    if (count < 0 || world < 1 || (count > 0 && (!ns || !algs || !rank_of))) return PALIAL_ERR_ARG;
    // longest processing time first on the flop counts; ties by index (deterministic on every rank)
    std::vector<int> order(count);
    std::iota(order.begin(), order.end(), 0);
    auto work = [&](int i) { return algorithmic_flops(algs[i], (double)ns[i]); };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return work(a) > work(b); });
    using Load = std::pair<double, int>;
    std::priority_queue<Load, std::vector<Load>, std::greater<Load>> load;
    for (int r = 0; r < world; r++) load.push({0.0, r});
    for (int i : order) {
        Load l = load.top();
        load.pop();
        rank_of[i] = l.second;
        l.first += work(i);
        load.push(l);
    }
    return PALIAL_OK;
}

int palial_gpu_batch_autotune(int count, const int *ns, const int *algs, uint64_t seed, int reps, int *bs_of_class,
                              double *timings, palial_status *st) {
    if (st) memset(st, 0, sizeof *st);
    if (count <= 0 || !ns || !algs || !bs_of_class) return set_status(st, PALIAL_ERR_ARG, "empty batch");
    int rc = ensure_init(st);
    if (rc) return rc;
    std::vector<int> vn(ns, ns + count), va(algs, algs + count);
    palial_opts o;
    palial_opts_default(&o);
    if (timings)
        for (int i = 0; i < 18; i++) timings[i] = -1;
    for (int c = 0; c < 6; c++) {
        std::vector<int> idx;
        for (int i = 0; i < count; i++)
            if (size_class(vn[i]) == c) idx.push_back(i);
        bs_of_class[c] = 64;
        if (idx.empty()) continue;
        double best = 1e30;
        for (int j = 0; j < 3; j++) {
            const int bs = kCandidates[j];
            if (bs > std::max(64, kClassEdges[c + 1])) continue;
            int cls[6];
            for (int q = 0; q < 6; q++) cls[q] = bs;
            BatchBufs b;
            rc = make_batch(b, idx, vn, va, cls, seed, st);
            if (rc) return rc;
            double t = 1e30;
            for (int r = 0; r <= std::max(1, reps); r++) {
                palial_status s2;
                rc = run_batch(b, o, &s2, nullptr);
                if (rc < 0) return set_status(st, rc, "autotune run: %s", s2.message);
                if (r > 0) t = std::min(t, s2.seconds);
            }
            if (timings) timings[c * 3 + j] = t;
            if (t < best) {
                best = t;
                bs_of_class[c] = bs;
            }
        }
    }
    return set_status(st, PALIAL_OK);
}

int palial_gpu_batch_synthetic(int count, uint64_t seed, int rank, int world, int autotune, const int *bs_of_class,
                               int reps, const palial_opts *opts, palial_status *st, palial_batch_report *rep) {
    if (st) memset(st, 0, sizeof *st);
    if (count <= 0 || world < 1 || rank < 0 || rank >= world || !rep)
        return set_status(st, PALIAL_ERR_ARG, "bad batch arguments");
    memset(rep, 0, sizeof *rep);
    int rc = ensure_init(st);
    if (rc) return rc;
    palial_opts o;
    palial_opts_default(&o);
    if (opts) o = *opts;
    std::vector<int> ns(count), algs(count), owner(count);
    palial_gpu_batch_sizes(count, seed, ns.data(), algs.data());
    palial_gpu_batch_partition(count, ns.data(), algs.data(), world, owner.data());
    std::vector<int> idx;
    for (int i = 0; i < count; i++)
        if (owner[i] == rank) idx.push_back(i);
    std::vector<int> mns, malgs;
    for (int i : idx) {
        mns.push_back(ns[i]);
        malgs.push_back(algs[i]);
    }
    int cls[6];
    for (int c = 0; c < 6; c++) cls[c] = bs_of_class ? bs_of_class[c] : (c < 4 ? 64 : 128);
    const auto t0 = std::chrono::steady_clock::now();
    if (autotune && !idx.empty()) {
        rc = palial_gpu_batch_autotune((int)idx.size(), mns.data(), malgs.data(), seed, 2, cls, rep->autotune_s, st);
        if (rc) return rc;
    }
    rep->autotune_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    rep->count = (int)idx.size();
    if (idx.empty()) return set_status(st, PALIAL_OK);
    BatchBufs b;
    rc = make_batch(b, idx, ns, algs, cls, seed, st);
    if (rc) return rc;
    std::vector<double> comp(idx.size()), times;
    palial_status s2;
    rc = run_batch(b, o, &s2, nullptr);  // warm-up (graph capture)
    if (rc < 0) return set_status(st, rc, "%s", s2.message);
    for (int r = 0; r < std::max(1, reps); r++) {
        rc = run_batch(b, o, &s2, comp.data());
        if (rc < 0) return set_status(st, rc, "%s", s2.message);
        times.push_back(s2.seconds);
    }
    const double t = percentile(times, 50);
    rep->seconds = t;
    rep->matrices_per_s = (double)idx.size() / t;
    rep->tflops = b.flops / t * 1e-12;
    for (int c = 0; c < 6; c++) {
        rep->bs_of_class[c] = cls[c];
        std::vector<double> v;
        for (size_t j = 0; j < idx.size(); j++)
            if (size_class(b.ns[j]) == c) v.push_back(comp[j] * 1e3);
        rep->count_of_class[c] = (int)v.size();
        rep->p50_ms[c] = percentile(v, 50);
        rep->p99_ms[c] = percentile(v, 99);
    }
    if (st) {
        st->seconds = t;
        st->tflops = rep->tflops;
        st->ntasks = s2.ntasks;
    }
    return set_status(st, PALIAL_OK);
}

int palial_gpu_batch_solve_autotune(int count, const int *ns, const int *algs, uint64_t seed, int reps, int *bs12,
                                    int *prec12, double *timings, palial_status *st) {
    if (st) memset(st, 0, sizeof *st);
    if (count <= 0 || !ns || !algs || !bs12 || !prec12) return set_status(st, PALIAL_ERR_ARG, "empty batch");
    int rc = ensure_init(st);
    if (rc) return rc;
    std::vector<int> vn(ns, ns + count), va(algs, algs + count);
    palial_opts o;
    palial_opts_default(&o);
    if (timings)
        for (int i = 0; i < 108; i++) timings[i] = -1;
    for (int k = 0; k < 12; k++) {
        const int a = k / 6, c = k % 6;
        std::vector<int> idx;
        for (int i = 0; i < count; i++)
            if (va[i] == a && size_class(vn[i]) == c) idx.push_back(i);
        bs12[k] = 64;
        prec12[k] = 0;
        if (idx.empty()) continue;
        double best = 1e30;
        for (int prec = 0; prec < 3; prec++)
            for (int j = 0; j < 3; j++) {
                const int bs = kCandidates[j];
                if (bs > std::max(64, kClassEdges[c + 1])) continue;
                int b12[12], p12[12];
                for (int q = 0; q < 12; q++) {
                    b12[q] = bs;
                    p12[q] = prec;
                }
                SolveBatch b;
                rc = make_solve_batch(b, idx, vn, va, b12, p12, seed, st);
                if (rc) return rc;
                double t = 1e30;
                for (int r = 0; r <= std::max(1, reps); r++) {
                    SolveResult res;
                    rc = run_solve_batch(b, o, res, st);
                    if (rc) return rc;
                    // a choice must reach the tolerance on every matrix
                    if (res.rc != PALIAL_OK) {
                        t = 1e30;
                        break;
                    }
                    if (r > 0) t = std::min(t, res.seconds);
                }
                if (timings) timings[k * 9 + prec * 3 + j] = t < 1e30 ? t : -2;
                if (t < best) {
                    best = t;
                    bs12[k] = bs;
                    prec12[k] = prec;
                }
            }
    }
    return set_status(st, PALIAL_OK);
}

int palial_gpu_batch_solve_synthetic(int count, uint64_t seed, int rank, int world, int autotune, const int *bs12_in,
                                     const int *prec12_in, int reps, const palial_opts *opts, palial_status *st,
                                     palial_batch_solve_report *rep) {
    if (st) memset(st, 0, sizeof *st);
    if (count <= 0 || world < 1 || rank < 0 || rank >= world || !rep)
        return set_status(st, PALIAL_ERR_ARG, "bad batch arguments");
    memset(rep, 0, sizeof *rep);
    int rc = ensure_init(st);
    if (rc) return rc;
    palial_opts o;
    palial_opts_default(&o);
    if (opts) o = *opts;
    std::vector<int> ns(count), algs(count), owner(count);
    palial_gpu_batch_sizes(count, seed, ns.data(), algs.data());
    palial_gpu_batch_partition(count, ns.data(), algs.data(), world, owner.data());
    std::vector<int> idx, mns, malgs;
    for (int i = 0; i < count; i++)
        if (owner[i] == rank) {
            idx.push_back(i);
            mns.push_back(ns[i]);
            malgs.push_back(algs[i]);
        }
    int bs12[12], prec12[12];
    for (int k = 0; k < 12; k++) {
        bs12[k] = bs12_in ? bs12_in[k] : (k % 6 < 4 ? 64 : 128);
        prec12[k] = prec12_in ? prec12_in[k] : 1;
    }
    const auto t0 = std::chrono::steady_clock::now();
    if (autotune && !idx.empty()) {
        rc = palial_gpu_batch_solve_autotune((int)idx.size(), mns.data(), malgs.data(), seed, 1, bs12, prec12,
                                             rep->autotune_s, st);
        if (rc) return rc;
    }
    rep->autotune_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    rep->count = (int)idx.size();
    for (int k = 0; k < 12; k++) {
        rep->bs_of_class[k] = bs12[k];
        rep->prec_of_class[k] = prec12[k];
    }
    if (idx.empty()) return set_status(st, PALIAL_OK);
    SolveBatch b;
    rc = make_solve_batch(b, idx, ns, algs, bs12, prec12, seed, st);
    if (rc) return rc;
    SolveResult res;
    rc = run_solve_batch(b, o, res, st);  // warm-up (allocations, DAGs)
    if (rc) return rc;
    std::vector<double> times;
    std::vector<SolveResult> runs;
    for (int r = 0; r < std::max(1, reps); r++) {
        rc = run_solve_batch(b, o, res, st);
        if (rc) return rc;
        runs.push_back(res);
        times.push_back(res.seconds);
        rep->max_backward_error = std::max(rep->max_backward_error, res.worst);
        rep->fallbacks = std::max(rep->fallbacks, res.fallbacks);
        rep->butterflies = std::max(rep->butterflies, res.butterflies);
        rep->max_iters = std::max(rep->max_iters, res.max_iters);
        if (res.rc != PALIAL_OK) rep->not_converged = 1;
    }
    const double t = percentile(times, 50);
    rep->seconds = t;
    rep->matrices_per_s = (double)idx.size() / t;
    rep->tflops = b.flops / t * 1e-12;
    // phases of the run closest to the median
    size_t med = 0;
    for (size_t r = 1; r < runs.size(); r++)
        if (std::fabs(runs[r].seconds - t) < std::fabs(runs[med].seconds - t)) med = r;
    for (int q = 0; q < 3; q++) rep->phase_seconds[q] = runs[med].phases[q];
    if (st) {
        st->seconds = t;
        st->tflops = rep->tflops;
        st->backward_error = rep->max_backward_error;
    }
    return set_status(st, rep->not_converged ? PALIAL_ERR_NOT_CONVERGED : PALIAL_OK,
                      rep->not_converged ? "batched solve above its tolerance" : nullptr);
}

}  // extern "C"
