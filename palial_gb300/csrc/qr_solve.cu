// qr_solve.cu -- linear solve and least squares through the tile QR (no reference
// counterpart: the reference's qr() stops at the factors, src/qr.h:15-192).
//
// A (rows x cols tile layout, rows >= cols, FP64, device) is copied into a work matrix of
// rows x (cols + nb) whose extra tile column holds the right-hand sides.  One persistent
// scheduler launch runs the flat-tree tile QR of A; its UNMQR/TSMQR tasks on the extra tile
// column apply Q^T to B as the factorization proceeds, and the blocked back-substitution
// R X = (Q^T B)(0:cols) follows in the same dispatch list (DAG in dag.cpp,
// build_qr_solve_dag).  For rows > cols the rows cols..rows-1 of Q^T B hold the least-squares
// residual: its 2-norm per column is min ||A x - b||_2.
#include <cuda_runtime.h>

#include <chrono>
#include <cstring>

#include "host_state.hpp"

namespace palial {
namespace {

// B (rows x nrhs, column-major, ld rows) -> tile column `tc` of the rows x * tile layout
// (width columns, zero beyond nrhs).
__global__ void rhs_to_tiles_kernel(const double *__restrict__ B, double *__restrict__ W, int rows, int nrhs,
                                    int nb, int width) {
    const long long total = (long long)rows * width;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e / rows), r = (int)(e % rows);
        const int tm = r / nb, rr = r % nb;
        W[(size_t)tm * nb * nb + rr + (size_t)c * nb] = c < nrhs ? B[r + (size_t)c * rows] : 0.0;
    }
}

// X (cols x nrhs, ld cols) <- the first cols rows of the tile column.
__global__ void tiles_to_x_kernel(const double *__restrict__ W, double *__restrict__ X, int cols, int nrhs, int nb) {
    const long long total = (long long)cols * nrhs;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e / cols), r = (int)(e % cols);
        X[r + (size_t)c * cols] = W[(size_t)(r / nb) * nb * nb + (r % nb) + (size_t)c * nb];
    }
}

// resid[c] = ||(Q^T b_c)(cols:rows)||_2, one CTA per right-hand side (sum of squares in a
// fixed order, so the result does not depend on the launch).
__global__ void ls_resid_kernel(const double *__restrict__ W, double *__restrict__ resid, int rows, int cols,
                                int nb) {
    __shared__ double red[256];
    const int c = blockIdx.x;
    double s = 0.0;
    for (int r = cols + threadIdx.x; r < rows; r += blockDim.x) {
        const double v = W[(size_t)(r / nb) * nb * nb + (r % nb) + (size_t)c * nb];
        s = fma(v, v, s);
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) resid[c] = sqrt(red[0]);
}

DevBuf qs_work, qs_s;
std::shared_ptr<Dag> qs_dag;
int qs_key[6] = {0, 0, 0, 0, -1, 0};
std::shared_ptr<Dag> ts_dag;  // FP64 triangular solves (build_trsolve_dag)
int ts_key[4] = {0, 0, 0, -1};

int grid_for(long long elems) {
    const long long b = (elems + 255) / 256;
    return (int)std::max(1LL, std::min<long long>(b, (long long)g.sms * 8));
}

}  // namespace

void qr_solve_release() {
    qs_work.release();
    qs_s.release();
    qs_dag.reset();
    qs_key[4] = -1;
    ts_dag.reset();
    ts_key[3] = -1;
}

// z = F^-1 v in FP64 with F the Cholesky (alg 0) or no-pivot LU (alg 1) factors held in the
// first n / nb tile columns of W, an n x (n + nb) tile matrix whose last tile column is the
// right-hand-side workspace; v, z n x nrhs column-major (nrhs <= nb).  One persistent
// scheduler launch: forward then backward substitution tasks (build_trsolve_dag).
int fp64_trsolve(int alg, double *W, int n, int nb, const double *v, double *z, int nrhs, cudaStream_t s,
                 palial_status *st) {
    const int workers = g.sms;
    const int key[4] = {n, nb, nrhs, alg};
    if (!ts_dag || memcmp(key, ts_key, sizeof key) != 0) {
        try {
            auto d = std::make_shared<Dag>(build_trsolve_dag(n, nb, nrhs, alg));
            order_dag(*d, 0, workers, 0);
            d->uid = g.next_uid++;
            ts_dag = d;
            memcpy(ts_key, key, sizeof key);
        } catch (const std::exception &ex) {
            return set_status(st, PALIAL_ERR_ARG, "%s", ex.what());
        }
    }
    const std::shared_ptr<Dag> dag = ts_dag;
    SchedParams p;
    palial_opts o;
    palial_opts_default(&o);
    int rc = sched_prepare(g.main, dag, W, nullptr, workers, 0, o.timeout_s, p, st);
    if (rc) return rc;
    const int width = ((nrhs + 63) / 64) * 64;
    double *rhs = W + (size_t)n * n;
    note_launch();
    rhs_to_tiles_kernel<<<grid_for((long long)n * width), 256, 0, s>>>(v, rhs, n, nrhs, nb, width);
    PALIAL_CK(cudaGetLastError(), "pack right-hand sides");
    PALIAL_CK(sched_enqueue(g.main, p, dag->nobj, workers, true, s), "launch scheduler");
    note_launch();
    tiles_to_x_kernel<<<grid_for((long long)n * nrhs), 256, 0, s>>>(rhs, z, n, nrhs, nb);
    PALIAL_CK(cudaGetLastError(), "unpack solution");
    int code = 0;
    PALIAL_CK(cudaMemcpyAsync(&code, g.main.status.ptr, sizeof code, cudaMemcpyDeviceToHost, s), "status");
    PALIAL_CK(cudaStreamSynchronize(s), "triangular solve");
    if (code) return set_status(st, code, "FP64 triangular solve: device error %d", code);
    return PALIAL_OK;
}

}  // namespace palial

using namespace palial;

extern "C" int palial_gpu_qr_solve(int rows, int cols, int nb, const double *dA, const double *dB, double *dX,
                                   int nrhs, double *dResid, const palial_opts *opts, palial_status *st,
                                   void *stream) {
    palial_opts o;
    palial_opts_default(&o);
    if (opts) o = *opts;
    if (st) memset(st, 0, sizeof *st);
    if (nb <= 0 || nb % 64 || rows <= 0 || cols <= 0 || rows % nb || cols % nb || rows < cols)
        return set_status(st, PALIAL_ERR_ARG, "QR solve needs rows >= cols, both multiples of NB (multiple of 64)");
    if (nrhs < 1 || nrhs > nb) return set_status(st, PALIAL_ERR_ARG, "nrhs must be in [1, NB]");
    if (!dA || !dB || !dX) return set_status(st, PALIAL_ERR_ARG, "NULL buffer");
    int rc = ensure_init(st);
    if (rc) return rc;
    int sms = g.sms;
    if (o.max_sms > 0) sms = std::min(sms, o.max_sms);
    const int wps = o.workers_per_sm > 0 ? std::min(o.workers_per_sm, g.occupancy) : 1;
    const int workers = sms * wps;
    const int prio = o.priority == 1 ? 1 : 0;
    const int key[6] = {rows, cols, nb, nrhs, prio, workers};
    if (!qs_dag || memcmp(key, qs_key, sizeof key) != 0 || o.shuffle_seed) {
        try {
            auto d = std::make_shared<Dag>(build_qr_solve_dag(rows, cols, nb, nrhs));
            order_dag(*d, prio, workers, o.shuffle_seed);
            d->uid = g.next_uid++;
            qs_dag = d;
            memcpy(qs_key, key, sizeof key);
        } catch (const std::exception &ex) {
            return set_status(st, PALIAL_ERR_ARG, "%s", ex.what());
        }
    }
    const std::shared_ptr<Dag> dag = qs_dag;
    const int mt = rows / nb, nt = cols / nb;
    const size_t tile = (size_t)nb * nb;
    PALIAL_CK(qs_work.ensure(sizeof(double) * tile * (size_t)mt * (nt + 1)), "alloc QR solve work");
    PALIAL_CK(qs_s.ensure(sizeof(double) * tile * (size_t)mt * nt), "alloc QR solve T factors");
    double *W = qs_work.as<double>();
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    SchedParams p;
    rc = sched_prepare(g.main, dag, W, qs_s.as<double>(), workers, o.trace, o.timeout_s, p, st);
    if (rc) return rc;
    const int width = ((nrhs + 63) / 64) * 64;
    const auto w0 = std::chrono::steady_clock::now();
    PALIAL_CK(cudaEventRecord(g.ev0, s), "event");
    PALIAL_CK(cudaMemcpyAsync(W, dA, sizeof(double) * tile * (size_t)mt * nt, cudaMemcpyDeviceToDevice, s), "copy A");
    note_launch();
    rhs_to_tiles_kernel<<<grid_for((long long)rows * width), 256, 0, s>>>(dB, W + tile * (size_t)mt * nt, rows, nrhs,
                                                                          nb, width);
    PALIAL_CK(cudaGetLastError(), "pack B");
    PALIAL_CK(sched_enqueue(g.main, p, dag->nobj, workers, true, s), "launch scheduler");
    note_launch();
    tiles_to_x_kernel<<<grid_for((long long)cols * nrhs), 256, 0, s>>>(W + tile * (size_t)mt * nt, dX, cols, nrhs, nb);
    PALIAL_CK(cudaGetLastError(), "unpack X");
    if (dResid) {
        note_launch();
        ls_resid_kernel<<<nrhs, 256, 0, s>>>(W + tile * (size_t)mt * nt, dResid, rows, cols, nb);
        PALIAL_CK(cudaGetLastError(), "residual norms");
    }
    PALIAL_CK(cudaEventRecord(g.ev1, s), "event");
    PALIAL_CK(cudaEventSynchronize(g.ev1), "QR solve");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, g.ev0, g.ev1);
    int hs[ST_NSLOTS];
    PALIAL_CK(cudaMemcpy(hs, g.main.status.ptr, sizeof hs, cudaMemcpyDeviceToHost), "read status");
    if (o.trace && hs[ST_CODE] == 0) {
        g.last_trace.dag = *dag;
        g.last_trace_workers = workers;
        g.last_trace.recs.resize(dag->records.size());
        PALIAL_CK(cudaMemcpy(g.last_trace.recs.data(), g.main.trace.ptr, sizeof(TraceRec) * dag->records.size(),
                             cudaMemcpyDeviceToHost),
                  "read trace");
        g.last_trace.valid = true;
    }
    if (st) {
        const double m = rows, n = cols;
        st->ntasks = (long long)dag->records.size();
        st->seconds = ms * 1e-3;
        st->total_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - w0).count();
        // Householder QR of an m x n matrix: 2 m n^2 - 2 n^3 / 3 flops
        st->tflops = (2.0 * m * n * n - 2.0 * n * n * n / 3.0) / std::max(1e-12, st->seconds) * 1e-12;
        st->task = hs[ST_TASK];
    }
    if (hs[ST_CODE] == PALIAL_ERR_TIMEOUT)
        return set_status(st, PALIAL_ERR_TIMEOUT, "dependency wait timed out in task %d", hs[ST_TASK]);
    if (hs[ST_CODE] != 0) return set_status(st, hs[ST_CODE], "device error %d", hs[ST_CODE]);
    return set_status(st, PALIAL_OK);
}

// Host buffers: A rows x cols in tile layout, B rows x nrhs and X cols x nrhs column-major,
// resid (optional) nrhs doubles.
extern "C" int palial_gpu_qr_solve_host(int rows, int cols, int nb, const double *A, const double *B, double *X,
                                        int nrhs, double *resid, const palial_opts *opts, palial_status *st) {
    if (st) memset(st, 0, sizeof *st);
    if (!A || !B || !X || nrhs < 1 || rows <= 0 || cols <= 0) return set_status(st, PALIAL_ERR_ARG, "bad arguments");
    int rc = ensure_init(st);
    if (rc) return rc;
    const auto t0 = std::chrono::steady_clock::now();
    const size_t ab = sizeof(double) * (size_t)rows * cols, bb = sizeof(double) * (size_t)rows * nrhs,
                 xb = sizeof(double) * (size_t)cols * nrhs;
    PALIAL_CK(g.smat.ensure(ab + bb + xb + sizeof(double) * (size_t)nrhs), "alloc host-solve buffers");
    double *dA = g.smat.as<double>();
    double *dB = dA + (size_t)rows * cols, *dX = dB + (size_t)rows * nrhs, *dR = dX + (size_t)cols * nrhs;
    PALIAL_CK(cudaMemcpy(dA, A, ab, cudaMemcpyHostToDevice), "copy A");
    PALIAL_CK(cudaMemcpy(dB, B, bb, cudaMemcpyHostToDevice), "copy B");
    rc = palial_gpu_qr_solve(rows, cols, nb, dA, dB, dX, nrhs, resid ? dR : nullptr, opts, st, nullptr);
    if (rc < 0) return rc;
    PALIAL_CK(cudaMemcpy(X, dX, xb, cudaMemcpyDeviceToHost), "copy X");
    if (resid) PALIAL_CK(cudaMemcpy(resid, dR, sizeof(double) * nrhs, cudaMemcpyDeviceToHost), "copy residuals");
    if (st) st->total_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}
