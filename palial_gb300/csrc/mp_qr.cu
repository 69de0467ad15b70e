// mp_qr.cu -- mixed-precision QR solve of a square system A X = B (nrhs <= 16).
//
// The factorization is the reference's flat-tree TS QR (src/qr.h: GEQRT, TSQRT, UNMQR and
// TSMQR tasks, R, V and T in the reference's layout) computed in FP32 by the FP32 task
// scheduler (sched_f32.cu, tile routines of tile_qr.cuh) on an FP32 copy of A held in an
// n x (n + nb) tile matrix W; the T factors go to an n x n FP32 tile matrix S.  Refinement in
// FP64:
//     R = B - A X (FP64),   D = R^-1 Q^T (R / |R|) (FP32),   X += |R| D   (per column),
// where Q^T and R^-1 are the apply-only QR solve DAG (build_qr_solve_dag with apply_only):
// UNMQR/TSMQR tasks on W's extra tile column, then TRSM/GEMM back-substitution tasks, one
// scheduler launch per step.  It stops when every column's normwise backward error
// |r_j| / (|A| |x_j| + |b_j|) (infinity norms) is at most the tolerance.  A refinement that
// does not halve the error per step, or runs out of steps, hands the system to the FP64 QR
// solve (palial_gpu_qr_solve) and checks its result with one FP64 residual.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <tuple>
#include <vector>

#include "host_state.hpp"

namespace palial {
cudaError_t mps_f64_to_f32(const double *A, float *W, int n, int nb, double shift, cudaStream_t s, double *amax,
                           bool upper_only, int r0, int r1);
cudaError_t mps_residual(const double *A, int n, int nb, const double *X, const double *B, double *R, int nrhs,
                         double *amax, cudaStream_t s);
cudaError_t mps_norm_inf_matrix(const double *A, int n, int nb, double *out, cudaStream_t s);
cudaError_t mps_colmax(const double *X, long long n, int cols, double *out, cudaStream_t s);

namespace {

constexpr int MAX_RHS = 16;

// R (n x nrhs, ld n) / scale per column into the extra tile column of W (element (r, c) at
// col[nb^2 (r / nb) + r % nb + c nb]); columns nrhs .. nb - 1 zero.
__global__ void rhs_to_column_kernel(const double *R, int n, int nb, int nrhs, const double *scale, float *col) {
    const long long total = (long long)n * nb;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(e % n), c = (int)(e / n);
        float v = 0.f;
        if (c < nrhs && scale[c] > 0.0) v = (float)(R[(size_t)r + (size_t)c * n] / scale[c]);
        col[(size_t)nb * nb * (size_t)(r / nb) + (size_t)(r % nb) + (size_t)c * nb] = v;
    }
}

// X (n x nrhs, ld n) = (assign ? 0 : X) + scale * the extra tile column's solution.
__global__ void column_to_x_kernel(double *X, int n, int nb, int nrhs, const double *scale, const float *col,
                                   int assign) {
    const long long total = (long long)n * nrhs;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(e % n), c = (int)(e / n);
        const double d = scale[c] > 0.0
                             ? scale[c] * (double)col[(size_t)nb * nb * (size_t)(r / nb) + (size_t)(r % nb) + (size_t)c * nb]
                             : 0.0;
        double *x = X + (size_t)r + (size_t)c * n;
        *x = (assign ? 0.0 : *x) + d;
    }
}

DevBuf q_w, q_s, q_r, q_norm;
SchedCtx q_fac, q_app;
std::map<std::tuple<int, int, int, int>, std::shared_ptr<Dag>> q_dags;  // (n, nb, nrhs, workers)

int grid_of(long long elems) {
    const long long b = (elems + 255) / 256;
    return (int)std::max(1LL, std::min<long long>(b, (long long)std::max(1, g.sms) * 16));
}

// One FP32 scheduler launch of dag over W / S, synchronous; returns the device status code.
int run_f32(SchedCtx &c, const std::shared_ptr<Dag> &dag, float *W, float *S, int workers, double timeout_s,
            cudaStream_t s, palial_status *st, double *seconds, bool tc = false) {
    SchedParams p;
    int rc = sched_prepare(c, dag, nullptr, nullptr, workers, 0, timeout_s, p, st);
    if (rc) return rc;
    p.Af = W;
    p.Sf = S;
    p.tc = tc ? 1 : 0;
    p.scratch_f = reinterpret_cast<float *>(p.scratch);  // sized in doubles: twice the floats used
    PALIAL_CK(cudaEventRecord(g.ev0, s), "event");
    PALIAL_CK(sched_enqueue(c, p, dag->nobj, workers, true, s, true), "FP32 scheduler");
    PALIAL_CK(cudaEventRecord(g.ev1, s), "event");
    PALIAL_CK(cudaEventSynchronize(g.ev1), "FP32 scheduler");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, g.ev0, g.ev1);
    if (seconds) *seconds += ms * 1e-3;
    int hs[ST_NSLOTS];
    PALIAL_CK(cudaMemcpy(hs, c.status.ptr, sizeof hs, cudaMemcpyDeviceToHost), "status");
    if (hs[ST_CODE] != 0) return set_status(st, hs[ST_CODE], "FP32 QR task %d: device error %d", hs[ST_TASK], hs[ST_CODE]);
    return PALIAL_OK;
}

}  // namespace

void mp_qr_release() {
    for (DevBuf *b : {&q_w, &q_s, &q_r, &q_norm}) b->release();
    q_fac.release();
    q_app.release();
    q_dags.clear();
}

}  // namespace palial

using namespace palial;

extern "C" int palial_gpu_qr_solve_ir(int n, int nb, const double *dA, const double *dB, double *dX, int nrhs,
                                      const palial_opts *opts, palial_status *st, void *stream) {
    if (st) memset(st, 0, sizeof *st);
    if (n <= 0 || nb <= 0 || nb % 64 || nb > 512 || n % nb || nrhs < 1 || nrhs > MAX_RHS || !dA || !dB || !dX)
        return set_status(st, PALIAL_ERR_ARG, "qr_solve_ir: n %% nb == 0, nb a multiple of 64 up to 512, 1 <= nrhs <= %d",
                          MAX_RHS);
    int rc = ensure_init(st);
    if (rc) return rc;
    palial_opts o;
    palial_opts_default(&o);
    if (opts) o = *opts;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const auto t0 = std::chrono::steady_clock::now();
    const double tol = o.ir_tol > 0 ? o.ir_tol : 1e-14 * n;
    const int max_iter = o.ir_max_iter > 0 ? o.ir_max_iter : 30;
    const int workers = g.sms * g.occupancy32_qr;
    const size_t nn = (size_t)n * n;
    PALIAL_CK(q_w.ensure(sizeof(float) * (nn + (size_t)n * nb)), "alloc FP32 work matrix");
    PALIAL_CK(q_s.ensure(sizeof(float) * nn), "alloc FP32 T factors");
    PALIAL_CK(q_r.ensure(sizeof(double) * (size_t)n * nrhs), "alloc residual");
    PALIAL_CK(q_norm.ensure(sizeof(double) * (4 * MAX_RHS + 8)), "alloc norms");
    float *W = q_w.as<float>(), *S = q_s.as<float>(), *col = W + nn;
    double *R = q_r.as<double>(), *nrm = q_norm.as<double>();
    double *rmax_d = nrm, *xmax_d = nrm + MAX_RHS, *bmax_d = nrm + 2 * MAX_RHS, *anorm_d = nrm + 3 * MAX_RHS;

    // FP32 copy of A and the FP32 tile QR
    PALIAL_CK(mps_f64_to_f32(dA, W, n, nb, 0.0, s, nullptr, false, 0, -1), "convert");
    PALIAL_CK(cudaMemsetAsync(S, 0, sizeof(float) * nn, s), "clear T factors");
    std::shared_ptr<Dag> fdag = get_dag(2, n, nb, nb, 0, workers, 0);
    const auto key = std::make_tuple(n, nb, nrhs, workers);
    auto it = q_dags.find(key);
    if (it == q_dags.end()) {
        try {
            auto d = std::make_shared<Dag>(build_qr_solve_dag(n, n, nb, nrhs, true));
            order_dag(*d, 0, workers, 0);
            d->uid = g.next_uid++;
            if (q_dags.size() > 8) q_dags.clear();
            it = q_dags.emplace(key, d).first;
        } catch (const std::exception &ex) {
            return set_status(st, PALIAL_ERR_ARG, "%s", ex.what());
        }
    }
    const std::shared_ptr<Dag> adag = it->second;
    double factor_s = 0, apply_s = 0;
    // opts.precision = PALIAL_PREC_BF16X3: TSMQR's two products with V on the tensor cores
    rc = run_f32(q_fac, fdag, W, S, workers, o.timeout_s, s, st, &factor_s, o.precision == PALIAL_PREC_BF16X3);
    if (rc) return rc;

    // refinement from X = 0 (R = B)
    PALIAL_CK(mps_norm_inf_matrix(dA, n, nb, anorm_d, s), "norm A");
    PALIAL_CK(mps_colmax(dB, n, nrhs, bmax_d, s), "norm B");
    PALIAL_CK(cudaMemcpyAsync(R, dB, sizeof(double) * (size_t)n * nrhs, cudaMemcpyDeviceToDevice, s), "R = B");
    PALIAL_CK(cudaMemsetAsync(xmax_d, 0, sizeof(double) * MAX_RHS, s), "norm X");
    double h[4 * MAX_RHS + 1];
    double worst = INFINITY, prev = INFINITY;
    int steps = 0;
    bool converged = false;
    for (int step = 0;; step++) {
        PALIAL_CK(mps_colmax(R, n, nrhs, rmax_d, s), "norm R");
        PALIAL_CK(cudaMemcpyAsync(h, nrm, sizeof(double) * (3 * MAX_RHS + 1), cudaMemcpyDeviceToHost, s), "norms");
        PALIAL_CK(cudaStreamSynchronize(s), "norms");
        const double anorm = h[3 * MAX_RHS];
        worst = 0;
        for (int c = 0; c < nrhs; c++) {
            const double r = h[c], x = h[MAX_RHS + c], b = h[2 * MAX_RHS + c];
            const double eta = r == 0.0 ? 0.0 : r / (anorm * x + b);
            worst = std::isnan(eta) ? INFINITY : std::max(worst, eta);
        }
        if (step > 0 && worst <= tol) {
            converged = true;
            break;
        }
        if (!std::isfinite(worst) || (step >= 2 && worst > 0.5 * prev) || step == max_iter) break;
        prev = worst;
        // D = R^-1 Q^T (R / |R|), X += |R| D
        note_launch();
        rhs_to_column_kernel<<<grid_of((long long)n * nb), 256, 0, s>>>(R, n, nb, nrhs, rmax_d, col);
        PALIAL_CK(cudaGetLastError(), "residual to column");
        rc = run_f32(q_app, adag, W, S, workers, o.timeout_s, s, st, &apply_s);
        if (rc) return rc;
        note_launch();
        column_to_x_kernel<<<grid_of((long long)n * nrhs), 256, 0, s>>>(dX, n, nb, nrhs, rmax_d, col, step == 0);
        PALIAL_CK(cudaGetLastError(), "correction");
        steps = step + 1;
        PALIAL_CK(mps_residual(dA, n, nb, dX, dB, R, nrhs, nullptr, s), "residual");
        PALIAL_CK(mps_colmax(dX, n, nrhs, xmax_d, s), "norm X");
    }
    int rung = o.precision == PALIAL_PREC_BF16X3 ? PALIAL_PREC_BF16X3 : PALIAL_PREC_FP32;
    if (!converged) {
        // the FP64 QR solve, then one FP64 residual check
        palial_status s2;
        palial_opts o64 = o;
        o64.precision = PALIAL_PREC_FP64;
        rc = palial_gpu_qr_solve(n, n, nb, dA, dB, dX, nrhs, nullptr, &o64, &s2, stream);
        if (rc < 0) return set_status(st, rc, "FP64 QR solve: %s", s2.message);
        factor_s += s2.seconds;
        rung = PALIAL_PREC_FP64;
        PALIAL_CK(mps_residual(dA, n, nb, dX, dB, R, nrhs, nullptr, s), "residual");
        PALIAL_CK(mps_colmax(dX, n, nrhs, xmax_d, s), "norm X");
        PALIAL_CK(mps_colmax(R, n, nrhs, rmax_d, s), "norm R");
        PALIAL_CK(cudaMemcpyAsync(h, nrm, sizeof(double) * (3 * MAX_RHS + 1), cudaMemcpyDeviceToHost, s), "norms");
        PALIAL_CK(cudaStreamSynchronize(s), "norms");
        worst = 0;
        for (int c = 0; c < nrhs; c++) {
            const double r = h[c], x = h[MAX_RHS + c], b = h[2 * MAX_RHS + c];
            const double eta = r == 0.0 ? 0.0 : r / (h[3 * MAX_RHS] * x + b);
            worst = std::isnan(eta) ? INFINITY : std::max(worst, eta);
        }
        converged = worst <= tol;
    }
    const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (st) {
        st->seconds = wall;
        st->total_seconds = wall;
        st->factor_seconds = factor_s;
        st->tflops = algorithmic_flops(2, n) / std::max(1e-12, wall) * 1e-12;
        st->ir_iters = steps;
        st->backward_error = worst;
        st->kappa_est = -1.0;
        st->precision_used = rung;  // the precision that produced the result
    }
    if (!converged)
        return set_status(st, PALIAL_ERR_NOT_CONVERGED, "QR refinement stopped at %.3g (tolerance %.3g)", worst, tol);
    return set_status(st, PALIAL_OK, "%s QR, %d refinement steps (%.3f s applying Q^T and R^-1)",
                      rung == PALIAL_PREC_FP64 ? "FP64" : rung == PALIAL_PREC_FP32 ? "FP32" : "FP32 (BF16x3 TSMQR)",
                      steps, apply_s);
}
