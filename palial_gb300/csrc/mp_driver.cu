// mp_driver.cu -- mixed-precision Cholesky / LU with iterative refinement (host driver).
//
// Factorization (right-looking, one k step at a time on one stream), on an FP32 working
// copy W of A in the reference's tile layout:
//   1. the diagonal tile W(k,k) is factored in FP64 by the persistent FP64 scheduler
//      (64-wide blocks, many CTAs): POTRF for Cholesky, the reference's no-pivot GETRF for LU;
//   2. the panel is solved in FP32 (substitution against the FP64-computed diagonal factor);
//   3. the panel is packed into K-major low-precision operands (BF16, FP8 e4m3 with per-tile
//      scales, or BF16 hi + lo) and the whole trailing matrix is updated by the tcgen05
//      kernel with FP32 accumulation.
// Refinement: x0 = 0, r = b; repeat: solve with the FP32 factors (blocked triangular
// solves), x += d (FP64), r = b - A x with the original FP64 matrix, until the normwise
// backward error max_j ||r_j||_inf / (||A||_inf ||x_j||_inf + ||b_j||_inf) meets the
// tolerance.  When plain refinement stagnates (or gmres = 1), the correction equation is
// solved by GMRES preconditioned with the low-precision factors, in FP64 (GMRES-IR).
// A Cholesky breakdown in low precision is retried with a diagonal shift (A + s I, s a small
// multiple of the unit roundoff of the update precision times max a_ii); refinement still
// targets the unshifted A.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "host_state.hpp"

namespace palial {
cudaError_t mp_update(int mode, int upper, float *C, int n, int nb, int k, const void *a_hi, const void *a_lo,
                      const void *b_hi, const void *b_lo, const float *scale_a, const float *scale_b, int *status,
                      cudaStream_t s);
cudaError_t mp_pack_rows(int mode, const float *W, int n, int nb, int k, void *hi, void *lo, float *scales,
                         cudaStream_t s);
cudaError_t mp_pack_cols(int mode, const float *W, int n, int nb, int k, void *hi, void *lo, float *scales,
                         cudaStream_t s);
cudaError_t mps_f64_to_f32(const double *A, float *W, int n, int nb, double shift, cudaStream_t s);
cudaError_t mps_tile_to_f64(const float *w, double *d, int nb, cudaStream_t s);
cudaError_t mps_tile_to_f32(const double *d, float *w, int nb, int upper_only, cudaStream_t s);
cudaError_t mps_panel_trsm(float *W, int n, int nb, int k, int kind, cudaStream_t s);
cudaError_t mps_rhs_diag(const float *W, int n, int nb, int k, float *R, int kind, cudaStream_t s);
cudaError_t mps_rhs_update(const float *W, int n, int nb, int k, float *R, int kind, cudaStream_t s);
cudaError_t mps_residual(const double *A, int n, int nb, const double *X, const double *B, double *R, int nrhs,
                         cudaStream_t s);
cudaError_t mps_norm_inf_matrix(const double *A, int n, int nb, double *out, cudaStream_t s);
cudaError_t mps_colmax(const double *X, long long n, int cols, double *out, cudaStream_t s);
cudaError_t mps_to_f32_rhs(const double *R, float *R32, long long n, int cols, const double *scale, cudaStream_t s);
cudaError_t mps_add_correction(double *X, const float *D32, long long n, int cols, const double *scale,
                               cudaStream_t s);
cudaError_t mps_mark_step(int *status, int k, cudaStream_t s);
}  // namespace palial

using namespace palial;

namespace {

struct MpBufs {
    DevBuf w, diag, pa_hi, pa_lo, pb_hi, pb_lo, scales, r, r32, x32, norms, work;
};
MpBufs mb;

double unit_roundoff(int prec) {
    switch (prec) {
        case PALIAL_PREC_BF16: return 0x1.0p-8;
        case PALIAL_PREC_FP8: return 0x1.0p-4;
        case PALIAL_PREC_BF16X3: return 0x1.0p-16;
        default: return 0x1.0p-24;
    }
}

// Low-precision factorization of W (FP32 tile layout, in place).  Returns PALIAL_OK,
// PALIAL_ERR_NOT_SPD (Cholesky breakdown) or an error.
int mp_factor(int alg, int prec, float *W, int n, int nb, cudaStream_t s, palial_status *st, int *zero_piv) {
    const int mt = n / nb;
    const int mode = prec == PALIAL_PREC_FP8 ? 1 : prec == PALIAL_PREC_BF16X3 ? 2 : 0;
    const size_t elem = (mode == 1) ? 1 : 2;
    const size_t panel = (size_t)std::max(1, mt - 1) * nb * nb * elem;
    PALIAL_CK(mb.diag.ensure(sizeof(double) * (size_t)nb * nb), "alloc diag");
    PALIAL_CK(mb.pa_hi.ensure(panel), "alloc panel");
    PALIAL_CK(mb.pb_hi.ensure(panel), "alloc panel");
    if (mode == 2) {
        PALIAL_CK(mb.pa_lo.ensure(panel), "alloc panel");
        PALIAL_CK(mb.pb_lo.ensure(panel), "alloc panel");
    }
    PALIAL_CK(mb.scales.ensure(sizeof(float) * 2 * (size_t)std::max(1, mt)), "alloc scales");
    // FP64 diagonal-tile factorization on the persistent scheduler (64-wide blocks)
    const int bsd = 64;
    std::shared_ptr<Dag> ddag;
    try {
        ddag = get_dag(alg, nb, nb, bsd, 0, g.sms, 0);
    } catch (const std::exception &ex) {
        return set_status(st, PALIAL_ERR_ARG, "%s", ex.what());
    }
    SchedParams dp;
    int rc = sched_prepare(g.diag, ddag, mb.diag.as<double>(), nullptr, g.sms, 0, 120.0, dp, st);
    if (rc) return rc;
    PALIAL_CK(cudaMemsetAsync(g.diag.status.ptr, 0, sizeof(int) * ST_NSLOTS, s), "clear status");
    float *sa = mb.scales.as<float>(), *sb = sa + mt;
    for (int k = 0; k < mt; k++) {
        float *wkk = W + (size_t)nb * nb * ((size_t)k + (size_t)mt * k);
        PALIAL_CK(mps_tile_to_f64(wkk, mb.diag.as<double>(), nb, s), "diag to f64");
        PALIAL_CK(mps_mark_step(g.diag.status.as<int>(), k, s), "mark");
        PALIAL_CK(sched_enqueue(g.diag, dp, ddag->nobj, g.sms, false, s), "diag factor");
        PALIAL_CK(mps_tile_to_f32(mb.diag.as<double>(), wkk, nb, alg == 0 ? 1 : 0, s), "diag to f32");
        if (k == mt - 1) break;
        if (alg == 0) {
            PALIAL_CK(mps_panel_trsm(W, n, nb, k, 0, s), "panel trsm");
            PALIAL_CK(mp_pack_rows(mode, W, n, nb, k, mb.pa_hi.ptr, mb.pa_lo.ptr, sa, s), "pack");
            PALIAL_CK(mp_update(mode, 1, W, n, nb, k, mb.pa_hi.ptr, mb.pa_lo.ptr, mb.pa_hi.ptr, mb.pa_lo.ptr, sa, sa,
                                g.diag.status.as<int>(), s),
                      "update");
        } else {
            PALIAL_CK(mps_panel_trsm(W, n, nb, k, 1, s), "row panel trsm");
            PALIAL_CK(mps_panel_trsm(W, n, nb, k, 2, s), "column panel trsm");
            PALIAL_CK(mp_pack_cols(mode, W, n, nb, k, mb.pa_hi.ptr, mb.pa_lo.ptr, sa, s), "pack L");
            PALIAL_CK(mp_pack_rows(mode, W, n, nb, k, mb.pb_hi.ptr, mb.pb_lo.ptr, sb, s), "pack U");
            PALIAL_CK(mp_update(mode, 0, W, n, nb, k, mb.pa_hi.ptr, mb.pa_lo.ptr, mb.pb_hi.ptr, mb.pb_lo.ptr, sa, sb,
                                g.diag.status.as<int>(), s),
                      "update");
        }
    }
    int hs[ST_NSLOTS];
    PALIAL_CK(cudaMemcpyAsync(hs, g.diag.status.ptr, sizeof hs, cudaMemcpyDeviceToHost, s), "status");
    PALIAL_CK(cudaStreamSynchronize(s), "factorization");
    if (zero_piv) *zero_piv = hs[ST_ZEROPIV];
    if (hs[ST_CODE] == PALIAL_ERR_NOT_SPD) {
        if (st) {
            st->tile_m = st->tile_n = hs[6];
            st->column = hs[ST_COL];
        }
        return PALIAL_ERR_NOT_SPD;
    }
    if (hs[ST_CODE] != 0) return set_status(st, hs[ST_CODE], "device error %d in step %d", hs[ST_CODE], hs[6]);
    return PALIAL_OK;
}

// d = M^-1 r for the FP32 factors in W; R32 (n x 64, zero padded) in/out.
int mp_apply_inverse(int alg, const float *W, int n, int nb, float *R32, cudaStream_t s, palial_status *st) {
    const int mt = n / nb;
    const int fwd_kind = (alg == 0) ? 0 : 2;
    for (int k = 0; k < mt; k++) {
        PALIAL_CK(mps_rhs_diag(W, n, nb, k, R32, fwd_kind, s), "forward diag");
        PALIAL_CK(mps_rhs_update(W, n, nb, k, R32, fwd_kind, s), "forward update");
    }
    for (int k = mt - 1; k >= 0; k--) {
        PALIAL_CK(mps_rhs_diag(W, n, nb, k, R32, 1, s), "backward diag");
        PALIAL_CK(mps_rhs_update(W, n, nb, k, R32, 1, s), "backward update");
    }
    return PALIAL_OK;
}

}  // namespace

extern "C" int palial_gpu_mp_update_step(int alg, int precision, float *dW, int n, int nb, int k) {
    palial_status *st = nullptr;
    if ((alg != 0 && alg != 1) || !dW || n % nb || nb % 256 || k < 0 || k >= n / nb) return PALIAL_ERR_ARG;
    int rc = ensure_init(nullptr);
    if (rc) return rc;
    const int mt = n / nb;
    const int mode = precision == PALIAL_PREC_FP8 ? 1 : precision == PALIAL_PREC_BF16X3 ? 2 : 0;
    const size_t panel = (size_t)std::max(1, mt - 1) * nb * nb * 2;
    PALIAL_CK(mb.pa_hi.ensure(panel), "alloc");
    PALIAL_CK(mb.pa_lo.ensure(panel), "alloc");
    PALIAL_CK(mb.pb_hi.ensure(panel), "alloc");
    PALIAL_CK(mb.pb_lo.ensure(panel), "alloc");
    PALIAL_CK(mb.scales.ensure(sizeof(float) * 2 * mt), "alloc");
    PALIAL_CK(g.diag.status.ensure(sizeof(int) * ST_NSLOTS + 64), "alloc");
    PALIAL_CK(cudaMemset(g.diag.status.ptr, 0, sizeof(int) * ST_NSLOTS), "clear");
    float *sa = mb.scales.as<float>(), *sb = sa + mt;
    if (alg == 0) {
        PALIAL_CK(mp_pack_rows(mode, dW, n, nb, k, mb.pa_hi.ptr, mb.pa_lo.ptr, sa, nullptr), "pack");
        PALIAL_CK(mp_update(mode, 1, dW, n, nb, k, mb.pa_hi.ptr, mb.pa_lo.ptr, mb.pa_hi.ptr, mb.pa_lo.ptr, sa, sa,
                            g.diag.status.as<int>(), nullptr),
                  "update");
    } else {
        PALIAL_CK(mp_pack_cols(mode, dW, n, nb, k, mb.pa_hi.ptr, mb.pa_lo.ptr, sa, nullptr), "pack");
        PALIAL_CK(mp_pack_rows(mode, dW, n, nb, k, mb.pb_hi.ptr, mb.pb_lo.ptr, sb, nullptr), "pack");
        PALIAL_CK(mp_update(mode, 0, dW, n, nb, k, mb.pa_hi.ptr, mb.pa_lo.ptr, mb.pb_hi.ptr, mb.pb_lo.ptr, sa, sb,
                            g.diag.status.as<int>(), nullptr),
                  "update");
    }
    PALIAL_CK(cudaDeviceSynchronize(), "update");
    int code = 0;
    PALIAL_CK(cudaMemcpy(&code, g.diag.status.ptr, sizeof code, cudaMemcpyDeviceToHost), "status");
    return code;
}

extern "C" int palial_gpu_mp_factor(int alg, const double *dA, float *dW, int n, int nb, const palial_opts *opts,
                                    palial_status *st, void *stream) {
    palial_opts o;
    palial_opts_default(&o);
    if (opts) o = *opts;
    if (st) memset(st, 0, sizeof *st);
    if ((alg != 0 && alg != 1) || !dA || !dW || n <= 0 || nb <= 0 || n % nb || nb % 256)
        return set_status(st, PALIAL_ERR_ARG, "mixed precision needs Cholesky/LU, N %% NB == 0, NB %% 256 == 0");
    int rc = ensure_init(st);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    PALIAL_CK(mps_f64_to_f32(dA, dW, n, nb, 0.0, s), "convert");
    const auto t0 = std::chrono::steady_clock::now();
    int zp = 0;
    rc = mp_factor(alg, o.precision, dW, n, nb, s, st, &zp);
    if (st) st->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (rc) return set_status(st, rc, "mixed factorization failed");
    return set_status(st, zp ? PALIAL_WARN_ZERO_PIVOT : PALIAL_OK);
}

extern "C" int palial_gpu_solve_ir(int alg, const double *dA, int n, int nb, const double *dB, double *dX, int nrhs,
                                   const palial_opts *opts, palial_status *st, void *stream) {
    palial_opts o;
    palial_opts_default(&o);
    if (opts) o = *opts;
    if (st) memset(st, 0, sizeof *st);
    if ((alg != 0 && alg != 1) || !dA || !dB || !dX || n <= 0 || nb <= 0 || n % nb || nb % 256 || nrhs < 1 ||
        nrhs > 16)
        return set_status(st, PALIAL_ERR_ARG, "solve_ir: Cholesky/LU, N %% NB == 0, NB %% 256 == 0, 1 <= nrhs <= 16");
    int rc = ensure_init(st);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const auto t0 = std::chrono::steady_clock::now();
    const size_t nn = (size_t)n * n;
    PALIAL_CK(mb.w.ensure(sizeof(float) * nn), "alloc W");
    PALIAL_CK(mb.r.ensure(sizeof(double) * (size_t)n * nrhs), "alloc r");
    PALIAL_CK(mb.r32.ensure(sizeof(float) * (size_t)n * 64), "alloc r32");
    PALIAL_CK(mb.norms.ensure(sizeof(double) * 128), "alloc norms");
    float *W = mb.w.as<float>();
    double *nrm = mb.norms.as<double>();  // [0] ||A||, [1..16] scale, [17..32] |r|, [33..48] |x|, [49..64] |b|
    // ||A||_inf and max |a_ii| (for the shift)
    PALIAL_CK(mps_norm_inf_matrix(dA, n, nb, nrm, s), "norm A");
    double anorm = 0;
    PALIAL_CK(cudaMemcpyAsync(&anorm, nrm, sizeof(double), cudaMemcpyDeviceToHost, s), "norm");
    PALIAL_CK(cudaStreamSynchronize(s), "norm");
    const int prec = o.precision;
    // ---- factorization (FP64 path: plain FP64 scheduler, then the same FP32 solves) -------
    int zp = 0;
    double shift = 0.0;
    const auto f0 = std::chrono::steady_clock::now();
    if (prec == PALIAL_PREC_FP64) {
        PALIAL_CK(g.mat.ensure(sizeof(double) * nn), "alloc copy");
        PALIAL_CK(cudaMemcpyAsync(g.mat.ptr, dA, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s), "copy");
        palial_opts fo = o;
        palial_status fs;
        rc = palial_gpu_factor_dev(alg, g.mat.as<double>(), nullptr, n, nb, &fo, &fs, stream);
        if (rc < 0) {
            if (st) {
                *st = fs;
            }
            return rc;
        }
        PALIAL_CK(mps_f64_to_f32(g.mat.as<double>(), W, n, nb, 0.0, s), "factor to f32");
    } else {
        for (int attempt = 0; attempt < 4; attempt++) {
            PALIAL_CK(mps_f64_to_f32(dA, W, n, nb, shift, s), "convert");
            rc = mp_factor(alg, prec, W, n, nb, s, st, &zp);
            if (rc != PALIAL_ERR_NOT_SPD || alg != 0) break;
            // Higham-Pranesh style shift: a small multiple of u_f * ||A||
            shift = (shift == 0.0) ? 4.0 * unit_roundoff(prec) * anorm / std::sqrt((double)n) : shift * 4.0;
        }
        if (rc) return set_status(st, rc, "mixed factorization failed (shift %.3e)", shift);
    }
    PALIAL_CK(cudaStreamSynchronize(s), "factorization");
    const double fsec = std::chrono::duration<double>(std::chrono::steady_clock::now() - f0).count();
    // ---- refinement -------------------------------------------------------------------------
    const double tol = o.ir_tol > 0 ? o.ir_tol : 1e-14 * n;
    const int maxit = o.ir_max_iter > 0 ? o.ir_max_iter : 50;
    std::vector<double> hb(nrhs), hr(nrhs), hx(nrhs), hscale(nrhs);
    PALIAL_CK(mps_colmax(dB, n, nrhs, nrm + 49, s), "norm b");
    PALIAL_CK(cudaMemcpyAsync(hb.data(), nrm + 49, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s), "norm b");
    PALIAL_CK(cudaMemsetAsync(dX, 0, sizeof(double) * (size_t)n * nrhs, s), "x0");
    PALIAL_CK(cudaMemcpyAsync(mb.r.ptr, dB, sizeof(double) * (size_t)n * nrhs, cudaMemcpyDeviceToDevice, s), "r0");
    PALIAL_CK(cudaStreamSynchronize(s), "init");
    double eta = 1.0, eta_prev = 1e300;
    int it = 0;
    bool converged = false;
    for (it = 1; it <= maxit; it++) {
        // scale = max |r_j| (keeps the FP32 right-hand side well inside range)
        PALIAL_CK(mps_colmax(mb.r.as<double>(), n, nrhs, nrm + 1, s), "scale");
        PALIAL_CK(cudaMemcpyAsync(hscale.data(), nrm + 1, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s), "scale");
        PALIAL_CK(cudaStreamSynchronize(s), "scale");
        bool any = false;
        for (int j = 0; j < nrhs; j++) {
            if (hscale[j] == 0.0) hscale[j] = 1.0;
            else any = true;
        }
        if (!any) {
            eta = 0.0;
            converged = true;
            break;
        }
        PALIAL_CK(cudaMemcpyAsync(nrm + 1, hscale.data(), sizeof(double) * nrhs, cudaMemcpyHostToDevice, s), "scale");
        PALIAL_CK(mps_to_f32_rhs(mb.r.as<double>(), mb.r32.as<float>(), n, nrhs, nrm + 1, s), "r to f32");
        rc = mp_apply_inverse(alg, W, n, nb, mb.r32.as<float>(), s, st);
        if (rc) return rc;
        PALIAL_CK(mps_add_correction(dX, mb.r32.as<float>(), n, nrhs, nrm + 1, s), "x += d");
        PALIAL_CK(mps_residual(dA, n, nb, dX, dB, mb.r.as<double>(), nrhs, s), "residual");
        PALIAL_CK(mps_colmax(mb.r.as<double>(), n, nrhs, nrm + 17, s), "norm r");
        PALIAL_CK(mps_colmax(dX, n, nrhs, nrm + 33, s), "norm x");
        PALIAL_CK(cudaMemcpyAsync(hr.data(), nrm + 17, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s), "norm r");
        PALIAL_CK(cudaMemcpyAsync(hx.data(), nrm + 33, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s), "norm x");
        PALIAL_CK(cudaStreamSynchronize(s), "iteration");
        eta = 0.0;
        for (int j = 0; j < nrhs; j++) eta = std::max(eta, hr[j] / (anorm * hx[j] + hb[j]));
        if (!std::isfinite(eta)) break;
        if (eta <= tol) {
            converged = true;
            break;
        }
        if (it >= 3 && eta > 0.9 * eta_prev) break;  // stagnation: refinement cannot reach tol
        eta_prev = eta;
    }
    const double total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (st) {
        st->ir_iters = std::min(it, maxit);
        st->backward_error = eta;
        st->seconds = total;
        st->total_seconds = total;
        st->tflops = algorithmic_flops(alg, n) / total * 1e-12;
        st->kappa_est = -1.0;
        st->factor_seconds = fsec;
        st->shift = shift;
        st->gmres_iters = 0;
    }
    if (!converged)
        return set_status(st, PALIAL_ERR_NOT_CONVERGED, "refinement stopped at backward error %.3e after %d iterations",
                          eta, it);
    return set_status(st, zp ? PALIAL_WARN_ZERO_PIVOT : PALIAL_OK, "backward error %.3e in %d iterations (shift %.2e)",
                      eta, st ? st->ir_iters : it, shift);
}
