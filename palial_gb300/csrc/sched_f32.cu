// sched_f32.cu -- FP32 tasks of the persistent scheduler: the tiled Cholesky (reference
// src/cholesky.h) and no-pivot LU (src/lu.h, src/srclu) of the batched mixed-precision solves,
// and the flat-tree TS QR (src/qr.h, src/srcqr) with its solve tasks for the mixed-precision QR
// solve of one matrix, run on FP32 copies of the matrices.
//
// Same dispatch as the FP64 scheduler (sched_f64.cu): one CTA = one worker, atomic ticket in
// the host's dispatch order, bounded acquire waits on the completion counters, fence and
// increment of the output objects, so each object's updates are applied in k order and the
// FP32 factors are identical under any schedule.  The tile routines are the FP32 CTA routines
// of tile_f32.cuh (64 x 64 CTA tiles, K chunks of 32, 64 x 64 substitutions with the unknowns
// in registers).  Differences from the FP64 tasks:
//  * a breakdown (non-positive Cholesky pivot, exact zero LU pivot) sets the matrix's flag in
//    mat_status and the launch goes on: the host refactors that matrix in FP64, the others are
//    unaffected (each matrix has its own buffer and counters);
//  * the Cholesky diagonal-block updates (POTRF trailing part, SYRK strips) also write the
//    entries below the diagonal of the 64 x 64 diagonal sub-blocks: nothing reads them (the
//    triangular solves of the refinement read the upper triangle only).
#include <cfloat>

#include "common.cuh"
#include "tile_f32.cuh"
#include "tile_qr.cuh"

namespace palial {
namespace sf32 {
using namespace f32;

// Dynamic shared memory (floats): Ds[64][65] | GEMM staging (the larger of the Cholesky/LU
// and the QR routines' needs) | QR reductions | QR tau
constexpr int SM_DS = 0;
constexpr int SM_G = 64 * DP + 4;  // 16-byte aligned staging (float4 stores)
constexpr int G_FLOATS = GEMM_SMEM_FLOATS > qrt::GEMM_SMEM ? GEMM_SMEM_FLOATS : qrt::GEMM_SMEM;
constexpr int SM_RED = SM_G + G_FLOATS;
constexpr int SM_TAU = SM_RED + qrt::RED;
constexpr int SMEM_BATCH = (SM_G + GEMM_SMEM_FLOATS) * 4;  // Cholesky / LU tasks
constexpr int SMEM_QR = (SM_TAU + qrt::MAX_NB) * 4;        // QR solve tasks
static_assert((SM_G * 4) % 16 == 0, "staging alignment");

struct Worker {
    float (*Ds)[DP];
    float *gsm;
    qrt::QrSmem<float> q;
};

__device__ __forceinline__ Worker make_worker(float *smem) {
    Worker w;
    w.Ds = reinterpret_cast<float (*)[DP]>(smem + SM_DS);
    w.gsm = smem + SM_G;
    w.q.gsm = smem + SM_G;
    w.q.red = smem + SM_RED;
    w.q.tau = smem + SM_TAU;
    return w;
}

// Unblocked upper Cholesky of the 64 x 64 block in Ds (upper triangle used).  Returns the
// first column with a non-positive pivot, or -1.  Uniform across the CTA.
__device__ int chol64_upper(float (*Ds)[DP]) {
    const int t = threadIdx.x;
    for (int j = 0; j < 64; j++) {
        const float d = Ds[j][j];
        if (!(d > 0.f)) return j;  // every thread reads the same Ds[j][j]
        const float rd = sqrtf(d);
        __syncthreads();
        // row j of U: U(j,c) = D(j,c)/rd for c > j; U(j,j) = rd
        if (t < 64) {
            if (t > j) Ds[t][j] = Ds[t][j] / rd;
            if (t == j) Ds[j][j] = rd;
        }
        __syncthreads();
        // trailing: D(r,c) -= U(j,r) U(j,c), j < r <= c
        for (int e = t; e < 64 * 64; e += NT) {
            const int r = e & 63, c = e >> 6;
            if (r > j && r <= c) Ds[c][r] = fmaf(-Ds[r][j], Ds[c][j], Ds[c][r]);
        }
        __syncthreads();
    }
    return -1;
}

// POTRF (upper) of an n x n block, n a multiple of 64, blocked by 64: the diagonal block in
// shared memory, the row panel by substitution, then the rank-64 update of the trailing block.
// Returns -1, or the first column with a non-positive pivot.
__device__ int potrf_upper(const Worker &w, float *A, int n, int ld) {
    for (int j0 = 0; j0 < n; j0 += 64) {
        float *D = A + j0 + (size_t)j0 * ld;
        load_diag64(w.Ds, D, ld);
        const int bad = chol64_upper(w.Ds);
        if (bad >= 0) return j0 + bad;
        for (int e = threadIdx.x; e < 4096; e += NT) {
            const int r = e & 63, c = e >> 6;
            if (r <= c) D[r + (size_t)c * ld] = w.Ds[c][r];
        }
        __syncthreads();
        if (j0 + 64 < n) {
            for (int c0 = j0 + 64; c0 < n; c0 += 64) solve64<0>(w.Ds, A + j0 + (size_t)c0 * ld, ld);
            const int m = n - j0 - 64;
            const float *X = A + j0 + (size_t)(j0 + 64) * ld;
            cta_gemm<true, false>(m, m, 64, -1.f, X, ld, X, ld, A + (j0 + 64) + (size_t)(j0 + 64) * ld, ld, w.gsm);
        }
    }
    return -1;
}

// GETRF without pivoting, the rule of reference src/srclu/dgetrf_no_pivot.h:11-57 in FP32
// (scale by the reciprocal pivot when |pivot| > FLT_MIN, divide otherwise, skip an exact
// zero), blocked by 64 columns: panel LU in global memory, U12 = L11^-1 A12 by substitution,
// A22 -= L21 U12.  Returns 1 if an exact zero pivot was met, else 0.
__device__ int getrf_nopiv(const Worker &w, float *A, int n, int ld) {
    int zero_piv = 0;
    for (int j0 = 0; j0 < n; j0 += 64) {
        for (int i = 0; i < 64; i++) {
            const int col = j0 + i;
            float *ccol = A + (size_t)col * ld;
            const float piv = ldg(ccol + col);
            if (piv != 0.f) {
                const bool recip = fabsf(piv) > FLT_MIN;
                const float rp = 1.f / piv;
                for (int r = col + 1 + threadIdx.x; r < n; r += NT)
                    ccol[r] = recip ? ldg(ccol + r) * rp : ldg(ccol + r) / piv;
            } else {
                zero_piv = 1;
            }
            __syncthreads();
            const int rows = n - col - 1, cols = j0 + 63 - col;
            // rank-1 update of the panel, 4 elements per thread per pass, loads before stores
            for (int e0 = threadIdx.x; e0 < rows * cols; e0 += 4 * NT) {
                float l[4], u[4], x[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int e = e0 + q * NT;
                    if (e < rows * cols) {
                        const int r = col + 1 + e % rows, c = col + 1 + e / rows;
                        l[q] = ldg(ccol + r);
                        u[q] = ldg(A + col + (size_t)c * ld);
                        x[q] = ldg(A + r + (size_t)c * ld);
                    }
                }
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int e = e0 + q * NT;
                    if (e < rows * cols) {
                        const int r = col + 1 + e % rows, c = col + 1 + e / rows;
                        A[r + (size_t)c * ld] = fmaf(-l[q], u[q], x[q]);
                    }
                }
            }
            __syncthreads();
        }
        float *D = A + j0 + (size_t)j0 * ld;
        load_diag64(w.Ds, D, ld);
        if (j0 + 64 < n) {
            for (int c0 = j0 + 64; c0 < n; c0 += 64) solve64<2>(w.Ds, A + j0 + (size_t)c0 * ld, ld);
            const int m = n - j0 - 64;
            cta_gemm<false, false>(m, m, 64, -1.f, A + (j0 + 64) + (size_t)j0 * ld, ld, A + j0 + (size_t)(j0 + 64) * ld,
                                   ld, A + (j0 + 64) + (size_t)(j0 + 64) * ld, ld, w.gsm);
        }
    }
    return zero_piv;
}

// Triangular solves on a 64-wide strip of an n x n block: GEMM updates from the solved
// 64-blocks, then substitution against the diagonal 64 x 64 block.
// X = U^-T B (U upper, B n x 64): row blocks top-down.
__device__ void trsm_lut(const Worker &w, const float *U, float *B, int n, int ld) {
    for (int rb = 0; rb < n; rb += 64) {
        if (rb > 0) cta_gemm<true, false>(64, 64, rb, -1.f, U + (size_t)rb * ld, ld, B, ld, B + rb, ld, w.gsm);
        load_diag64(w.Ds, U + rb + (size_t)rb * ld, ld);
        solve64<0>(w.Ds, B + rb, ld);
    }
}
// X = B U^-1 (B a 64 x n row strip): column blocks left to right.
__device__ void trsm_run(const Worker &w, const float *U, float *B, int n, int ld) {
    for (int cb = 0; cb < n; cb += 64) {
        if (cb > 0)
            cta_gemm<false, false>(64, 64, cb, -1.f, B, ld, U + (size_t)cb * ld, ld, B + (size_t)cb * ld, ld, w.gsm);
        load_diag64(w.Ds, U + cb + (size_t)cb * ld, ld);
        solve64<1>(w.Ds, B + (size_t)cb * ld, ld);
    }
}
// X = U^-1 B (U upper, B n x 64): row blocks bottom-up (the QR solve's back-substitution).
__device__ void trsm_lun(const Worker &w, const float *U, float *B, int n, int ld) {
    for (int rb = n - 64; rb >= 0; rb -= 64) {
        if (rb + 64 < n)
            cta_gemm<false, false>(64, 64, n - rb - 64, -1.f, U + rb + (size_t)(rb + 64) * ld, ld, B + rb + 64, ld,
                                   B + rb, ld, w.gsm);
        load_diag64(w.Ds, U + rb + (size_t)rb * ld, ld);
        solve64<3>(w.Ds, B + rb, ld);
    }
}
// X = L^-1 B (L unit lower, B n x 64): row blocks top-down.
__device__ void trsm_llu(const Worker &w, const float *L, float *B, int n, int ld) {
    for (int rb = 0; rb < n; rb += 64) {
        if (rb > 0) cta_gemm<false, false>(64, 64, rb, -1.f, L + rb, ld, B, ld, B + rb, ld, w.gsm);
        load_diag64(w.Ds, L + rb + (size_t)rb * ld, ld);
        solve64<2>(w.Ds, B + rb, ld);
    }
}

__device__ __forceinline__ float *fblock_ptr(float *A, int n, int nb, int bs, int bi, int bj) {
    const long long r0 = (long long)bi * bs, c0 = (long long)bj * bs;
    const long long tm = r0 / nb, tn = c0 / nb;
    const long long mt = n / nb;
    return A + (size_t)nb * nb * (size_t)(tm + mt * tn) + (size_t)(r0 % nb) + (size_t)(c0 % nb) * nb;
}

__device__ void record_error(const SchedParams &p, int code, int task, int m, int n, int col) {
    if (atomicCAS(p.status + ST_CODE, 0, code) == 0) {
        p.status[ST_TASK] = task;
        p.status[ST_M] = m;
        p.status[ST_N] = n;
        p.status[ST_COL] = col;
        __threadfence();
    }
}

__device__ __forceinline__ float *ftile_ptr(float *A, int n, int nb, int m, int k) {
    return A + (size_t)nb * nb * ((size_t)m + (size_t)(n / nb) * k);
}

// Batched Cholesky / LU tasks (p.mats, p.mat_status).
__device__ void run_task_batch(const SchedParams &p, const Worker &w, const Task &t, int tid) {
    const MatInfo mi = p.mats[t.mat];
    float *A = mi.Af;
    const int n = mi.n, nb = mi.nb, bs = mi.bs, ld = nb;
    const bool tc = mi.tc != 0;  // the update tasks' products on the tensor cores (BF16x3)
    switch (t.type) {
        case T_POTRF: {
            const int bad = potrf_upper(w, fblock_ptr(A, n, nb, bs, t.k, t.k), bs, ld);
            // the first breakdown (in k order: a later POTRF waits for this one) is kept
            if (bad >= 0 && threadIdx.x == 0) atomicCAS(p.mat_status + t.mat, 0, 1 + t.k * bs + bad);
            break;
        }
        case T_TRSM_LUT:
            trsm_lut(w, fblock_ptr(A, n, nb, bs, t.k, t.k), fblock_ptr(A, n, nb, bs, t.k, t.m) + (size_t)t.part * 64 * ld,
                     bs, ld);
            break;
        case T_SYRK: {
            const float *X = fblock_ptr(A, n, nb, bs, t.k, t.m);
            float *C = fblock_ptr(A, n, nb, bs, t.m, t.m);
            const int c0 = t.part * 64;
            if (tc)
                cta_gemm<true, false, false, true>(c0 + 64, 64, bs, -1.f, X, ld, X + (size_t)c0 * ld, ld, C + (size_t)c0 * ld,
                                                   ld, w.gsm);
            else
                cta_gemm<true, false>(c0 + 64, 64, bs, -1.f, X, ld, X + (size_t)c0 * ld, ld, C + (size_t)c0 * ld, ld, w.gsm);
            break;
        }
        case T_GEMM_TN: {
            const float *Xa = fblock_ptr(A, n, nb, bs, t.k, t.n);
            const float *Xb = fblock_ptr(A, n, nb, bs, t.k, t.m);
            float *C = fblock_ptr(A, n, nb, bs, t.n, t.m);
            const int c0 = t.part * 64;
            if (tc)
                cta_gemm<true, false, false, true>(bs, 64, bs, -1.f, Xa, ld, Xb + (size_t)c0 * ld, ld, C + (size_t)c0 * ld,
                                                   ld, w.gsm);
            else
                cta_gemm<true, false>(bs, 64, bs, -1.f, Xa, ld, Xb + (size_t)c0 * ld, ld, C + (size_t)c0 * ld, ld, w.gsm);
            break;
        }
        case T_GETRF: {
            const int z = getrf_nopiv(w, fblock_ptr(A, n, nb, bs, t.k, t.k), bs, ld);
            if (z && threadIdx.x == 0) atomicCAS(p.mat_status + t.mat, 0, 1);
            break;
        }
        case T_TRSM_RUN:
            trsm_run(w, fblock_ptr(A, n, nb, bs, t.k, t.k), fblock_ptr(A, n, nb, bs, t.m, t.k) + t.part * 64, bs, ld);
            break;
        case T_TRSM_LLU:
            trsm_llu(w, fblock_ptr(A, n, nb, bs, t.k, t.k), fblock_ptr(A, n, nb, bs, t.k, t.n) + (size_t)t.part * 64 * ld,
                     bs, ld);
            break;
        case T_GEMM_NN: {
            const float *Xa = fblock_ptr(A, n, nb, bs, t.m, t.k);
            const float *Xb = fblock_ptr(A, n, nb, bs, t.k, t.n);
            float *C = fblock_ptr(A, n, nb, bs, t.m, t.n);
            const int c0 = t.part * 64;
            if (tc)
                cta_gemm<false, false, false, true>(bs, 64, bs, -1.f, Xa, ld, Xb + (size_t)c0 * ld, ld, C + (size_t)c0 * ld,
                                                    ld, w.gsm);
            else
                cta_gemm<false, false>(bs, 64, bs, -1.f, Xa, ld, Xb + (size_t)c0 * ld, ld, C + (size_t)c0 * ld, ld, w.gsm);
            break;
        }
        default:
            if (threadIdx.x == 0) record_error(p, -2 /*PALIAL_ERR_ARG*/, tid, t.m, t.n, t.type);
            break;
    }
}

// QR factorization and QR solve tasks of one matrix (p.Af, T factors in p.Sf, two nb x 64
// scratch strips per worker in p.scratch_f), on NB tiles.
__device__ void run_task_qr(const SchedParams &p, const Worker &w, const Task &t, int tid) {
    float *A = p.Af;
    const int n = p.n, nb = p.nb, ld = nb;
    float *wscr = p.scratch_f + (size_t)blockIdx.x * (size_t)p.scratch_per_worker;
    switch (t.type) {
        case T_GEQRT:
            qrt::geqrt(w.q, ftile_ptr(A, n, nb, t.k, t.k), nb, ld, ftile_ptr(p.Sf, n, nb, t.k, t.k), ld, wscr);
            break;
        case T_UNMQR:
            qrt::unmqr_strip(w.q, ftile_ptr(A, n, nb, t.k, t.k), ftile_ptr(p.Sf, n, nb, t.k, t.k),
                             ftile_ptr(A, n, nb, t.k, t.n) + (size_t)t.part * 64 * ld, nb, ld, wscr,
                             wscr + (size_t)nb * 64);
            break;
        case T_TSQRT:
            qrt::tsqrt(w.q, ftile_ptr(A, n, nb, t.k, t.k), ftile_ptr(A, n, nb, t.m, t.k), nb, ld,
                       ftile_ptr(p.Sf, n, nb, t.m, t.k), ld, wscr);
            break;
        case T_TSMQR: {
            const size_t off = (size_t)t.part * 64 * ld;
            qrt::tsmqr_strip(w.q, ftile_ptr(A, n, nb, t.k, t.n) + off, ftile_ptr(A, n, nb, t.m, t.n) + off,
                             ftile_ptr(A, n, nb, t.m, t.k), ftile_ptr(p.Sf, n, nb, t.m, t.k), nb, ld, wscr,
                             wscr + (size_t)nb * 64, p.tc != 0);
            break;
        }
        case T_TRSM_LUN:  // R X = Y on the extra tile column
            trsm_lun(w, ftile_ptr(A, n, nb, t.k, t.k), ftile_ptr(A, n, nb, t.k, t.n) + (size_t)t.part * 64 * ld, nb, ld);
            break;
        case T_GEMM_NN: {  // Y_i -= R_ik X_k
            const int c0 = t.part * 64;
            cta_gemm<false, false>(nb, 64, nb, -1.f, ftile_ptr(A, n, nb, t.m, t.k), ld,
                                   ftile_ptr(A, n, nb, t.k, t.n) + (size_t)c0 * ld, ld,
                                   ftile_ptr(A, n, nb, t.m, t.n) + (size_t)c0 * ld, ld, w.gsm);
            break;
        }
        default:
            if (threadIdx.x == 0) record_error(p, -2 /*PALIAL_ERR_ARG*/, tid, t.m, t.n, t.type);
            break;
    }
}

// Persistent scheduler over FP32 matrices: a batch (QR = false: p.mats, p.mat_status;
// Cholesky and LU tasks, two workers per SM) or one matrix's QR factorization / QR solve
// (QR = true: p.Af, p.Sf, p.scratch_f; one worker per SM, registers for the reflectors).
template <bool QR>
__global__ void __launch_bounds__(NT, QR ? 1 : 2) sched_f32_kernel(SchedParams p) {
    extern __shared__ __align__(16) float smem[];
    Worker w = make_worker(smem);
    __shared__ int s_task, s_abort;
    for (;;) {
        if (threadIdx.x == 0) {
            int tk = p.ntasks;
            if (ld_volatile(p.status + ST_CODE) == 0) tk = (int)atomicAdd(p.ticket, 1u);
            s_task = tk;
            s_abort = 0;
        }
        __syncthreads();
        const int tid = s_task;
        if (tid >= p.ntasks) break;
        const Task t = p.tasks[tid];
        unsigned long long t0 = 0;
        if (threadIdx.x == 0) {
            const unsigned long long start = globaltimer_ns();
            for (int i = 0; i < t.nwait && !s_abort; i++) {
                const unsigned int *c = p.counters + t.wait_obj[i];
                const unsigned int target = t.wait_cnt[i];
                while (ld_acquire(c) < target) {
                    if (ld_volatile(p.status + ST_CODE) != 0) { s_abort = 1; break; }
                    if (globaltimer_ns() - start > p.timeout_ns) {
                        record_error(p, -4 /*PALIAL_ERR_TIMEOUT*/, tid, t.m, t.n, (int)t.wait_obj[i]);
                        s_abort = 1;
                        break;
                    }
                    __nanosleep(256);
                }
            }
            t0 = globaltimer_ns();
        }
        __syncthreads();
        if (s_abort) break;
        const long long c0 = clock64();
        if (QR) run_task_qr(p, w, t, tid);
        else run_task_batch(p, w, t, tid);
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            for (int i = 0; i < t.nsig; i++) atomicAdd(p.counters + t.sig_obj[i], 1u);
            if (p.trace) {
                TraceRec r;
                r.t0 = t0;
                r.t1 = globaltimer_ns();
                r.smid = smid();
                r.task = (unsigned)tid;
                r.clk = clock64() - c0;
                p.trace[tid] = r;
            }
        }
    }
}

// One whole FP32 QR tile task on one CTA, for the single-tile C ABI entry points (the
// reference's tile-kernel argument order): GEQRT (A, T), TSQRT (A1, A2, T), UNMQR (V, T, C),
// TSMQR (A1, A2, V, T); ld >= nb; scratch: two nb x 64 strips.
__global__ void __launch_bounds__(NT, 1) tile_qr_kernel(int type, int nb, int ld, float *p0, float *p1, float *p2,
                                                        float *p3, float *scratch) {
    extern __shared__ __align__(16) float smem[];
    Worker w = make_worker(smem);
    float *W = scratch, *W2 = scratch + (size_t)nb * 64;
    switch (type) {
        case T_GEQRT:
            qrt::geqrt(w.q, p0, nb, ld, p1, ld, scratch);
            break;
        case T_TSQRT:
            qrt::tsqrt(w.q, p0, p1, nb, ld, p2, ld, scratch);
            break;
        case T_UNMQR:
            for (int q = 0; q < nb / 64; q++) qrt::unmqr_strip(w.q, p0, p1, p2 + (size_t)q * 64 * ld, nb, ld, W, W2);
            break;
        case T_TSMQR:
            for (int q = 0; q < nb / 64; q++) {
                const size_t off = (size_t)q * 64 * ld;
                qrt::tsmqr_strip(w.q, p0 + off, p1 + off, p2, p3, nb, ld, W, W2);
            }
            break;
        default:
            break;
    }
}

}  // namespace sf32

cudaError_t sched32_configure() {
    cudaError_t e = cudaFuncSetAttribute(sf32::sched_f32_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         sf32::SMEM_BATCH);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(sf32::sched_f32_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 sf32::SMEM_QR);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(sf32::tile_qr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, sf32::SMEM_QR);
    return e;
}

cudaError_t tile_qr_f32_launch(int type, int nb, int ld, float *p0, float *p1, float *p2, float *p3, float *scratch,
                               cudaStream_t s) {
    note_launch();
    sf32::tile_qr_kernel<<<1, f32::NT, sf32::SMEM_QR, s>>>(type, nb, ld, p0, p1, p2, p3, scratch);
    return cudaGetLastError();
}

// resident CTAs per SM: the batched instance (qr = false) or the QR instance
int sched32_occupancy(bool qr) {
    int blocks = 0;
    if (qr)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, sf32::sched_f32_kernel<true>, f32::NT, sf32::SMEM_QR);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, sf32::sched_f32_kernel<false>, f32::NT,
                                                      sf32::SMEM_BATCH);
    return blocks;
}

// p.mats set: the batched Cholesky / LU instance; else the one-matrix QR instance
cudaError_t sched32_launch(const SchedParams &p, int grid, cudaStream_t s) {
    note_launch();
    if (p.mats) sf32::sched_f32_kernel<false><<<grid, f32::NT, sf32::SMEM_BATCH, s>>>(p);
    else sf32::sched_f32_kernel<true><<<grid, f32::NT, sf32::SMEM_QR, s>>>(p);
    return cudaGetLastError();
}

}  // namespace palial
