// mp_diag.cu -- FP32 factorization of one diagonal tile of the mixed-precision path, in one
// CTA, in place on the FP32 working copy.
//
// The mixed-precision factorization keeps its working copy in FP32 and its trailing updates in
// BF16/FP8, so the diagonal tiles need FP32 accuracy, not FP64; and FP32 runs 64 times faster
// per SM than FP64 on this part.  The tile (nb x nb, column-major, ld = nb, nb a multiple of
// 64 up to 1024) is factored right-looking in 64-column steps:
//   1. the 64 x 64 diagonal block in shared memory (Cholesky: U^T U, upper; LU: no pivoting
//      with the reference's pivot rule, src/srclu/dgetrf_no_pivot.h:11-57: scale by the
//      reciprocal when |pivot| > FLT_MIN, divide otherwise, skip an exact zero);
//   2. the panel(s) by substitution, one thread per column (or row), the 64 unknowns in
//      registers: Cholesky U12 = U11^-T A12; LU U12 = L11^-1 A12 and L21 = A21 U11^-1;
//   3. the trailing block by a register-tiled (8 x 8 per thread) product from panel chunks
//      staged in shared memory: Cholesky A22 -= U12^T U12 (upper triangle only), LU
//      A22 -= L21 U12.
// Errors go to the status words of the factorization: a non-positive Cholesky pivot records
// PALIAL_ERR_NOT_SPD with the step and column; an exact zero LU pivot sets the zero-pivot
// flag.  A CTA that finds an error already recorded does nothing.
#include <cuda_runtime.h>

#include <cfloat>

#include "common.cuh"

namespace palial {
namespace mpd {

constexpr int NT = 512;   // threads (chol64/getrf64 map 8 threads per column of the 64 x 64 block)
constexpr int DP = 65;    // padded leading dimension of the 64 x 64 block in shared memory
constexpr int MT = 8;     // micro-tile edge
constexpr int PP = 65;    // pitch of the staged panel columns

__host__ __device__ constexpr int chunk_k(int nb) { return nb <= 512 ? 32 : 16; }
// staging area after Ds (floats): two chunks of chunk_k x (nb - 64) for the trailing update, and
// for nb <= 512 room for the whole panel (nb - 64 columns at pitch PP) so that its columns are
// solved in one pass
__host__ __device__ constexpr int stage_floats(int nb) {
    return (nb <= 512 && (nb - 64) * PP > 2 * chunk_k(nb) * (nb - 64)) ? (nb - 64) * PP : 2 * chunk_k(nb) * (nb - 64);
}
// shared memory (floats): Ds[64][65] + the staging area + a flag word
__host__ __device__ constexpr int smem_floats(int nb) { return 64 * DP + stage_floats(nb) + 64; }

// ---- 64 x 64 diagonal block in shared memory ---------------------------------------------
// Ds[c][r] = A(r, c).  Blocked by 16: the 16 x 16 diagonal block is factored by warp 0 in
// registers (lane l < 16 holds its column; pivots and factor rows broadcast by shuffles), then
// the 16-row panel(s) by substitution and the rank-16 update of the rest of the block by all
// threads (thread t: column q = t / 8, rows i = t % 8 + 8 j).
constexpr unsigned FULL = 0xffffffffu;

// Cholesky of the 16 x 16 block at (c0, c0) by warp 0: lane l < 16 keeps column c0 + l in
// registers (rows c0 .. c0 + 15); the pivot and the factor row U(p, .) travel by shuffles.  The
// arithmetic per entry is that of a shared-memory sweep: U(p, l) = a(p, l) * rsqrt(d), U(p, p) =
// d * rsqrt(d), a(i, l) = fma(-U(p, i), U(p, l), a(i, l)) for p < i <= l.  The pivot steps are
// template-unrolled so that the column stays in registers.
template <int P>
__device__ __forceinline__ void chol16_pivot(float (&c)[16], int lc, int &fail) {
    if constexpr (P < 16) {
        const float d = __shfl_sync(FULL, c[P], P);
        if (!(d > 0.f) && fail < 0) fail = P;
        const float ri = rsqrtf(d);
        c[P] = lc > P ? c[P] * ri : (lc == P ? d * ri : c[P]);
        const float u = c[P];
#pragma unroll
        for (int i = P + 1; i < 16; i++) {
            const float upi = __shfl_sync(FULL, c[P], i);  // U(P, i) from lane i
            if (i <= lc) c[i] = fmaf(-upi, u, c[i]);
        }
        chol16_pivot<P + 1>(c, lc, fail);
    }
}

// Returns the first failing pivot or -1 (warp-uniform).
__device__ __forceinline__ int chol16_warp(float (*Ds)[DP], int c0) {
    const int l = threadIdx.x & 31, lc = l & 15;
    float *col = &Ds[c0 + lc][c0];
    float c[16];
#pragma unroll
    for (int i = 0; i < 16; i++) c[i] = col[i];
    int fail = -1;
    chol16_pivot<0>(c, lc, fail);
    if (l < 16) {
#pragma unroll
        for (int i = 0; i < 16; i++) col[i] = c[i];
    }
    __syncwarp();
    return fail;
}

// No-pivot LU of the 16 x 16 block at (c0, c0) by lanes 0..15 of warp 0 in shared memory,
// with the reference's pivot rule; returns 1 if an exact zero pivot was skipped.
__device__ __forceinline__ int getrf16_warp(float (*Ds)[DP], int c0) {
    const int l = threadIdx.x & 31;
    float *col = &Ds[c0 + (l & 15)][c0];
    float *pcol = nullptr;
    int zero = 0;
    for (int p = 0; p < 16; p++) {
        pcol = &Ds[c0 + p][c0];
        const float piv = pcol[p];
        if (piv != 0.f) {
            // L(i, p) = A(i, p) / piv, lane i scales row i of column p
            if (l > p && l < 16) pcol[l] = fabsf(piv) > FLT_MIN ? pcol[l] * (1.f / piv) : pcol[l] / piv;
        } else {
            zero = 1;
        }
        __syncwarp();
        if (l > p && l < 16) {
            const float u = col[p];  // U(p, l)
            float lv[16], cv[16];
#pragma unroll
            for (int i = 0; i < 16; i++) {
                lv[i] = pcol[i];  // L(i, p)
                cv[i] = col[i];
            }
#pragma unroll
            for (int i = 0; i < 16; i++)
                if (i > p) col[i] = fmaf(-lv[i], u, cv[i]);
        }
        __syncwarp();
    }
    return zero;
}

// Returns the first failing column (Cholesky) or -1.  sflag: one shared int.
__device__ __forceinline__ int chol64(float (*Ds)[DP], int *sflag) {
    const int q = threadIdx.x >> 3, i0 = threadIdx.x & 7;
    for (int c0 = 0; c0 < 64; c0 += 16) {
        if (threadIdx.x < 32) {
            const int bad = chol16_warp(Ds, c0);
            if (threadIdx.x == 0) *sflag = bad;
        }
        __syncthreads();
        const int bad = *sflag;
        if (bad >= 0) return c0 + bad;
        const int c1 = c0 + 16;
        if (c1 == 64) break;
        // row panel U(c0:c1, c1:64) = U11^-T A(c0:c1, c1:64), one column per thread
        if (threadIdx.x < 64 - c1) {
            const int col = c1 + threadIdx.x;
            float x[16];
#pragma unroll
            for (int i = 0; i < 16; i++) x[i] = Ds[col][c0 + i];
#pragma unroll
            for (int p = 0; p < 16; p++) {
                x[p] = x[p] / Ds[c0 + p][c0 + p];
#pragma unroll
                for (int i = p + 1; i < 16; i++) x[i] = fmaf(-Ds[c0 + i][c0 + p], x[p], x[i]);  // U(p,i)
            }
#pragma unroll
            for (int i = 0; i < 16; i++) Ds[col][c0 + i] = x[i];
        }
        __syncthreads();
        // A(i, q) -= U(c0:c1, i)^T U(c0:c1, q), c1 <= i <= q
        if (q >= c1) {
            float uq[16];
#pragma unroll
            for (int k = 0; k < 16; k++) uq[k] = Ds[q][c0 + k];
            float out[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const int i = i0 + 8 * j;
                float a = Ds[q][i];
#pragma unroll
                for (int k = 0; k < 16; k++) a = fmaf(-Ds[i][c0 + k], uq[k], a);
                out[j] = a;
            }
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const int i = i0 + 8 * j;
                if (i >= c1 && i <= q) Ds[q][i] = out[j];
            }
        }
        __syncthreads();
    }
    return -1;
}

// No-pivot LU of the block; returns 1 if an exact zero pivot was skipped.
__device__ __forceinline__ int getrf64(float (*Ds)[DP], int *sflag) {
    const int q = threadIdx.x >> 3, i0 = threadIdx.x & 7;
    int zero = 0;
    for (int c0 = 0; c0 < 64; c0 += 16) {
        if (threadIdx.x < 32) {
            const int z = getrf16_warp(Ds, c0);
            if (threadIdx.x == 0) *sflag = z;
        }
        __syncthreads();
        zero |= *sflag;
        const int c1 = c0 + 16;
        if (c1 == 64) break;
        if (threadIdx.x < 64 - c1) {
            // row panel U(c0:c1, col) = L11^-1 A(c0:c1, col) (unit lower)
            const int col = c1 + threadIdx.x;
            float x[16];
#pragma unroll
            for (int i = 0; i < 16; i++) x[i] = Ds[col][c0 + i];
#pragma unroll
            for (int p = 0; p < 16; p++)
#pragma unroll
                for (int i = p + 1; i < 16; i++) x[i] = fmaf(-Ds[c0 + p][c0 + i], x[p], x[i]);  // L(i,p)
#pragma unroll
            for (int i = 0; i < 16; i++) Ds[col][c0 + i] = x[i];
        } else if (threadIdx.x >= 64 && threadIdx.x < 128 - c1) {
            // column panel L(row, c0:c1) = A(row, c0:c1) U11^-1, the reference's pivot rule
            const int row = c1 + threadIdx.x - 64;
            float x[16];
#pragma unroll
            for (int k = 0; k < 16; k++) x[k] = Ds[c0 + k][row];
#pragma unroll
            for (int p = 0; p < 16; p++) {
                const float u = Ds[c0 + p][c0 + p];
                if (u != 0.f) x[p] = fabsf(u) > FLT_MIN ? x[p] * (1.f / u) : x[p] / u;
#pragma unroll
                for (int k = p + 1; k < 16; k++) x[k] = fmaf(-x[p], Ds[c0 + k][c0 + p], x[k]);  // U(p,k)
            }
#pragma unroll
            for (int k = 0; k < 16; k++) Ds[c0 + k][row] = x[k];
        }
        __syncthreads();
        // A(i, q) -= L(i, c0:c1) U(c0:c1, q), i, q >= c1
        if (q >= c1) {
            float uq[16];
#pragma unroll
            for (int k = 0; k < 16; k++) uq[k] = Ds[q][c0 + k];
            float out[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const int i = i0 + 8 * j;
                float a = Ds[q][i];
#pragma unroll
                for (int k = 0; k < 16; k++) a = fmaf(-Ds[c0 + k][i], uq[k], a);
                out[j] = a;
            }
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const int i = i0 + 8 * j;
                if (i >= c1) Ds[q][i] = out[j];
            }
        }
        __syncthreads();
    }
    return zero;
}

// ---- panels by substitution ----------------------------------------------------------------
// One vector of 64 entries (b[i * stride], i < 64), solved in place against the block in Ds,
// in two halves of 32 unknowns kept in registers:
//   KIND 0: U^T x = b (U upper, non-unit): coefficient of x_p in row u is U(p,u) = Ds[u][p]
//   KIND 1: L x = b (L unit lower):           coefficient L(u,p) = Ds[p][u]
//   KIND 2: x U = b (row vector, U upper):    coefficient U(p,u) = Ds[u][p], the reference's
//           pivot rule on the division (reciprocal when |u_uu| > FLT_MIN, zero skipped)
template <int KIND>
__device__ __forceinline__ float coef(const float (*Ds)[DP], int u, int p) {
    return KIND == 1 ? Ds[p][u] : Ds[u][p];
}
template <int KIND>
__device__ __forceinline__ float finish(const float (*Ds)[DP], int u, float s) {
    if (KIND == 1) return s;
    const float d = Ds[u][u];
    if (KIND == 0) return s / d;
    return d == 0.f ? s : (fabsf(d) > FLT_MIN ? s * (1.f / d) : s / d);
}
// Right-looking: once unknown p is final, every later unknown is updated at once (independent
// FMAs).  Two halves of 32 unknowns in registers (the first half is read back from v for the
// second half's right-hand side).  v[i * stride] holds the vector.
template <int KIND>
__device__ __noinline__ void solve_vec(const float (*Ds)[DP], float *v, size_t stride) {
    {
        float x[32];
#pragma unroll
        for (int i = 0; i < 32; i++) x[i] = v[(size_t)i * stride];
#pragma unroll
        for (int p = 0; p < 32; p++) {
            x[p] = finish<KIND>(Ds, p, x[p]);
#pragma unroll
            for (int i = p + 1; i < 32; i++) x[i] = fmaf(-coef<KIND>(Ds, i, p), x[p], x[i]);
        }
#pragma unroll
        for (int i = 0; i < 32; i++) v[(size_t)i * stride] = x[i];
    }
    float y[32];
#pragma unroll
    for (int i = 0; i < 32; i++) y[i] = v[(size_t)(32 + i) * stride];
#pragma unroll 4
    for (int p = 0; p < 32; p++) {
        const float xp = v[(size_t)p * stride];
#pragma unroll
        for (int i = 0; i < 32; i++) y[i] = fmaf(-coef<KIND>(Ds, 32 + i, p), xp, y[i]);
    }
#pragma unroll
    for (int p = 0; p < 32; p++) {
        y[p] = finish<KIND>(Ds, 32 + p, y[p]);
#pragma unroll
        for (int i = p + 1; i < 32; i++) y[i] = fmaf(-coef<KIND>(Ds, 32 + i, 32 + p), y[p], y[i]);
    }
#pragma unroll
    for (int i = 0; i < 32; i++) v[(size_t)(32 + i) * stride] = y[i];
}

// ---- trailing update -----------------------------------------------------------------------
// C (m x m at C, ld) -= A^T B where A, B are KC x m chunks As[kk][i], Bs[kk][j] in shared
// memory, accumulated over all 64 rows of the panel in chunks staged by `stage`.
// UPPER: only micro-tiles with bj >= bi, and inside diagonal micro-tiles only i <= j.
template <bool UPPER, class Stage>
__device__ __forceinline__ void trailing(float *C, int ld, int m, int kc, float *As, float *Bs, Stage stage) {
    const int mb = m / MT;
    const int tiles = UPPER ? mb * (mb + 1) / 2 : mb * mb;  // UPPER: micro-tiles with bj >= bi
    for (int base = 0; base < tiles; base += NT) {
        const int u = base + threadIdx.x;
        // consecutive threads take consecutive row blocks bi of one column block bj, so a warp's
        // accesses to a column of C are contiguous
        int bi = 0, bj = 0;
        if (UPPER) {
            int rem = u;  // column block bj holds bj + 1 micro-tiles (bi <= bj)
            while (bj < mb && rem > bj) {
                rem -= bj + 1;
                bj++;
            }
            bi = rem;
        } else {
            bi = u % mb;
            bj = u / mb;
        }
        const bool active = u < tiles;
        float acc[MT][MT];
#pragma unroll
        for (int i = 0; i < MT; i++)
#pragma unroll
            for (int j = 0; j < MT; j++) acc[i][j] = 0.f;
        for (int k0 = 0; k0 < 64; k0 += kc) {
            __syncthreads();
            stage(k0);
            __syncthreads();
            if (active) {
                for (int kk = 0; kk < kc; kk++) {
                    const float4 a0 = *reinterpret_cast<const float4 *>(As + (size_t)kk * m + bi * MT);
                    const float4 a1 = *reinterpret_cast<const float4 *>(As + (size_t)kk * m + bi * MT + 4);
                    const float4 b0 = *reinterpret_cast<const float4 *>(Bs + (size_t)kk * m + bj * MT);
                    const float4 b1 = *reinterpret_cast<const float4 *>(Bs + (size_t)kk * m + bj * MT + 4);
                    const float a[MT] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
                    const float b[MT] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
                    for (int i = 0; i < MT; i++)
#pragma unroll
                        for (int j = 0; j < MT; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
                }
            }
        }
        if (active) {
            // C micro-tile: per column two float4 (rows bi*8 .. bi*8+7), all loads before the
            // stores; inside a diagonal micro-tile of the upper update the strictly lower entries
            // are written back unchanged
            float4 cv[MT][2];
#pragma unroll
            for (int j = 0; j < MT; j++) {
                const float *cc = C + bi * MT + (size_t)(bj * MT + j) * ld;
                cv[j][0] = *reinterpret_cast<const float4 *>(cc);
                cv[j][1] = *reinterpret_cast<const float4 *>(cc + 4);
            }
#pragma unroll
            for (int j = 0; j < MT; j++) {
                float o[MT] = {cv[j][0].x, cv[j][0].y, cv[j][0].z, cv[j][0].w,
                               cv[j][1].x, cv[j][1].y, cv[j][1].z, cv[j][1].w};
#pragma unroll
                for (int i = 0; i < MT; i++)
                    if (!UPPER || bi < bj || i <= j) o[i] -= acc[i][j];
                float *cc = C + bi * MT + (size_t)(bj * MT + j) * ld;
                *reinterpret_cast<float4 *>(cc) = make_float4(o[0], o[1], o[2], o[3]);
                *reinterpret_cast<float4 *>(cc + 4) = make_float4(o[4], o[5], o[6], o[7]);
            }
        }
    }
}

// status: int[8] of the factorization (ST_CODE, ..., [6] = step)
template <int ALG>
__global__ void __launch_bounds__(NT, 1) diag_factor_kernel(float *T, int nb, int ld, int k, int col0, int *status) {
    extern __shared__ __align__(16) float smem[];
    float (*Ds)[DP] = reinterpret_cast<float (*)[DP]>(smem);
    const int kc = chunk_k(nb);
    float *As = smem + 64 * DP;
    float *Bs = As + (size_t)kc * (nb - 64);
    int *sflag = reinterpret_cast<int *>(As + stage_floats(nb));
    if (ld_volatile(status + ST_CODE) != 0) return;
    if (threadIdx.x == 0) status[6] = k;  // current step (error reports of later kernels)
    int zero = 0;
    for (int j0 = 0; j0 < nb; j0 += 64) {
        float *D = T + j0 + (size_t)j0 * ld;
#pragma unroll
        for (int j = 0; j < 4096 / NT; j++) {
            const int e = threadIdx.x + NT * j;
            Ds[e >> 6][e & 63] = D[(e & 63) + (size_t)(e >> 6) * ld];
        }
        __syncthreads();
        if (ALG == 0) {
            const int bad = chol64(Ds, sflag);
            if (bad >= 0) {
                if (threadIdx.x == 0 && atomicCAS(status + ST_CODE, 0, -3 /*PALIAL_ERR_NOT_SPD*/) == 0) {
                    status[ST_COL] = col0 + j0 + bad;
                    status[ST_M] = status[ST_N] = k;
                    status[6] = k;
                    __threadfence();
                }
                return;
            }
        } else {
            zero |= getrf64(Ds, sflag);
        }
        for (int e = threadIdx.x; e < 4096; e += NT) {
            const int r = e & 63, c = e >> 6;
            if (ALG == 1 || r <= c) D[r + (size_t)c * ld] = Ds[c][r];
        }
        const int m = nb - j0 - 64;
        if (m == 0) break;
        __syncthreads();
        // panels
        float *A12 = T + j0 + (size_t)(j0 + 64) * ld;  // 64 x m, columns at stride ld
        // column panel: staged through shared memory (coalesced loads and stores; a thread
        // solves one column, Ps[c][i] with an odd pitch so the threads' columns do not share banks)
        {
            float *Ps = As;  // the trailing update's chunk space is free here
            const int cwmax = stage_floats(nb) / PP;
            for (int c0 = 0; c0 < m; c0 += cwmax) {
                const int cw = min(cwmax, m - c0);
                // 16-byte loads, four per thread in flight before the shared stores (the panel
                // comes from L2: one latency per batch instead of one per element)
                const int nv = cw * 16;  // float4 per 64-row column: 16
                for (int e0 = threadIdx.x; e0 < nv; e0 += 4 * NT) {
                    float4 v[4];
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const int e = e0 + u * NT;
                        if (e < nv)
                            v[u] = *reinterpret_cast<const float4 *>(A12 + 4 * (e & 15) + (size_t)(c0 + (e >> 4)) * ld);
                    }
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const int e = e0 + u * NT;
                        if (e < nv) {
                            float *d = Ps + (e >> 4) * PP + 4 * (e & 15);
                            d[0] = v[u].x;
                            d[1] = v[u].y;
                            d[2] = v[u].z;
                            d[3] = v[u].w;
                        }
                    }
                }
                __syncthreads();
                for (int c = threadIdx.x; c < cw; c += NT) {
                    if (ALG == 0) solve_vec<0>(Ds, Ps + c * PP, 1);
                    else solve_vec<1>(Ds, Ps + c * PP, 1);
                }
                __syncthreads();
                for (int e = threadIdx.x; e < nv; e += NT) {
                    const float *d = Ps + (e >> 4) * PP + 4 * (e & 15);
                    *reinterpret_cast<float4 *>(A12 + 4 * (e & 15) + (size_t)(c0 + (e >> 4)) * ld) =
                        make_float4(d[0], d[1], d[2], d[3]);
                }
                __syncthreads();
            }
        }
        if (ALG == 1) {
            float *A21 = T + (j0 + 64) + (size_t)j0 * ld;  // m x 64, rows contiguous
            for (int r = threadIdx.x; r < m; r += NT) solve_vec<2>(Ds, A21 + r, ld);
        }
        __syncthreads();
        float *C = T + (j0 + 64) + (size_t)(j0 + 64) * ld;
        if (ALG == 0) {
            // As[kk][i] = U12(k0 + kk, i), contiguous in kk in global memory: each thread loads
            // 4 consecutive kk of one column (float4) and a warp covers 32 consecutive columns,
            // so the shared stores of a warp hit 32 different banks
            auto stage = [&](int k0) {
                const int nv = (kc / 4) * m;
                for (int e0 = threadIdx.x; e0 < nv; e0 += 4 * NT) {
                    float4 v[4];  // four loads in flight per thread
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const int e = e0 + u * NT;
                        if (e < nv) v[u] = *reinterpret_cast<const float4 *>(A12 + (k0 + 4 * (e / m)) + (size_t)(e % m) * ld);
                    }
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const int e = e0 + u * NT;
                        if (e < nv) {
                            const int i = e % m, kq = 4 * (e / m);
                            As[(size_t)(kq + 0) * m + i] = v[u].x;
                            As[(size_t)(kq + 1) * m + i] = v[u].y;
                            As[(size_t)(kq + 2) * m + i] = v[u].z;
                            As[(size_t)(kq + 3) * m + i] = v[u].w;
                        }
                    }
                }
            };
            trailing<true>(C, ld, m, kc, As, As, stage);
        } else {
            const float *A21 = T + (j0 + 64) + (size_t)j0 * ld;
            auto stage = [&](int k0) {
                for (int e = threadIdx.x; e < kc * m; e += NT) {
                    const int i = e % m, kk = e / m;  // L21(i, k0+kk): contiguous in i
                    As[(size_t)kk * m + i] = A21[i + (size_t)(k0 + kk) * ld];
                }
                for (int e = threadIdx.x; e < (kc / 4) * m; e += NT) {
                    const int j = e % m, kq = 4 * (e / m);  // U12(k0+kq.., j): float4 along kk
                    const float4 v = *reinterpret_cast<const float4 *>(A12 + (k0 + kq) + (size_t)j * ld);
                    Bs[(size_t)(kq + 0) * m + j] = v.x;
                    Bs[(size_t)(kq + 1) * m + j] = v.y;
                    Bs[(size_t)(kq + 2) * m + j] = v.z;
                    Bs[(size_t)(kq + 3) * m + j] = v.w;
                }
            };
            trailing<false>(C, ld, m, kc, As, Bs, stage);
        }
        __syncthreads();
    }
    if (ALG == 1 && zero && threadIdx.x == 0) atomicOr(status + ST_ZEROPIV, 1);
}

// ---- Cholesky of a 256 x 256 block held in shared memory -----------------------------------
// The upper triangle (32896 floats, packed by columns: column c's rows 0..c at c (c + 1) / 2)
// stays in shared memory for the whole factorization: one load and one store of the block,
// no global traffic between the 64-column steps (their latency grows when the trailing update
// loads HBM beside this kernel).  Per step: the 64 x 64 diagonal block through Ds (chol64), the
// row panel solved in place in its packed columns (solve_vec, one column per thread), the panel
// transposed into UT[p][i] once, and the trailing upper triangle updated from UT with 8 x 8
// register tiles (K = 64 in one pass).  The operations and their order per entry are those of
// diag_factor_kernel<0>, so the factors are bit-identical.
constexpr int H256 = 256;
constexpr int PK256 = H256 * (H256 + 1) / 2;
constexpr int UTP = 196;  // pitch of UT rows (float4-aligned)
constexpr int SMEM256_FLOATS = PK256 + 64 * DP + 64 * UTP + 64;

__device__ __forceinline__ int poff(int c) { return (c * (c + 1)) >> 1; }

__global__ void __launch_bounds__(NT, 1) chol256_smem_kernel(float *T, int ld, int k, int col0, int *status) {
    extern __shared__ __align__(16) float smem[];
    float *P = smem;
    float (*Ds)[DP] = reinterpret_cast<float (*)[DP]>(smem + PK256);
    float *UT = smem + PK256 + 64 * DP;
    int *sflag = reinterpret_cast<int *>(UT + 64 * UTP);
    if (ld_volatile(status + ST_CODE) != 0) return;
    if (threadIdx.x == 0) status[6] = k;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // load the upper triangle, one warp per column (rows in 32-row pieces, all loads of a
    // column in flight)
    for (int c = warp; c < H256; c += NT / 32) {
        const float *src = T + (size_t)c * ld;
        float v[8];
#pragma unroll
        for (int j = 0; j < 8; j++) v[j] = (32 * j + lane <= c) ? __ldcg(src + 32 * j + lane) : 0.f;
#pragma unroll
        for (int j = 0; j < 8; j++)
            if (32 * j + lane <= c) P[poff(c) + 32 * j + lane] = v[j];
    }
    __syncthreads();
    const int q8 = threadIdx.x >> 3, i8 = threadIdx.x & 7;
    for (int j0 = 0; j0 < H256; j0 += 64) {
        for (int e = threadIdx.x; e < 4096; e += NT) {
            const int r = e & 63, c = e >> 6;
            Ds[c][r] = r <= c ? P[poff(j0 + c) + j0 + r] : 0.f;
        }
        __syncthreads();
        const int bad = chol64(Ds, sflag);
        if (bad >= 0) {
            if (threadIdx.x == 0 && atomicCAS(status + ST_CODE, 0, -3 /*PALIAL_ERR_NOT_SPD*/) == 0) {
                status[ST_COL] = col0 + j0 + bad;
                status[ST_M] = status[ST_N] = k;
                status[6] = k;
                __threadfence();
            }
            return;
        }
        for (int e = threadIdx.x; e < 4096; e += NT) {
            const int r = e & 63, c = e >> 6;
            if (r <= c) P[poff(j0 + c) + j0 + r] = Ds[c][r];
        }
        const int m = H256 - j0 - 64;
        if (m == 0) break;
        __syncthreads();
        // row panel U12 = U11^-T A12 in place: column j0 + 64 + c, rows j0 .. j0 + 63
        for (int c = threadIdx.x; c < m; c += NT) solve_vec<0>(Ds, P + poff(j0 + 64 + c) + j0, 1);
        __syncthreads();
        // UT[p][i] = U12(p, i)
        for (int e = threadIdx.x; e < 64 * m; e += NT) {
            const int pr = e & 63, i = e >> 6;
            UT[pr * UTP + i] = P[poff(j0 + 64 + i) + j0 + pr];
        }
        __syncthreads();
        // A22(i, q) -= sum_p U12(p, i) U12(p, q), i <= q: 8 x 8 micro-tiles (bi <= bj)
        const int mb = m / MT, tiles = mb * (mb + 1) / 2;
        for (int u = threadIdx.x; u < tiles; u += NT) {
            int bj = 0, rem = u;  // column block bj holds bj + 1 micro-tiles
            while (bj < mb && rem > bj) {
                rem -= bj + 1;
                bj++;
            }
            const int bi = rem;
            float acc[MT][MT];
#pragma unroll
            for (int i = 0; i < MT; i++)
#pragma unroll
                for (int j = 0; j < MT; j++) acc[i][j] = 0.f;
#pragma unroll 4
            for (int pr = 0; pr < 64; pr++) {
                const float4 a0 = *reinterpret_cast<const float4 *>(UT + pr * UTP + bi * MT);
                const float4 a1 = *reinterpret_cast<const float4 *>(UT + pr * UTP + bi * MT + 4);
                const float4 b0 = *reinterpret_cast<const float4 *>(UT + pr * UTP + bj * MT);
                const float4 b1 = *reinterpret_cast<const float4 *>(UT + pr * UTP + bj * MT + 4);
                const float a[MT] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
                const float b[MT] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
                for (int i = 0; i < MT; i++)
#pragma unroll
                    for (int j = 0; j < MT; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
            }
#pragma unroll
            for (int j = 0; j < MT; j++) {
                const int q = j0 + 64 + bj * MT + j;
                float *col = P + poff(q) + j0 + 64 + bi * MT;
#pragma unroll
                for (int i = 0; i < MT; i++)
                    if (bi < bj || i <= j) col[i] -= acc[i][j];
            }
        }
        __syncthreads();
    }
    (void)q8;
    (void)i8;
    // store the upper triangle back
    for (int c = warp; c < H256; c += NT / 32) {
        float *dst = T + (size_t)c * ld;
#pragma unroll
        for (int j = 0; j < 8; j++)
            if (32 * j + lane <= c) dst[32 * j + lane] = P[poff(c) + 32 * j + lane];
    }
}

}  // namespace mpd

cudaError_t mpd_configure() {
    const int bytes = mpd::smem_floats(1024) * 4;
    cudaError_t e = cudaFuncSetAttribute(mpd::diag_factor_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(mpd::chol256_smem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             mpd::SMEM256_FLOATS * 4);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(mpd::diag_factor_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

cudaError_t mps_block_inverse(const float *W, int n, int nb, int k, int factors, float *binv, cudaStream_t s,
                              int blocks);
cudaError_t mps_half_panel(float *T, int h, int ld, const float *binv, int alg, cudaStream_t s);
cudaError_t mps_half_update(float *T, int h, int ld, int alg, cudaStream_t s);

// Cholesky blocks of 256 by the shared-memory-resident kernel (1, default) or the staged one (0);
// the two give the same bits (palial_gpu_set_diag_kernel).
int g_chol_smem = 1;
int set_diag_kernel(int kind) {
    const int old = g_chol_smem;
    if (kind == 0 || kind == 1) g_chol_smem = kind;
    return old;
}

// Factor diagonal tile k of the FP32 tile matrix W (n x n, tile nb) in place.  Tiles of
// NB >= 512 go two-level: A11 (h = NB/2) in one CTA; on many CTAs the off-diagonal blocks
// (Cholesky A12 <- U11^-T A12; LU U12 <- L11^-1 A12 and L21 <- A21 U11^-1) and the update of
// A22 (Cholesky its upper part -= A12^T A12, LU -= L21 U12); then A22 in one CTA (the one-CTA
// kernel's time grows about 3.5x per doubling of the size, the multi-CTA steps are short).
// binv: scratch for the inverses of A11's 64 x 64 diagonal factor blocks (2 nb x 64 floats).
cudaError_t mpd_factor_tile(int alg, float *W, int n, int nb, int k, int *status, float *binv, cudaStream_t s) {
    if (nb % 64 || nb > 1024) return cudaErrorInvalidValue;
    const int mt = n / nb;
    float *T = W + (size_t)nb * nb * ((size_t)k + (size_t)mt * k);
    if (nb >= 512 && nb % 128 == 0 && binv) {
        const int h = nb / 2;
        const int bytes = mpd::smem_floats(h) * 4;
        cudaError_t e;
        note_launch();
        if (alg == 0 && h == mpd::H256 && g_chol_smem)
            mpd::chol256_smem_kernel<<<1, mpd::NT, mpd::SMEM256_FLOATS * 4, s>>>(T, nb, k, 0, status);
        else if (alg == 0) mpd::diag_factor_kernel<0><<<1, mpd::NT, bytes, s>>>(T, h, nb, k, 0, status);
        else mpd::diag_factor_kernel<1><<<1, mpd::NT, bytes, s>>>(T, h, nb, k, 0, status);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = mps_block_inverse(W, n, nb, k, alg == 0 ? 1 : 2, binv, s, h / 64);
        if (e == cudaSuccess) e = mps_half_panel(T, h, nb, binv, alg, s);
        if (e == cudaSuccess) e = mps_half_update(T, h, nb, alg, s);
        if (e != cudaSuccess) return e;
        note_launch();
        if (alg == 0 && h == mpd::H256 && g_chol_smem)
            mpd::chol256_smem_kernel<<<1, mpd::NT, mpd::SMEM256_FLOATS * 4, s>>>(T + (size_t)h * (nb + 1), nb, k, h,
                                                                                status);
        else if (alg == 0)
            mpd::diag_factor_kernel<0><<<1, mpd::NT, bytes, s>>>(T + (size_t)h * (nb + 1), h, nb, k, h, status);
        else mpd::diag_factor_kernel<1><<<1, mpd::NT, bytes, s>>>(T + (size_t)h * (nb + 1), h, nb, k, h, status);
        return cudaGetLastError();
    }
    const int bytes = mpd::smem_floats(nb) * 4;
    note_launch();
    if (alg == 0 && nb == mpd::H256 && g_chol_smem)
        mpd::chol256_smem_kernel<<<1, mpd::NT, mpd::SMEM256_FLOATS * 4, s>>>(T, nb, k, 0, status);
    else if (alg == 0) mpd::diag_factor_kernel<0><<<1, mpd::NT, bytes, s>>>(T, nb, nb, k, 0, status);
    else mpd::diag_factor_kernel<1><<<1, mpd::NT, bytes, s>>>(T, nb, nb, k, 0, status);
    return cudaGetLastError();
}

}  // namespace palial
