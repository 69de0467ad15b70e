// tile_f32.cuh -- FP32 CTA routines (256 threads) for the mixed-precision path: panel
// triangular solves and their GEMM updates, on FP32 tile-layout data.  Same structure as the
// FP64 routines of tile_f64.cuh; loads bypass L1 (tiles are written by other SMs).
#pragma once
#include "common.cuh"
#include "tc_gemm.cuh"

namespace palial {
namespace f32 {

constexpr int NT = 256;
constexpr int BM = 64;
constexpr int KC = 32;
constexpr int SP = BM + 4;   // float4-aligned pitch
constexpr int GEMM_SMEM_FLOATS = 2 * KC * SP;
constexpr int DP = 65;

__device__ __forceinline__ float ldg(const float *p) { return __ldcg(p); }

// Stage op(X)[i0:i0+64, p0:p0+KC] into Xs[p][i].  TX: element (i,p) at X[p + i*ld], else at
// X[i + p*ld].
template <bool TX>
__device__ __forceinline__ void stage(float (*Xs)[SP], const float *X, int ld, int i0, int p0) {
    const int t = threadIdx.x;
    if (!TX) {
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const int e = t + q * NT;           // 512 float4 = 32 x 64
            const int p = e >> 4, i = (e & 15) * 4;
            const float4 v = __ldcg(reinterpret_cast<const float4 *>(X + (size_t)(i0 + i) + (size_t)(p0 + p) * ld));
            *reinterpret_cast<float4 *>(&Xs[p][i]) = v;
        }
    } else {
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const int e = t + q * NT;
            const int i = e >> 3, p = (e & 7) * 4;
            const float4 v = __ldcg(reinterpret_cast<const float4 *>(X + (size_t)(p0 + p) + (size_t)(i0 + i) * ld));
            Xs[p][i] = v.x;
            Xs[p + 1][i] = v.y;
            Xs[p + 2][i] = v.z;
            Xs[p + 3][i] = v.w;
        }
    }
}

// The same staging split in two halves, so the next chunk's global loads can be in flight
// while the current chunk is computed: stage_load reads into registers, stage_store writes them.
template <bool TX>
__device__ __forceinline__ void stage_load(float4 (&v)[2], const float *X, int ld, int i0, int p0) {
    const int t = threadIdx.x;
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const int e = t + q * NT;
        if (!TX) {
            const int p = e >> 4, i = (e & 15) * 4;
            v[q] = __ldcg(reinterpret_cast<const float4 *>(X + (size_t)(i0 + i) + (size_t)(p0 + p) * ld));
        } else {
            const int i = e >> 3, p = (e & 7) * 4;
            v[q] = __ldcg(reinterpret_cast<const float4 *>(X + (size_t)(p0 + p) + (size_t)(i0 + i) * ld));
        }
    }
}
template <bool TX>
__device__ __forceinline__ void stage_store(float (*Xs)[SP], const float4 (&v)[2]) {
    const int t = threadIdx.x;
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const int e = t + q * NT;
        if (!TX) {
            const int p = e >> 4, i = (e & 15) * 4;
            *reinterpret_cast<float4 *>(&Xs[p][i]) = v[q];
        } else {
            const int i = e >> 3, p = (e & 7) * 4;
            Xs[p][i] = v[q].x;
            Xs[p + 1][i] = v[q].y;
            Xs[p + 2][i] = v[q].z;
            Xs[p + 3][i] = v[q].w;
        }
    }
}

// C[M x N] += alpha * op(A) op(B) (beta = 1), dims multiples of 64 / 32.  KEEP_LOWER leaves
// the entries below C's diagonal unchanged (an upper-triangle update).  TC: the products on the
// warp tensor cores in BF16x3 (tc_gemm.cuh) instead of FP32 FMAs.  Ends synced.
template <bool TA, bool TB, bool KEEP_LOWER = false, bool TC = false>
__device__ __forceinline__ void cta_gemm(int M, int N, int K, float alpha, const float *A, int lda, const float *B, int ldb, float *C,
                         int ldc, float *smem) {
    float (*As)[SP] = reinterpret_cast<float (*)[SP]>(smem);
    float (*Bs)[SP] = reinterpret_cast<float (*)[SP]>(smem + KC * SP);
    if (TC) {
        for (int i0 = 0; i0 < M; i0 += BM)
            for (int j0 = 0; j0 < N; j0 += BM) {
                tcg::Frag f;
                tcg::zero(f);
                float4 ra[2], rb[2];
                if (K > 0) {
                    stage_load<TA>(ra, A, lda, i0, 0);
                    stage_load<!TB>(rb, B, ldb, j0, 0);
                }
                for (int p0 = 0; p0 < K; p0 += KC) {
                    stage_store<TA>(As, ra);
                    stage_store<!TB>(Bs, rb);
                    __syncthreads();
                    if (p0 + KC < K) {
                        stage_load<TA>(ra, A, lda, i0, p0 + KC);
                        stage_load<!TB>(rb, B, ldb, j0, p0 + KC);
                    }
                    tcg::bf16x3_chunk<SP>(&As[0][0], &Bs[0][0], f);
                    __syncthreads();
                }
                float cv[4][4];
#pragma unroll
                for (int nt = 0; nt < 4; nt++)
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        int r, c;
                        tcg::frag_coord(nt, e, r, c);
                        cv[nt][e] = __ldcg(C + (size_t)(i0 + r) + (size_t)(j0 + c) * ldc);
                    }
#pragma unroll
                for (int nt = 0; nt < 4; nt++)
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        int r, c;
                        tcg::frag_coord(nt, e, r, c);
                        if (KEEP_LOWER && i0 + r > j0 + c) continue;
                        C[(size_t)(i0 + r) + (size_t)(j0 + c) * ldc] = fmaf(alpha, f.acc[nt][e], cv[nt][e]);
                    }
            }
        __syncthreads();
        return;
    }
    // thread: rows 4*tr .. 4*tr+3 (tr = t % 16, so a warp's 16 row groups are contiguous in a
    // column of C) and columns 4*tc .. 4*tc+3 (tc = t / 16)
    const int tr = threadIdx.x & 15, tc = threadIdx.x >> 4;
    for (int i0 = 0; i0 < M; i0 += BM)
        for (int j0 = 0; j0 < N; j0 += BM) {
            float acc[4][4] = {};
            float4 ra[2], rb[2];  // the next chunk, in flight during the current one's compute
            if (K > 0) {
                stage_load<TA>(ra, A, lda, i0, 0);
                stage_load<!TB>(rb, B, ldb, j0, 0);
            }
            for (int p0 = 0; p0 < K; p0 += KC) {
                stage_store<TA>(As, ra);
                stage_store<!TB>(Bs, rb);
                __syncthreads();
                if (p0 + KC < K) {
                    stage_load<TA>(ra, A, lda, i0, p0 + KC);
                    stage_load<!TB>(rb, B, ldb, j0, p0 + KC);
                }
#pragma unroll 8
                for (int p = 0; p < KC; p++) {
                    const float4 a = *reinterpret_cast<const float4 *>(&As[p][tr * 4]);
                    const float4 b = *reinterpret_cast<const float4 *>(&Bs[p][tc * 4]);
                    const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
                    for (int x = 0; x < 4; x++)
#pragma unroll
                        for (int y = 0; y < 4; y++) acc[x][y] = fmaf(av[x], bv[y], acc[x][y]);
                }
                __syncthreads();
            }
            // all loads of the output block first (see tile_f64.cuh, cta_gemm); one float4 per
            // column (ldc and the row offsets are multiples of 4)
            float4 cv[4];
#pragma unroll
            for (int y = 0; y < 4; y++)
                cv[y] = __ldcg(reinterpret_cast<const float4 *>(C + (size_t)(i0 + tr * 4) + (size_t)(j0 + tc * 4 + y) * ldc));
#pragma unroll
            for (int y = 0; y < 4; y++) {
                float4 o = make_float4(fmaf(alpha, acc[0][y], cv[y].x), fmaf(alpha, acc[1][y], cv[y].y),
                                       fmaf(alpha, acc[2][y], cv[y].z), fmaf(alpha, acc[3][y], cv[y].w));
                if (KEEP_LOWER) {
                    const int r = i0 + tr * 4, c = j0 + tc * 4 + y;
                    if (r + 0 > c) o.x = cv[y].x;
                    if (r + 1 > c) o.y = cv[y].y;
                    if (r + 2 > c) o.z = cv[y].z;
                    if (r + 3 > c) o.w = cv[y].w;
                }
                *reinterpret_cast<float4 *>(C + (size_t)(i0 + tr * 4) + (size_t)(j0 + tc * 4 + y) * ldc) = o;
            }
        }
    __syncthreads();
}

// C[M x 16] += alpha * op(A) B with B K x 16 (element (p, j) at B[p + j*ldb], 16-byte aligned
// columns): the refinement solves' right-hand-side blocks (at most 16 right-hand sides).
// Thread t computes row t/4 and columns 4*(t%4)..+3 of each 64-row block.  Ends synced.
constexpr int RW = 16;       // right-hand-side width of the refinement solves
constexpr int RP = RW + 4;   // pitch of the staged B chunk
template <bool TA>
__device__ __forceinline__ void cta_gemm_rw(int M, int K, float alpha, const float *A, int lda, const float *B, int ldb, float *C,
                            int ldc, float *smem) {
    float (*As)[SP] = reinterpret_cast<float (*)[SP]>(smem);
    float (*Bs)[RP] = reinterpret_cast<float (*)[RP]>(smem + KC * SP);
    const int tx = threadIdx.x & 3, ty = threadIdx.x >> 2;
    for (int i0 = 0; i0 < M; i0 += BM) {
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        float4 ra[2], rbv = make_float4(0.f, 0.f, 0.f, 0.f);  // the next chunk, in flight
        const int bj = threadIdx.x / (KC / 4), bp = (threadIdx.x % (KC / 4)) * 4;
        const bool bthr = threadIdx.x < KC * RW / 4;
        if (K > 0) {
            stage_load<TA>(ra, A, lda, i0, 0);
            if (bthr) rbv = __ldcg(reinterpret_cast<const float4 *>(B + (size_t)bp + (size_t)bj * ldb));
        }
        for (int p0 = 0; p0 < K; p0 += KC) {
            stage_store<TA>(As, ra);
            if (bthr) {
                Bs[bp][bj] = rbv.x;
                Bs[bp + 1][bj] = rbv.y;
                Bs[bp + 2][bj] = rbv.z;
                Bs[bp + 3][bj] = rbv.w;
            }
            __syncthreads();
            if (p0 + KC < K) {
                stage_load<TA>(ra, A, lda, i0, p0 + KC);
                if (bthr) rbv = __ldcg(reinterpret_cast<const float4 *>(B + (size_t)(p0 + KC + bp) + (size_t)bj * ldb));
            }
#pragma unroll 8
            for (int p = 0; p < KC; p++) {
                const float a = As[p][ty];
                const float4 b = *reinterpret_cast<const float4 *>(&Bs[p][tx * 4]);
                acc[0] = fmaf(a, b.x, acc[0]);
                acc[1] = fmaf(a, b.y, acc[1]);
                acc[2] = fmaf(a, b.z, acc[2]);
                acc[3] = fmaf(a, b.w, acc[3]);
            }
            __syncthreads();
        }
        float cv[4];
#pragma unroll
        for (int y = 0; y < 4; y++) cv[y] = ldg(C + (size_t)(i0 + ty) + (size_t)(tx * 4 + y) * ldc);
#pragma unroll
        for (int y = 0; y < 4; y++) C[(size_t)(i0 + ty) + (size_t)(tx * 4 + y) * ldc] = fmaf(alpha, acc[y], cv[y]);
    }
    __syncthreads();
}

// C[64 x 16] += alpha * op(A) B as cta_gemm_rw for M = 64, with K staged in chunks of 128 (K a
// multiple of 128): each chunk's loads (a 32 KB slice of A, 8 KB of B) are one round trip, in
// flight while the previous chunk is computed, so a K = 512 product costs four memory round
// trips instead of sixteen.  Shared layouts: op(A) = A^T is stored row-major by output row
// (Ar[i][p], float4 stores), op(A) = A column-major by K (Ac[p][i]); B as Bs[p][j].
constexpr int KC2 = 128;
constexpr int AP2 = KC2 + 4;  // pitch of Ar (float4-aligned, rows 4 banks apart)
constexpr int RW2_SMEM_FLOATS = (64 * AP2 > KC2 * SP ? 64 * AP2 : KC2 * SP) + KC2 * RP;
template <bool TA>
__device__ __forceinline__ void cta_gemm_rw128(int K, float alpha, const float *A, int lda, const float *B, int ldb,
                                               float *C, int ldc, float *smem) {
    float (*Ar)[AP2] = reinterpret_cast<float (*)[AP2]>(smem);
    float (*Ac)[SP] = reinterpret_cast<float (*)[SP]>(smem);
    float (*Bs)[RP] = reinterpret_cast<float (*)[RP]>(smem + (64 * AP2 > KC2 * SP ? 64 * AP2 : KC2 * SP));
    const int t = threadIdx.x, tx = t & 3, ty = t >> 2;
    static_assert(NT == 256, "thread mapping");
    float4 ra[8], rb[2];
    auto load = [&](int p0) {
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int e = t + NT * q;
            if (TA) {
                const int i = e >> 5, p = (e & 31) * 4;
                ra[q] = __ldcg(reinterpret_cast<const float4 *>(A + (size_t)(p0 + p) + (size_t)i * lda));
            } else {
                const int p = e >> 4, i = (e & 15) * 4;
                ra[q] = __ldcg(reinterpret_cast<const float4 *>(A + (size_t)i + (size_t)(p0 + p) * lda));
            }
        }
#pragma unroll
        for (int q = 0; q < 2; q++) {
            // a warp spans the 16 right-hand sides (B is small and in L2): conflict-free stores
            const int e = t + NT * q;
            const int j = e & 15, p = (e >> 4) * 4;
            rb[q] = __ldcg(reinterpret_cast<const float4 *>(B + (size_t)(p0 + p) + (size_t)j * ldb));
        }
    };
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    if (K > 0) load(0);
    for (int p0 = 0; p0 < K; p0 += KC2) {
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int e = t + NT * q;
            if (TA) {
                const int i = e >> 5, p = (e & 31) * 4;
                *reinterpret_cast<float4 *>(&Ar[i][p]) = ra[q];
            } else {
                const int p = e >> 4, i = (e & 15) * 4;
                *reinterpret_cast<float4 *>(&Ac[p][i]) = ra[q];
            }
        }
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const int e = t + NT * q;
            const int j = e & 15, p = (e >> 4) * 4;
            Bs[p][j] = rb[q].x;
            Bs[p + 1][j] = rb[q].y;
            Bs[p + 2][j] = rb[q].z;
            Bs[p + 3][j] = rb[q].w;
        }
        __syncthreads();
        if (p0 + KC2 < K) load(p0 + KC2);
#pragma unroll 8
        for (int p = 0; p < KC2; p++) {
            const float a = TA ? Ar[ty][p] : Ac[p][ty];
            const float4 b = *reinterpret_cast<const float4 *>(&Bs[p][tx * 4]);
            acc[0] = fmaf(a, b.x, acc[0]);
            acc[1] = fmaf(a, b.y, acc[1]);
            acc[2] = fmaf(a, b.z, acc[2]);
            acc[3] = fmaf(a, b.w, acc[3]);
        }
        __syncthreads();
    }
    float cv[4];
#pragma unroll
    for (int y = 0; y < 4; y++) cv[y] = ldg(C + (size_t)ty + (size_t)(tx * 4 + y) * ldc);
#pragma unroll
    for (int y = 0; y < 4; y++) C[(size_t)ty + (size_t)(tx * 4 + y) * ldc] = fmaf(alpha, acc[y], cv[y]);
    __syncthreads();
}

__device__ __forceinline__ void load_diag64(float (*Ds)[DP], const float *A, int ld) {
#pragma unroll
    for (int j = 0; j < 4096 / NT; j++) {
        const int e = threadIdx.x + NT * j;
        Ds[e >> 6][e & 63] = ldg(A + (e & 63) + (size_t)(e >> 6) * ld);
    }
    __syncthreads();
}

// 64 x 64 substitution, triangle in Ds (Ds[c][r] = T(r,c)), right-hand sides B (global, ld):
//   KIND 0: U^T X = B;  KIND 1: X U = B;  KIND 2: L X = B (unit lower);  KIND 3: U X = B.
// Threads 0..63 each solve one right-hand side (a column of B; a row for KIND 1) with its 64
// unknowns in registers, in two halves of 32 (no barrier inside the solve).  Ends synced.
template <int KIND>
__device__ __forceinline__ int sub_row(int j) { return KIND == 3 ? 63 - j : j; }  // solve order
template <int KIND>
__device__ __forceinline__ float sub_coef(const float (*Ds)[DP], int u, int p) {
    // coefficient of unknown p in the equation of unknown u
    return (KIND == 0 || KIND == 1) ? Ds[u][p] : Ds[p][u];
}
template <int KIND>
__device__ __forceinline__ void solve64(float (*Ds)[DP], float *B, int ld) {
    if (threadIdx.x < 64) {
        const size_t vstride = (KIND == 1) ? 1 : (size_t)ld;   // between right-hand sides
        const size_t estride = (KIND == 1) ? (size_t)ld : 1;   // between entries of one
        float *b = B + (size_t)threadIdx.x * vstride;
#pragma unroll 1
        for (int h = 0; h < 64; h += 32) {
            float x[32];
#pragma unroll
            for (int i = 0; i < 32; i++) x[i] = ldg(b + (size_t)sub_row<KIND>(h + i) * estride);
            if (h) {
#pragma unroll 4
                for (int pj = 0; pj < 32; pj++) {
                    const int pu = sub_row<KIND>(pj);
                    const float xp = b[(size_t)pu * estride];
#pragma unroll
                    for (int i = 0; i < 32; i++) x[i] = fmaf(-sub_coef<KIND>(Ds, sub_row<KIND>(h + i), pu), xp, x[i]);
                }
            }
#pragma unroll
            for (int i = 0; i < 32; i++) {
                const int u = sub_row<KIND>(h + i);
                float acc = x[i];
#pragma unroll
                for (int pi = 0; pi < i; pi++) acc = fmaf(-sub_coef<KIND>(Ds, u, sub_row<KIND>(h + pi)), x[pi], acc);
                x[i] = (KIND == 2) ? acc : acc / Ds[u][u];
            }
#pragma unroll
            for (int i = 0; i < 32; i++) b[(size_t)sub_row<KIND>(h + i) * estride] = x[i];
        }
    }
    __syncthreads();
}

}  // namespace f32
}  // namespace palial
