// tile_f32.cuh -- FP32 CTA routines (256 threads) for the mixed-precision path: panel
// triangular solves and their GEMM updates, on FP32 tile-layout data.  Same structure as the
// FP64 routines of tile_f64.cuh; loads bypass L1 (tiles are written by other SMs).
#pragma once
#include "common.cuh"

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

// C[M x N] += alpha * op(A) op(B) (beta = 1), dims multiples of 64 / 32.  Ends synced.
template <bool TA, bool TB>
__device__ void cta_gemm(int M, int N, int K, float alpha, const float *A, int lda, const float *B, int ldb, float *C,
                         int ldc, float *smem) {
    float (*As)[SP] = reinterpret_cast<float (*)[SP]>(smem);
    float (*Bs)[SP] = reinterpret_cast<float (*)[SP]>(smem + KC * SP);
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    for (int i0 = 0; i0 < M; i0 += BM)
        for (int j0 = 0; j0 < N; j0 += BM) {
            float acc[4][4] = {};
            for (int p0 = 0; p0 < K; p0 += KC) {
                stage<TA>(As, A, lda, i0, p0);
                stage<!TB>(Bs, B, ldb, j0, p0);
                __syncthreads();
#pragma unroll 8
                for (int p = 0; p < KC; p++) {
                    const float4 a = *reinterpret_cast<const float4 *>(&As[p][ty * 4]);
                    const float4 b = *reinterpret_cast<const float4 *>(&Bs[p][tx * 4]);
                    const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
                    for (int x = 0; x < 4; x++)
#pragma unroll
                        for (int y = 0; y < 4; y++) acc[x][y] = fmaf(av[x], bv[y], acc[x][y]);
                }
                __syncthreads();
            }
#pragma unroll
            for (int y = 0; y < 4; y++)
#pragma unroll
                for (int x = 0; x < 4; x++) {
                    float *c = C + (size_t)(i0 + ty * 4 + x) + (size_t)(j0 + tx * 4 + y) * ldc;
                    *c = fmaf(alpha, acc[x][y], ldg(c));
                }
        }
    __syncthreads();
}

__device__ inline void load_diag64(float (*Ds)[DP], const float *A, int ld) {
    for (int e = threadIdx.x; e < 4096; e += NT) Ds[e >> 6][e & 63] = ldg(A + (e & 63) + (size_t)(e >> 6) * ld);
    __syncthreads();
}

// 64 x 64 substitution, triangle in Ds (Ds[c][r] = T(r,c)), right-hand sides B (global, ld):
//   KIND 0: U^T X = B;  KIND 1: X U = B;  KIND 2: L X = B (unit lower);  KIND 3: U X = B.
template <int KIND>
__device__ void solve64(float (*Ds)[DP], float (*Bs)[DP], float *B, int ld) {
    for (int e = threadIdx.x; e < 4096; e += NT) Bs[e >> 6][e & 63] = ldg(B + (e & 63) + (size_t)(e >> 6) * ld);
    __syncthreads();
    for (int q = 0; q < 64; q++) {
        const int p = (KIND == 3) ? 63 - q : q;
        if (KIND == 0 || KIND == 3) {
            if (threadIdx.x < 64) Bs[threadIdx.x][p] = Bs[threadIdx.x][p] / Ds[p][p];
            __syncthreads();
            for (int e = threadIdx.x; e < 4096; e += NT) {
                const int i = e & 63, c = e >> 6;
                if (KIND == 0 && i > p) Bs[c][i] = fmaf(-Ds[i][p], Bs[c][p], Bs[c][i]);   // U(p,i)
                if (KIND == 3 && i < p) Bs[c][i] = fmaf(-Ds[p][i], Bs[c][p], Bs[c][i]);   // U(i,p)
            }
        } else if (KIND == 1) {
            if (threadIdx.x < 64) Bs[p][threadIdx.x] = Bs[p][threadIdx.x] / Ds[p][p];
            __syncthreads();
            for (int e = threadIdx.x; e < 4096; e += NT) {
                const int r = e & 63, c = e >> 6;
                if (c > p) Bs[c][r] = fmaf(-Bs[p][r], Ds[c][p], Bs[c][r]);
            }
        } else {
            for (int e = threadIdx.x; e < 4096; e += NT) {
                const int i = e & 63, c = e >> 6;
                if (i > p) Bs[c][i] = fmaf(-Ds[p][i], Bs[c][p], Bs[c][i]);
            }
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < 4096; e += NT) B[(e & 63) + (size_t)(e >> 6) * ld] = Bs[e >> 6][e & 63];
    __syncthreads();
}

}  // namespace f32
}  // namespace palial
