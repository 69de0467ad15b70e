// tile_f64.cuh -- FP64 tile routines executed by one CTA (256 threads) of the persistent
// scheduler.  GB300 runs FP64 at about 2 DFMA per clock per SM, so every routine here is
// bound by the FP64 pipe; the design goal is to keep >= 4 warps with independent DFMAs in
// flight.  Tiles are produced by other SMs, so every global load of matrix data bypasses L1
// (ld.global.cg): an SM's L1 is not coherent with writes made elsewhere.
#pragma once
#include "common.cuh"

namespace palial {
namespace f64 {

constexpr int NT = 256;          // threads per CTA
constexpr int BM = 64;           // output sub-block
constexpr int KC = 32;           // K chunk staged in shared memory
constexpr int SP = BM + 2;       // shared pitch (doubles), keeps double2 alignment

// Stored-matrix masks applied while loading an operand.
enum Mask { M_NONE = 0, M_UPPER = 1, M_UNIT_LOWER = 2 };

// Shared memory used by cta_gemm: As[KC][SP] + Bs[KC][SP].
constexpr int GEMM_SMEM_DOUBLES = 2 * KC * SP;

__device__ __forceinline__ double ldg(const double *p) { return __ldcg(p); }
__device__ __forceinline__ double2 ldg2(const double *p) { return __ldcg(reinterpret_cast<const double2 *>(p)); }

// Load stored element (r, c) under a mask; the masked-out triangle is never read (another
// task may be writing it concurrently, e.g. R above the reflectors of a QR diagonal tile).
template <int MASK>
__device__ __forceinline__ double masked_ld(const double *p, int r, int c) {
    if (MASK == M_UPPER) return r > c ? 0.0 : ldg(p);
    if (MASK == M_UNIT_LOWER) return r < c ? 0.0 : (r == c ? 1.0 : ldg(p));
    return ldg(p);
}

// Stage op(X)[i0:i0+64, p0:p0+KC] into Xs[p][i] (k-major).  TX: X stored transposed (element
// (i,p) of op(X) at X[p + i*ld]); otherwise at X[i + p*ld].  MASK refers to the stored
// coordinates (r, c) of X.  Rows/cols beyond (mlim, klim) read as zero.
template <bool TX, int MASK>
__device__ __forceinline__ void stage_a(double (*Xs)[SP], const double *X, int ld, int i0, int p0,
                                        int klim) {
    const int t = threadIdx.x;
    if (!TX) {
        // p-rows of 64 contiguous doubles: each thread moves 4 double2.
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int e = t + q * NT;
            const int p = e >> 5, i = (e & 31) * 2;
            double2 v = make_double2(0.0, 0.0);
            if (p0 + p < klim) {
                if (MASK == M_NONE) {
                    v = ldg2(X + (size_t)(i0 + i) + (size_t)(p0 + p) * ld);
                } else {
                    const double *q0 = X + (size_t)(i0 + i) + (size_t)(p0 + p) * ld;
                    v.x = masked_ld<MASK>(q0, i0 + i, p0 + p);
                    v.y = masked_ld<MASK>(q0 + 1, i0 + i + 1, p0 + p);
                }
            }
            *reinterpret_cast<double2 *>(&Xs[p][i]) = v;
        }
    } else {
        // columns of KC contiguous doubles along p, transposed into Xs[p][i].
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int e = t + q * NT;
            const int i = e >> 4, p = (e & 15) * 2;
            double2 v = make_double2(0.0, 0.0);
            if (p0 + p < klim) {
                const double *q0 = X + (size_t)(p0 + p) + (size_t)(i0 + i) * ld;
                if (MASK == M_NONE) {
                    v = ldg2(q0);
                } else {
                    v.x = masked_ld<MASK>(q0, p0 + p, i0 + i);
                    v.y = masked_ld<MASK>(q0 + 1, p0 + p + 1, i0 + i);
                }
            }
            Xs[p][i] = v.x;
            Xs[p + 1][i] = v.y;
        }
    }
}

// C[M x N] = beta*C + alpha * op(A) op(B), all dims multiples of 64 (K of 32).
//  TA: op(A) = A^T (A stored K x M);  TB: op(B) = B^T (B stored N x K).
//  MA/MB: masks on stored A/B.  CUP: only write C entries with row <= col (diagonal blocks of
//  an upper-triangular update): entry (i, j) is written only if i <= j + coff, and blocks
//  entirely below that line are skipped.
//  Triangular masks also shrink the K range to where op(A) is nonzero.
// Ends with __syncthreads(); all global writes are visible to the CTA afterwards.
template <bool TA, bool TB, int MA = M_NONE, int MB = M_NONE, bool CUP = false>
__device__ void cta_gemm(int M, int N, int K, double alpha, const double *A, int lda,
                         const double *B, int ldb, double beta, double *C, int ldc, double *smem,
                         int coff = 0) {
    double (*As)[SP] = reinterpret_cast<double (*)[SP]>(smem);
    double (*Bs)[SP] = reinterpret_cast<double (*)[SP]>(smem + KC * SP);
    const int t = threadIdx.x;
    const int tx = t & 15, ty = t >> 4;
    for (int i0 = 0; i0 < M; i0 += BM) {
        // K range where op(A)(i, p) can be nonzero for rows i in [i0, i0+64).
        int klo = 0, khi = K;
        if (MA == M_UPPER) {  // stored upper: (r <= c)
            if (TA) khi = min(K, i0 + BM);  // op(A)(i,p) = X(p,i): p <= i
            else klo = i0;                  // X(i,p): i <= p
        } else if (MA == M_UNIT_LOWER) {    // stored unit lower: (r >= c)
            if (TA) klo = i0;               // X(p,i): p >= i
            else khi = min(K, i0 + BM);     // X(i,p): i >= p
        }
        klo = (klo / KC) * KC;
        for (int j0 = 0; j0 < N; j0 += BM) {
            if (CUP && i0 > j0 + coff + BM - 1) continue;
            double acc[4][4];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) acc[a][b] = 0.0;
            for (int p0 = klo; p0 < khi; p0 += KC) {
                stage_a<TA, MA>(As, A, lda, i0, p0, K);
                stage_a<!TB, MB>(Bs, B, ldb, j0, p0, K);
                __syncthreads();
#pragma unroll 8
                for (int p = 0; p < KC; p++) {
                    const double2 a01 = *reinterpret_cast<const double2 *>(&As[p][ty * 4]);
                    const double2 a23 = *reinterpret_cast<const double2 *>(&As[p][ty * 4 + 2]);
                    const double2 b01 = *reinterpret_cast<const double2 *>(&Bs[p][tx * 4]);
                    const double2 b23 = *reinterpret_cast<const double2 *>(&Bs[p][tx * 4 + 2]);
                    const double av[4] = {a01.x, a01.y, a23.x, a23.y};
                    const double bv[4] = {b01.x, b01.y, b23.x, b23.y};
#pragma unroll
                    for (int a = 0; a < 4; a++)
#pragma unroll
                        for (int b = 0; b < 4; b++) acc[a][b] = fma(av[a], bv[b], acc[a][b]);
                }
                __syncthreads();
            }
            // all loads of the output block before any store: a load issued after a store the
            // compiler cannot prove disjoint would wait for a full memory round trip each time
            double cv[4][4];
#pragma unroll
            for (int b = 0; b < 4; b++) {
                const int j = j0 + tx * 4 + b;
#pragma unroll
                for (int a = 0; a < 4; a++) {
                    const int i = i0 + ty * 4 + a;
                    const bool skip = (CUP && i > j + coff) || beta == 0.0;
                    cv[a][b] = skip ? 0.0 : ldg(C + (size_t)i + (size_t)j * ldc);
                }
            }
#pragma unroll
            for (int b = 0; b < 4; b++) {
                const int j = j0 + tx * 4 + b;
#pragma unroll
                for (int a = 0; a < 4; a++) {
                    const int i = i0 + ty * 4 + a;
                    if (CUP && i > j + coff) continue;
                    const double v = alpha * acc[a][b];
                    C[(size_t)i + (size_t)j * ldc] = (beta == 0.0) ? v : fma(beta, cv[a][b], v);
                }
            }
        }
    }
    __syncthreads();
}

// Y[M x N] = alpha * X + beta * Y  (column-major, any M, N).  Ends with __syncthreads().
__device__ inline void cta_axpby(int M, int N, double alpha, const double *X, int ldx, double beta,
                                 double *Y, int ldy) {
    // 4 elements per thread per pass, loads before stores
    for (int e0 = threadIdx.x; e0 < M * N; e0 += 4 * NT) {
        double xv[4], yv[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int e = e0 + q * NT;
            if (e < M * N) {
                const int i = e % M, j = e / M;
                xv[q] = ldg(X + (size_t)i + (size_t)j * ldx);
                yv[q] = beta == 0.0 ? 0.0 : ldg(Y + (size_t)i + (size_t)j * ldy);
            }
        }
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int e = e0 + q * NT;
            if (e < M * N) {
                const int i = e % M, j = e / M;
                Y[(size_t)i + (size_t)j * ldy] = (beta == 0.0) ? alpha * xv[q] : fma(alpha, xv[q], beta * yv[q]);
            }
        }
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------------------
// 64 x 64 diagonal-block helpers (shared memory Ds[64][65], column-major D(r,c) = Ds[c][r]).
// ---------------------------------------------------------------------------------------
constexpr int DP = 65;

__device__ inline void load_diag64(double (*Ds)[DP], const double *A, int ld) {
    for (int e = threadIdx.x; e < 64 * 64; e += NT) {
        const int r = e & 63, c = e >> 6;
        Ds[c][r] = ldg(A + r + (size_t)c * ld);
    }
    __syncthreads();
}

// Unblocked upper Cholesky of the 64x64 block held in Ds (upper triangle used).  Returns
// the first column with a non-positive pivot, or -1.  Uniform across the CTA.
__device__ inline int chol64_upper(double (*Ds)[DP], int *s_flag) {
    const int t = threadIdx.x;
    if (t == 0) *s_flag = -1;
    __syncthreads();
    for (int j = 0; j < 64; j++) {
        const double d = Ds[j][j];
        if (!(d > 0.0)) {
            if (t == 0 && *s_flag < 0) *s_flag = j;
            __syncthreads();
            return *s_flag;
        }
        const double rd = sqrt(d);
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
            if (r > j && r <= c) Ds[c][r] = fma(-Ds[r][j], Ds[c][j], Ds[c][r]);
        }
        __syncthreads();
    }
    return -1;
}

}  // namespace f64
}  // namespace palial
