// sched_f64.cu -- persistent device-side DAG scheduler and the FP64 tile tasks of the tiled
// Cholesky (reference src/cholesky.h), no-pivot LU (src/lu.h, src/srclu) and flat-tree
// TS QR (src/qr.h, src/srcqr).
//
// One CTA = one worker.  A worker takes the next task record (atomic ticket, dispatch order
// fixed by the host), waits on the completion counters of the objects it reads/updates
// (acquire loads with a %globaltimer deadline), runs the tile routine, and releases its
// output objects (fence + atomic increment).  Each object's updates are therefore applied in
// program order (k order), so the factors are bit-identical under any dispatch order or
// worker count.
#include <cstdio>

#include "common.cuh"
#include "tile_f64.cuh"

namespace palial {
using namespace f64;

// Dynamic shared memory layout of a worker (doubles):
//   Ds[64][65] | Is[64][65] | U[union: gemm staging (2*KC*SP) or Bs[64][65]] | misc
// (Is is spare room for a second 64x64 block.)
constexpr int SM_DS = 0;
constexpr int SM_IS = SM_DS + 64 * DP;
constexpr int SM_U = SM_IS + 64 * DP;
constexpr int SM_U_SIZE = (GEMM_SMEM_DOUBLES > 64 * DP) ? GEMM_SMEM_DOUBLES : 64 * DP;
constexpr int SM_RED = SM_U + SM_U_SIZE;         // 512 doubles: reductions / tau
constexpr int SM_TOTAL_DOUBLES = SM_RED + 1024 + 64;
constexpr int SCHED_SMEM_BYTES = SM_TOTAL_DOUBLES * 8;

struct Worker {
    double *smem;
    double (*Ds)[DP];
    double (*Is)[DP];
    double (*Bs)[DP];
    double *gsm;   // gemm staging
    double *red;   // 1024 doubles
    int *sflag;
};

__device__ __forceinline__ Worker make_worker(double *smem) {
    Worker w;
    w.smem = smem;
    w.Ds = reinterpret_cast<double (*)[DP]>(smem + SM_DS);
    w.Is = reinterpret_cast<double (*)[DP]>(smem + SM_IS);
    w.Bs = reinterpret_cast<double (*)[DP]>(smem + SM_U);
    w.gsm = smem + SM_U;
    w.red = smem + SM_RED;
    w.sflag = reinterpret_cast<int *>(smem + SM_RED + 1024);
    return w;
}

// ---------------------------------------------------------------------------------------
// 64 x 64 triangular solves by substitution (the column-oriented order of BLAS dtrsm),
// with the triangle in w.Ds (Ds[c][r] = T(r,c)) and the right-hand sides B (64 x 64, global,
// ld) staged in w.Bs.  No explicit inverse: no-pivot LU can meet ill-conditioned diagonal
// blocks, and substitution keeps the reference's backward error.
//   KIND 0: U^T X = B (U upper, non-unit)   -- Cholesky TRSM (left, upper, trans)
//   KIND 1: X U = B   (U upper, non-unit)   -- LU TRSM (right, upper, no-trans)
//   KIND 2: L X = B   (L unit lower)        -- LU TRSM (left, lower, unit)
//   KIND 3: U X = B   (U upper, non-unit)   -- QR solve back-substitution (left, upper)
// ---------------------------------------------------------------------------------------
template <int KIND>
__device__ void solve64(const Worker &w, double *B, int ld) {
    // Bs[c][r] = B(r, c)
    for (int e = threadIdx.x; e < 4096; e += NT) {
        const int r = e & 63, c = e >> 6;
        w.Bs[c][r] = ldg(B + r + (size_t)c * ld);
    }
    __syncthreads();
    for (int pp = 0; pp < 64; pp++) {
        const int p = (KIND == 3) ? 63 - pp : pp;
        if (KIND == 3) {
            // unknown row p (last first): X(p,c) = B(p,c) / U(p,p); rows i < p: B(i,c) -= U(i,p) X(p,c)
            if (threadIdx.x < 64) w.Bs[threadIdx.x][p] = w.Bs[threadIdx.x][p] / w.Ds[p][p];
            __syncthreads();
            for (int e = threadIdx.x; e < 64 * 64; e += NT) {
                const int i = e & 63, c = e >> 6;
                if (i < p) w.Bs[c][i] = fma(-w.Ds[p][i], w.Bs[c][p], w.Bs[c][i]);
            }
        } else if (KIND == 0) {
            if (threadIdx.x < 64) w.Bs[threadIdx.x][p] = w.Bs[threadIdx.x][p] / w.Ds[p][p];
            __syncthreads();
            // rows i > p of every column c: B(i,c) -= U(p,i) X(p,c)
            for (int e = threadIdx.x; e < 64 * 64; e += NT) {
                const int i = e & 63, c = e >> 6;
                if (i > p) w.Bs[c][i] = fma(-w.Ds[i][p], w.Bs[c][p], w.Bs[c][i]);
            }
        } else if (KIND == 1) {
            // unknown column p: X(:,p) = B(:,p) / U(p,p); then B(:,q) -= X(:,p) U(p,q), q > p
            if (threadIdx.x < 64) w.Bs[p][threadIdx.x] = w.Bs[p][threadIdx.x] / w.Ds[p][p];
            __syncthreads();
            for (int e = threadIdx.x; e < 64 * 64; e += NT) {
                const int r = e & 63, q = e >> 6;
                if (q > p) w.Bs[q][r] = fma(-w.Bs[p][r], w.Ds[q][p], w.Bs[q][r]);
            }
        } else {
            for (int e = threadIdx.x; e < 64 * 64; e += NT) {
                const int i = e & 63, c = e >> 6;
                if (i > p) w.Bs[c][i] = fma(-w.Ds[p][i], w.Bs[c][p], w.Bs[c][i]);
            }
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < 4096; e += NT) {
        const int r = e & 63, c = e >> 6;
        B[r + (size_t)c * ld] = w.Bs[c][r];
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------------------
// POTRF (upper) of an n x n block, n multiple of 64.  Blocked by 64: factor the diagonal
// block in shared memory, solve the row panel by substitution, then the upper-triangular
// rank-64 update of the trailing block.
// Returns -1, or the first column with a non-positive pivot.
// ---------------------------------------------------------------------------------------
__device__ int potrf_upper(const Worker &w, double *A, int n, int ld) {
    for (int j0 = 0; j0 < n; j0 += 64) {
        double *D = A + j0 + (size_t)j0 * ld;
        load_diag64(w.Ds, D, ld);
        const int bad = chol64_upper(w.Ds, w.sflag);
        if (bad >= 0) return j0 + bad;
        for (int e = threadIdx.x; e < 4096; e += NT) {
            const int r = e & 63, c = e >> 6;
            if (r <= c) D[r + (size_t)c * ld] = w.Ds[c][r];
        }
        __syncthreads();
        if (j0 + 64 < n) {
            for (int c0 = j0 + 64; c0 < n; c0 += 64) solve64<0>(w, A + j0 + (size_t)c0 * ld, ld);
            const int m = n - j0 - 64;
            const double *X = A + j0 + (size_t)(j0 + 64) * ld;
            cta_gemm<true, false, M_NONE, M_NONE, true>(m, m, 64, -1.0, X, ld, X, ld, 1.0,
                                                        A + (j0 + 64) + (size_t)(j0 + 64) * ld, ld, w.gsm, 0);
        }
    }
    return -1;
}

// ---------------------------------------------------------------------------------------
// GETRF without pivoting (reference src/srclu/dgetrf_no_pivot.h:11-57 rule: scale the column
// by the reciprocal pivot when |pivot| > DBL_MIN, divide otherwise, skip an exact zero),
// blocked by 64 columns: panel LU in global memory, U12 = L11^-1 A12 by substitution,
// A22 -= L21 U12.  Returns 1 if an exact zero pivot was met, else 0.
// ---------------------------------------------------------------------------------------
__device__ int getrf_nopiv(const Worker &w, double *A, int n, int ld) {
    const double sfmin = 2.2250738585072014e-308;  // dlamch('S') for IEEE double
    int zero_piv = 0;
    for (int j0 = 0; j0 < n; j0 += 64) {
        for (int i = 0; i < 64; i++) {
            const int col = j0 + i;
            double *ccol = A + (size_t)col * ld;
            const double piv = ldg(ccol + col);
            if (piv != 0.0) {
                const bool recip = fabs(piv) > sfmin;
                const double rp = 1.0 / piv;
                for (int r = col + 1 + threadIdx.x; r < n; r += NT)
                    ccol[r] = recip ? ldg(ccol + r) * rp : ldg(ccol + r) / piv;
            } else {
                zero_piv = 1;
            }
            __syncthreads();
            const int rows = n - col - 1, cols = j0 + 63 - col;
            // rank-1 update of the panel, 4 elements per thread per pass with all loads issued
            // before the stores (a load after a possibly aliasing store waits a round trip)
            for (int e0 = threadIdx.x; e0 < rows * cols; e0 += 4 * NT) {
                double l[4], u[4], x[4];
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
                        A[r + (size_t)c * ld] = fma(-l[q], u[q], x[q]);
                    }
                }
            }
            __syncthreads();
        }
        double *D = A + j0 + (size_t)j0 * ld;
        load_diag64(w.Ds, D, ld);
        if (j0 + 64 < n) {
            for (int c0 = j0 + 64; c0 < n; c0 += 64) solve64<2>(w, A + j0 + (size_t)c0 * ld, ld);
            const int m = n - j0 - 64;
            cta_gemm<false, false>(m, m, 64, -1.0, A + (j0 + 64) + (size_t)j0 * ld, ld,
                                   A + j0 + (size_t)(j0 + 64) * ld, ld, 1.0,
                                   A + (j0 + 64) + (size_t)(j0 + 64) * ld, ld, w.gsm);
        }
    }
    return zero_piv;
}

// ---------------------------------------------------------------------------------------
// Triangular solves on a 64-wide strip: GEMM updates from the solved blocks, then
// substitution against the diagonal 64x64 block.  n = block size, B = strip origin.
// ---------------------------------------------------------------------------------------
// X = U^-T B (U upper, B n x 64): row blocks top-down.
__device__ void trsm_lut(const Worker &w, const double *U, double *B, int n, int ld) {
    for (int rb = 0; rb < n; rb += 64) {
        if (rb > 0)
            cta_gemm<true, false>(64, 64, rb, -1.0, U + (size_t)rb * ld, ld, B, ld, 1.0, B + rb, ld, w.gsm);
        load_diag64(w.Ds, U + rb + (size_t)rb * ld, ld);
        solve64<0>(w, B + rb, ld);
    }
}
// X = B U^-1 (B 64 x n row strip): column blocks left to right.
__device__ void trsm_run(const Worker &w, const double *U, double *B, int n, int ld) {
    for (int cb = 0; cb < n; cb += 64) {
        if (cb > 0)
            cta_gemm<false, false>(64, 64, cb, -1.0, B, ld, U + (size_t)cb * ld, ld, 1.0, B + (size_t)cb * ld, ld,
                                   w.gsm);
        load_diag64(w.Ds, U + cb + (size_t)cb * ld, ld);
        solve64<1>(w, B + (size_t)cb * ld, ld);
    }
}
// X = U^-1 B (U upper, B n x 64): row blocks bottom-up.
__device__ void trsm_lun(const Worker &w, const double *U, double *B, int n, int ld) {
    for (int rb = n - 64; rb >= 0; rb -= 64) {
        if (rb + 64 < n)
            cta_gemm<false, false>(64, 64, n - rb - 64, -1.0, U + rb + (size_t)(rb + 64) * ld, ld, B + rb + 64, ld, 1.0,
                                   B + rb, ld, w.gsm);
        load_diag64(w.Ds, U + rb + (size_t)rb * ld, ld);
        solve64<3>(w, B + rb, ld);
    }
}
// X = L^-1 B (L unit lower, B n x 64): row blocks top-down.
__device__ void trsm_llu(const Worker &w, const double *L, double *B, int n, int ld) {
    for (int rb = 0; rb < n; rb += 64) {
        if (rb > 0) cta_gemm<false, false>(64, 64, rb, -1.0, L + rb, ld, B, ld, 1.0, B + rb, ld, w.gsm);
        load_diag64(w.Ds, L + rb + (size_t)rb * ld, ld);
        solve64<2>(w, B + rb, ld);
    }
}

// ---------------------------------------------------------------------------------------
// Householder generation (LAPACK dlarfg, published algorithm): given alpha and x (len m),
// produce beta, tau and v (x overwritten by v's tail, v(0) = 1 implicit) such that
// (I - tau v v^T) [alpha; x] = [beta; 0], beta = -sign(alpha) * ||[alpha; x]||.
// x is strided by 1; all threads participate; returns tau, writes beta to *alpha_p.
// ---------------------------------------------------------------------------------------
__device__ double block_sum(const Worker &w, double v) {
    // warp reduce then CTA reduce through w.red[0..7]; result broadcast
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) w.red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < NT / 32; i++) s += w.red[i];
    __syncthreads();
    return s;
}

__device__ double block_absmax(const Worker &w, double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) w.red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < NT / 32; i++) s = fmax(s, w.red[i]);
    __syncthreads();
    return s;
}

__device__ __forceinline__ double lapy2(double x, double y) {
    const double xa = fabs(x), ya = fabs(y);
    const double wv = fmax(xa, ya), z = fmin(xa, ya);
    if (z == 0.0) return wv;
    const double q = z / wv;
    return wv * sqrt(1.0 + q * q);
}

__device__ double norm2_block(const Worker &w, const double *x, int m) {
    // scaled sum of squares: max |x|, then sum (x/scale)^2 (avoids overflow/underflow)
    double mx = 0.0;
    for (int r = threadIdx.x; r < m; r += NT) mx = fmax(mx, fabs(ldg(x + r)));
    const double scale = block_absmax(w, mx);
    if (scale == 0.0) return 0.0;
    const double inv = 1.0 / scale;
    double s = 0.0;
    for (int r = threadIdx.x; r < m; r += NT) {
        const double q = ldg(x + r) * inv;
        s = fma(q, q, s);
    }
    return scale * sqrt(block_sum(w, s));
}

__device__ double larfg(const Worker &w, double *alpha_p, double *x, int m) {
    const double safmin = 2.2250738585072014e-308 / 1.1102230246251565e-16;  // dlamch('S')/dlamch('E')
    double alpha = ldg(alpha_p);
    double xnorm = norm2_block(w, x, m);
    if (xnorm == 0.0) return 0.0;  // H = I, alpha unchanged
    double beta = -copysign(lapy2(alpha, xnorm), alpha);
    int knt = 0;
    if (fabs(beta) < safmin) {
        const double rs = 1.0 / safmin;
        do {
            knt++;
            for (int r = threadIdx.x; r < m; r += NT) x[r] = ldg(x + r) * rs;
            __syncthreads();
            beta *= rs;
            alpha *= rs;
        } while (fabs(beta) < safmin && knt < 20);
        xnorm = norm2_block(w, x, m);
        beta = -copysign(lapy2(alpha, xnorm), alpha);
    }
    const double tau = (beta - alpha) / beta;
    const double sc = 1.0 / (alpha - beta);
    for (int r = threadIdx.x; r < m; r += NT) x[r] = ldg(x + r) * sc;
    for (int j = 0; j < knt; j++) beta *= safmin;
    __syncthreads();
    if (threadIdx.x == 0) *alpha_p = beta;
    __syncthreads();
    return tau;
}

// Apply one Householder reflector to column cj, one warp: s = head + <v, cj(r0:nb)>, where
// v = ci(r0:nb) and head = the column's entry on the reflector's unit position (*hj, which is
// updated too), then cj(r0:nb) += (-tau s) v.  The lane's slice of cj and v stays in registers
// between the dot product and the update (up to 16 entries per lane, nb - r0 <= 512; longer
// columns are handled in passes with batched loads), so no load waits behind a store.  The
// summation order is the plain lane-strided one either way.
__device__ __forceinline__ void reflect_col(const double *ci, double *cj, double *hj, int r0, int nb, double tau,
                                            int lane) {
    constexpr int U = 16;
    double s = (lane == 0) ? ldg(hj) : 0.0;
    if (nb - r0 <= 32 * U) {
        double vi[U], vj[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int r = r0 + lane + 32 * u;
            vi[u] = r < nb ? ldg(ci + r) : 0.0;
            vj[u] = r < nb ? ldg(cj + r) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < U; u++)
            if (r0 + lane + 32 * u < nb) s = fma(vi[u], vj[u], s);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        const double f = -tau * s;
        if (lane == 0) *hj = ldg(hj) + f;
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int r = r0 + lane + 32 * u;
            if (r < nb) cj[r] = fma(f, vi[u], vj[u]);
        }
        return;
    }
    for (int r = r0 + lane; r < nb; r += 32) s = fma(ldg(ci + r), ldg(cj + r), s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    const double f = -tau * s;
    if (lane == 0) *hj = ldg(hj) + f;
    for (int b = r0 + lane; b < nb; b += 32 * U) {
        double vi[U], vj[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int r = b + 32 * u;
            vi[u] = r < nb ? ldg(ci + r) : 0.0;
            vj[u] = r < nb ? ldg(cj + r) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int r = b + 32 * u;
            if (r < nb) cj[r] = fma(f, vi[u], vj[u]);
        }
    }
}

// T (upper, nb x nb, ld) of the forward column-wise compact WY form: T(i,i) = tau_i,
// T(0:i,i) = -tau_i T(0:i,0:i) z, z_j = <v_j, v_i> for j < i (LAPACK dlarft 'F','C').
// dot(j, i) is supplied by the caller as a functor evaluated by one warp.
template <class Dot>
__device__ void larft(const Worker &w, int nb, const double *tau, double *T, int ldt, Dot dot) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double *z = w.red + 8;  // up to 1016 doubles (nb <= 1016)
    for (int i = 0; i < nb; i++) {
        const double ti = tau[i];
        for (int j = warp; j < i; j += NT / 32) {
            double s = dot(j, i, lane);
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) z[j] = -ti * s;
        }
        __syncthreads();
        for (int r = threadIdx.x; r < i; r += NT) {
            double s = 0.0;
            for (int p = r; p < i; p++) s = fma(ldg(T + r + (size_t)p * ldt), z[p], s);
            T[r + (size_t)i * ldt] = s;
        }
        if (threadIdx.x == 0) T[i + (size_t)i * ldt] = ti;
        __syncthreads();
    }
}

// GEQRT of an nb x nb tile (reference src/srcqr/dgeqrt.h:9-56 = dgeqr2 + dlarft): unblocked
// Householder QR; R in the upper triangle, V below the diagonal, T into Tm (upper).
__device__ void geqrt(const Worker &w, double *A, int nb, int ld, double *Tm, int ldt) {
    double *tau = w.smem + SM_U;  // nb doubles (gemm staging area is free here)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = 0; i < nb; i++) {
        double *ci = A + (size_t)i * ld;
        const double ti = larfg(w, ci + i, ci + i + 1, nb - i - 1);
        if (threadIdx.x == 0) tau[i] = ti;
        // apply H_i to A(i:, i+1:)
        if (ti != 0.0) {
            for (int j = i + 1 + warp; j < nb; j += NT / 32) {
                double *cj = A + (size_t)j * ld;
                reflect_col(ci, cj, cj + i, i + 1, nb, ti, lane);
            }
        }
        __syncthreads();
    }
    // z_j = <v_j, v_i>, v_j = e_j + A(j+1:, j): for j < i, = A(i,j) + sum_{r>i} A(r,j) A(r,i)
    larft(w, nb, tau, Tm, ldt, [&](int j, int i, int ln) {
        const double *cj = A + (size_t)j * ld, *ci = A + (size_t)i * ld;
        double s = (ln == 0) ? ldg(cj + i) : 0.0;
        for (int r = i + 1 + ln; r < nb; r += 32) s = fma(ldg(cj + r), ldg(ci + r), s);
        return s;
    });
}

// TSQRT (reference src/srcqr/dtsqrt.h:11-109): QR of [R = A1 upper; A2] column by column.
// A1's strictly lower part (the GEQRT reflectors) is neither read nor written.
__device__ void tsqrt(const Worker &w, double *A1, double *A2, int nb, int ld, double *Tm, int ldt) {
    double *tau = w.smem + SM_U;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = 0; i < nb; i++) {
        double *vi = A2 + (size_t)i * ld;
        const double ti = larfg(w, A1 + i + (size_t)i * ld, vi, nb);
        if (threadIdx.x == 0) tau[i] = ti;
        if (ti != 0.0) {
            for (int j = i + 1 + warp; j < nb; j += NT / 32)
                reflect_col(vi, A2 + (size_t)j * ld, A1 + i + (size_t)j * ld, 0, nb, ti, lane);
        }
        __syncthreads();
    }
    // the identity parts of [I; V] are orthogonal, so z_j = <A2(:,j), A2(:,i)>
    larft(w, nb, tau, Tm, ldt, [&](int j, int i, int ln) {
        const double *cj = A2 + (size_t)j * ld, *ci = A2 + (size_t)i * ld;
        double s = 0.0;
        for (int r = ln; r < nb; r += 32) s = fma(ldg(cj + r), ldg(ci + r), s);
        return s;
    });
}

// UNMQR strip (reference src/srcqr/dormqr.h:9-53 = dlarfb 'L','T','F','C'):
// C <- C - V T^T V^T C on a 64-column strip; W, W2 are nb x 64 scratch.
__device__ void unmqr_strip(const Worker &w, const double *V, const double *T, double *C, int nb, int ld,
                            double *W, double *W2) {
    cta_gemm<true, false, M_UNIT_LOWER>(nb, 64, nb, 1.0, V, ld, C, ld, 0.0, W, nb, w.gsm);
    cta_gemm<true, false, M_UPPER>(nb, 64, nb, 1.0, T, ld, W, nb, 0.0, W2, nb, w.gsm);
    cta_gemm<false, false, M_UNIT_LOWER>(nb, 64, nb, -1.0, V, ld, W2, nb, 1.0, C, ld, w.gsm);
}

// TSMQR strip (reference src/srcqr/dtsmqr.h -> dparfb.h -> dpamm.h, L = 0): the block
// reflector [I; V] T [I; V]^T applied as Q^T to [A1; A2] on a 64-column strip.  The
// reference forms W = A1 + V^T A2, W2 = T^T W, A1 -= W2, A2 -= V W2 with the whole NB x NB T
// (5 NB^2 flops per column).  Here the reflectors go in groups of 64, first to last: Q is the
// product of the groups' block reflectors, whose T factors are the 64 x 64 diagonal blocks of T
// (the compact WY form built forward, column by column), so for each group b
//   W = A1[b rows] + V[:, b]^T A2;  W2 = T_bb^T W;  A1[b rows] -= W2;  A2 -= V[:, b] W2
// gives the same transformation in 4 NB^2 + 64 NB flops per column (17 % fewer at NB = 512).
// W, W2: 64 x 64 scratch.
__device__ void tsmqr_strip(const Worker &w, double *A1, double *A2, const double *V, const double *T, int nb,
                            int ld, double *W, double *W2) {
    for (int b = 0; b < nb; b += 64) {
        const double *Vb = V + (size_t)b * ld;
        cta_axpby(64, 64, 1.0, A1 + b, ld, 0.0, W, 64);
        cta_gemm<true, false>(64, 64, nb, 1.0, Vb, ld, A2, ld, 1.0, W, 64, w.gsm);
        cta_gemm<true, false, M_UPPER>(64, 64, 64, 1.0, T + b + (size_t)b * ld, ld, W, 64, 0.0, W2, 64, w.gsm);
        cta_axpby(64, 64, -1.0, W2, 64, 1.0, A1 + b, ld);
        cta_gemm<false, false>(nb, 64, 64, -1.0, Vb, ld, W2, 64, 1.0, A2, ld, w.gsm);
    }
}

// ---------------------------------------------------------------------------------------
// Task dispatch
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ double *tile_ptr(double *A, int n, int nb, int m, int k) {
    return A + (size_t)nb * nb * ((size_t)m + (size_t)(n / nb) * k);
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

__device__ void run_task(const SchedParams &p, const Worker &w, const Task &t, int tid, double *wscr) {
    int n = p.n, nb = p.nb, bs = p.bs;
    double *A = p.A;
    if (p.mats) {
        const MatInfo mi = p.mats[t.mat];
        A = mi.A;
        n = mi.n;
        nb = mi.nb;
        bs = mi.bs;
    }
    const int ld = nb;
    switch (t.type) {
        case T_POTRF: {
            double *D = block_ptr(A, n, nb, bs, t.k, t.k);
            const int bad = potrf_upper(w, D, bs, ld);
            if (bad >= 0 && threadIdx.x == 0) {
                const long long r = (long long)t.k * bs + bad;
                record_error(p, -3 /*PALIAL_ERR_NOT_SPD*/, tid, (int)(r / nb), (int)(r / nb), (int)(r % nb));
            }
            break;
        }
        case T_TRSM_LUT: {
            const double *U = block_ptr(A, n, nb, bs, t.k, t.k);
            double *B = block_ptr(A, n, nb, bs, t.k, t.m) + (size_t)t.part * 64 * ld;
            trsm_lut(w, U, B, bs, ld);
            break;
        }
        case T_SYRK: {
            const double *X = block_ptr(A, n, nb, bs, t.k, t.m);
            double *C = block_ptr(A, n, nb, bs, t.m, t.m);
            const int c0 = t.part * 64;
            cta_gemm<true, false, M_NONE, M_NONE, true>(c0 + 64, 64, bs, -1.0, X, ld, X + (size_t)c0 * ld, ld, 1.0,
                                                        C + (size_t)c0 * ld, ld, w.gsm, c0);
            break;
        }
        case T_GEMM_TN: {
            const double *Xa = block_ptr(A, n, nb, bs, t.k, t.n);
            const double *Xb = block_ptr(A, n, nb, bs, t.k, t.m);
            double *C = block_ptr(A, n, nb, bs, t.n, t.m);
            const int c0 = t.part * 64;
            cta_gemm<true, false>(bs, 64, bs, -1.0, Xa, ld, Xb + (size_t)c0 * ld, ld, 1.0, C + (size_t)c0 * ld, ld,
                                  w.gsm);
            break;
        }
        case T_GETRF: {
            double *D = block_ptr(A, n, nb, bs, t.k, t.k);
            const int z = getrf_nopiv(w, D, bs, ld);
            if (z && threadIdx.x == 0) atomicOr(p.status + ST_ZEROPIV, 1);
            break;
        }
        case T_TRSM_RUN: {
            const double *U = block_ptr(A, n, nb, bs, t.k, t.k);
            double *B = block_ptr(A, n, nb, bs, t.m, t.k) + t.part * 64;
            trsm_run(w, U, B, bs, ld);
            break;
        }
        case T_TRSM_LLU: {
            const double *L = block_ptr(A, n, nb, bs, t.k, t.k);
            double *B = block_ptr(A, n, nb, bs, t.k, t.n) + (size_t)t.part * 64 * ld;
            trsm_llu(w, L, B, bs, ld);
            break;
        }
        case T_GEMM_NN: {
            const double *Xa = block_ptr(A, n, nb, bs, t.m, t.k);
            const double *Xb = block_ptr(A, n, nb, bs, t.k, t.n);
            double *C = block_ptr(A, n, nb, bs, t.m, t.n);
            const int c0 = t.part * 64;
            cta_gemm<false, false>(bs, 64, bs, -1.0, Xa, ld, Xb + (size_t)c0 * ld, ld, 1.0, C + (size_t)c0 * ld, ld,
                                   w.gsm);
            break;
        }
        case T_TRSM_LUN: {
            const double *U = block_ptr(A, n, nb, bs, t.k, t.k);
            double *B = block_ptr(A, n, nb, bs, t.k, t.n) + (size_t)t.part * 64 * ld;
            trsm_lun(w, U, B, bs, ld);
            break;
        }
        case T_GEQRT: {
            geqrt(w, tile_ptr(A, n, nb, t.k, t.k), nb, ld, tile_ptr(p.S, n, nb, t.k, t.k), ld);
            break;
        }
        case T_UNMQR: {
            double *C = tile_ptr(A, n, nb, t.k, t.n) + (size_t)t.part * 64 * ld;
            unmqr_strip(w, tile_ptr(A, n, nb, t.k, t.k), tile_ptr(p.S, n, nb, t.k, t.k), C, nb, ld, wscr,
                        wscr + (size_t)nb * 64);
            break;
        }
        case T_TSQRT: {
            tsqrt(w, tile_ptr(A, n, nb, t.k, t.k), tile_ptr(A, n, nb, t.m, t.k), nb, ld,
                  tile_ptr(p.S, n, nb, t.m, t.k), ld);
            break;
        }
        case T_TSMQR: {
            const size_t off = (size_t)t.part * 64 * ld;
            tsmqr_strip(w, tile_ptr(A, n, nb, t.k, t.n) + off, tile_ptr(A, n, nb, t.m, t.n) + off,
                        tile_ptr(A, n, nb, t.m, t.k), tile_ptr(p.S, n, nb, t.m, t.k), nb, ld, wscr,
                        wscr + (size_t)nb * 64);
            break;
        }
        default:
            break;
    }
}

// Persistent scheduler: launch with at most (SMs x resident CTAs) blocks of NT threads.
__global__ void __launch_bounds__(NT, 1) sched_f64_kernel(SchedParams p) {
    extern __shared__ __align__(16) double smem[];
    Worker w = make_worker(smem);
    __shared__ int s_task, s_abort;
    // worker-private scratch (QR strips)
    double *wscr = p.scratch + (long long)blockIdx.x * p.scratch_per_worker;
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
        run_task(p, w, t, tid, wscr);
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

// ---------------------------------------------------------------------------------------
// One whole tile task (all strips) on one CTA, for the single-tile C ABI entry points.
// p0..p3 are the tile arguments in the order of the reference's tile kernels; ld >= nb.
// scratch: two nb x 64 strips (QR update kernels).
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(NT, 1) tile_task_kernel(int type, int nb, int ld, double *p0, double *p1,
                                                          double *p2, double *p3, double *scratch, int *status) {
    extern __shared__ __align__(16) double smem[];
    Worker w = make_worker(smem);
    double *W = scratch;
    double *W2 = W + (size_t)nb * 64;
    const int parts = nb / 64;
    switch (type) {
        case T_POTRF: {
            const int bad = potrf_upper(w, p0, nb, ld);
            if (bad >= 0 && threadIdx.x == 0) {
                status[ST_COL] = bad;
                status[ST_CODE] = -3;
            }
            break;
        }
        case T_GETRF: {
            const int z = getrf_nopiv(w, p0, nb, ld);
            if (z && threadIdx.x == 0) status[ST_ZEROPIV] = 1;
            break;
        }
        case T_TRSM_LUT:
            for (int q = 0; q < parts; q++) trsm_lut(w, p0, p1 + (size_t)q * 64 * ld, nb, ld);
            break;
        case T_TRSM_RUN:
            for (int q = 0; q < parts; q++) trsm_run(w, p0, p1 + q * 64, nb, ld);
            break;
        case T_TRSM_LLU:
            for (int q = 0; q < parts; q++) trsm_llu(w, p0, p1 + (size_t)q * 64 * ld, nb, ld);
            break;
        case T_TRSM_LUN:
            for (int q = 0; q < parts; q++) trsm_lun(w, p0, p1 + (size_t)q * 64 * ld, nb, ld);
            break;
        case T_SYRK:
            for (int q = 0; q < parts; q++) {
                const int c0 = q * 64;
                cta_gemm<true, false, M_NONE, M_NONE, true>(c0 + 64, 64, nb, -1.0, p0, ld, p0 + (size_t)c0 * ld, ld,
                                                            1.0, p1 + (size_t)c0 * ld, ld, w.gsm, c0);
            }
            break;
        case T_GEMM_TN:
            cta_gemm<true, false>(nb, nb, nb, -1.0, p0, ld, p1, ld, 1.0, p2, ld, w.gsm);
            break;
        case T_GEMM_NN:
            cta_gemm<false, false>(nb, nb, nb, -1.0, p0, ld, p1, ld, 1.0, p2, ld, w.gsm);
            break;
        case T_GEQRT:
            geqrt(w, p0, nb, ld, p1, ld);
            break;
        case T_UNMQR:
            for (int q = 0; q < parts; q++)
                unmqr_strip(w, p0, p1, p2 + (size_t)q * 64 * ld, nb, ld, W, W2);
            break;
        case T_TSQRT:
            tsqrt(w, p0, p1, nb, ld, p2, ld);
            break;
        case T_TSMQR:
            for (int q = 0; q < parts; q++) {
                const size_t off = (size_t)q * 64 * ld;
                tsmqr_strip(w, p0 + off, p1 + off, p2, p3, nb, ld, W, W2);
            }
            break;
        default:
            break;
    }
}

// ---------------------------------------------------------------------------------------
// Host-side launch helpers (called from runtime.cu)
// ---------------------------------------------------------------------------------------
int sched_smem_bytes() { return SCHED_SMEM_BYTES; }

cudaError_t sched_configure() {
    cudaError_t e = cudaFuncSetAttribute(sched_f64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SCHED_SMEM_BYTES);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(tile_task_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SCHED_SMEM_BYTES);
}

cudaError_t tile_task_launch(int type, int nb, int ld, double *p0, double *p1, double *p2, double *p3, double *scratch,
                             int *status, cudaStream_t s) {
    note_launch();
    tile_task_kernel<<<1, NT, SCHED_SMEM_BYTES, s>>>(type, nb, ld, p0, p1, p2, p3, scratch, status);
    return cudaGetLastError();
}

int sched_occupancy() {
    int blocks = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, sched_f64_kernel, NT, SCHED_SMEM_BYTES);
    return blocks;
}

cudaError_t sched_launch(const SchedParams &p, int grid, cudaStream_t s) {
    note_launch();
    sched_f64_kernel<<<grid, NT, SCHED_SMEM_BYTES, s>>>(p);
    return cudaGetLastError();
}

// Scratch (doubles) the scheduler needs: per-worker strips for the QR update tasks.
long long sched_scratch_doubles(int alg, int n, int nb, int bs, int workers, long long *per_worker) {
    (void)n;
    (void)bs;
    const long long pw = (alg == 2 || alg == 3 || alg == 4) ? 2LL * nb * 64 : 0;
    if (per_worker) *per_worker = pw;
    return pw * workers;
}

}  // namespace palial
