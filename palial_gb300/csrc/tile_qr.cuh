// tile_qr.cuh -- the flat-tree TS QR tile routines of the reference (src/qr.h tasks over
// src/srcqr: GEQRT = dgeqr2 + dlarft, UNMQR = dlarfb, TSQRT, TSMQR = dparfb/dpamm) for one CTA
// of 256 threads, on element type T.  The mixed-precision QR runs them in FP32 inside the FP32
// task scheduler.  They restate the published algorithms (LAPACK dlarfg / dlarft 'F','C' /
// dlarfb 'L','T','F','C'; the TS kernels of tile QR; the compact-WY merge of Schreiber and Van
// Loan) with the output layout of the FP64 routines of sched_f64.cu: R in the upper triangle,
// V below the diagonal (unit implicit) and in the full TSQRT tiles, T upper triangular in S.
// GEQRT and TSQRT are blocked by 64-column panels (the same reflectors and T as the unblocked
// column sweep up to rounding): the per-column, latency-bound work stays inside a panel and the
// rest runs as CTA GEMMs.
#pragma once
#include <cfloat>

#include "common.cuh"
#include "tc_gemm.cuh"

namespace palial {
namespace qrt {

constexpr int NT = 256;          // threads per CTA
constexpr int BM = 64;           // output sub-block of cta_gemm
constexpr int KC = 32;           // K chunk staged in shared memory
constexpr int SP = BM + 4;       // shared pitch
constexpr int GEMM_SMEM = 2 * KC * SP;  // elements of T used by cta_gemm
constexpr int RED = 1024 + 64;   // reduction / larft scratch (elements of T), nb <= 1016
constexpr int MAX_NB = 512;      // tau array

enum Mask { M_NONE = 0, M_UPPER = 1, M_UNIT_LOWER = 2 };

template <class T>
struct Lim;
template <>
struct Lim<float> {
    __device__ static float sfmin() { return FLT_MIN; }
    __device__ static float eps() { return 5.9604644775390625e-08f; }  // 2^-24, slamch('E')
};
template <>
struct Lim<double> {
    __device__ static double sfmin() { return 2.2250738585072014e-308; }
    __device__ static double eps() { return 1.1102230246251565e-16; }  // 2^-53, dlamch('E')
};

template <class T>
__device__ __forceinline__ T ldg(const T *p) {
    return __ldcg(p);  // tiles are written by other SMs: bypass L1
}

// Stored element (r, c) under a mask; the masked-out triangle is never read.
template <class T, int MASK>
__device__ __forceinline__ T masked_ld(const T *p, int r, int c) {
    if (MASK == M_UPPER) return r > c ? T(0) : ldg(p);
    if (MASK == M_UNIT_LOWER) return r < c ? T(0) : (r == c ? T(1) : ldg(p));
    return ldg(p);
}

// Shared memory of one worker for the QR routines.
template <class T>
struct QrSmem {
    T *gsm;  // GEMM_SMEM
    T *red;  // RED
    T *tau;  // MAX_NB
};

// Stage op(X)[i0:i0+64, p0:p0+KC] into Xs[p][i]; TX: element (i, p) of op(X) at X[p + i*ld],
// else at X[i + p*ld].  MASK refers to X's stored coordinates; p >= klim reads as zero.
template <class T, bool TX, int MASK>
__device__ __forceinline__ void stage(T (*Xs)[SP], const T *X, int ld, int i0, int p0, int klim) {
#pragma unroll
    for (int q = 0; q < (64 * KC) / NT; q++) {
        const int e = (int)threadIdx.x + q * NT;
        if (!TX) {
            const int p = e >> 6, i = e & 63;  // consecutive threads: consecutive rows
            Xs[p][i] = (p0 + p < klim) ? masked_ld<T, MASK>(X + (size_t)(i0 + i) + (size_t)(p0 + p) * ld, i0 + i, p0 + p)
                                       : T(0);
        } else {
            const int p = e & 31, i = e >> 5;  // consecutive threads: consecutive p
            Xs[p][i] = (p0 + p < klim) ? masked_ld<T, MASK>(X + (size_t)(p0 + p) + (size_t)(i0 + i) * ld, p0 + p, i0 + i)
                                       : T(0);
        }
    }
}

// C[M x N] = beta C + alpha op(A) op(B), M, N multiples of 64, K a multiple of 32.  TA: op(A) =
// A^T (A stored K x M); TB: op(B) = B^T (B stored N x K).  MA / MB: triangular masks on the
// stored operands (the K range shrinks to where op(A) is nonzero).  Ends synced.
template <class T, bool TA, bool TB, int MA = M_NONE, int MB = M_NONE>
__device__ void cta_gemm(int M, int N, int K, T alpha, const T *A, int lda, const T *B, int ldb, T beta, T *C,
                         int ldc, T *smem, bool tc = false) {
    T(*As)[SP] = reinterpret_cast<T(*)[SP]>(smem);
    T(*Bs)[SP] = reinterpret_cast<T(*)[SP]>(smem + KC * SP);
    if constexpr (sizeof(T) == 4) {
        if (tc) {  // FP32 data: the products on the warp tensor cores in BF16x3 (tc_gemm.cuh)
            for (int i0 = 0; i0 < M; i0 += BM) {
                int klo = 0, khi = K;
                if (MA == M_UPPER) {
                    if (TA) khi = min(K, i0 + BM);
                    else klo = i0;
                } else if (MA == M_UNIT_LOWER) {
                    if (TA) klo = i0;
                    else khi = min(K, i0 + BM);
                }
                klo = (klo / KC) * KC;
                for (int j0 = 0; j0 < N; j0 += BM) {
                    tcg::Frag f;
                    tcg::zero(f);
                    for (int p0 = klo; p0 < khi; p0 += KC) {
                        stage<T, TA, MA>(As, A, lda, i0, p0, K);
                        stage<T, !TB, MB>(Bs, B, ldb, j0, p0, K);
                        __syncthreads();
                        tcg::bf16x3_chunk<SP>(reinterpret_cast<const float *>(&As[0][0]),
                                              reinterpret_cast<const float *>(&Bs[0][0]), f);
                        __syncthreads();
                    }
                    T cv[4][4];
#pragma unroll
                    for (int nt = 0; nt < 4; nt++)
#pragma unroll
                        for (int e = 0; e < 4; e++) {
                            int r, c;
                            tcg::frag_coord(nt, e, r, c);
                            cv[nt][e] = beta == T(0) ? T(0) : ldg(C + (size_t)(i0 + r) + (size_t)(j0 + c) * ldc);
                        }
#pragma unroll
                    for (int nt = 0; nt < 4; nt++)
#pragma unroll
                        for (int e = 0; e < 4; e++) {
                            int r, c;
                            tcg::frag_coord(nt, e, r, c);
                            const T v = alpha * f.acc[nt][e];
                            C[(size_t)(i0 + r) + (size_t)(j0 + c) * ldc] = beta == T(0) ? v : fma(beta, cv[nt][e], v);
                        }
                }
            }
            __syncthreads();
            return;
        }
    }
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    for (int i0 = 0; i0 < M; i0 += BM) {
        int klo = 0, khi = K;
        if (MA == M_UPPER) {
            if (TA) khi = min(K, i0 + BM);  // op(A)(i, p) = X(p, i): p <= i
            else klo = i0;                  // X(i, p): i <= p
        } else if (MA == M_UNIT_LOWER) {
            if (TA) klo = i0;               // X(p, i): p >= i
            else khi = min(K, i0 + BM);     // X(i, p): i >= p
        }
        klo = (klo / KC) * KC;
        for (int j0 = 0; j0 < N; j0 += BM) {
            T acc[4][4];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) acc[a][b] = T(0);
            for (int p0 = klo; p0 < khi; p0 += KC) {
                stage<T, TA, MA>(As, A, lda, i0, p0, K);
                stage<T, !TB, MB>(Bs, B, ldb, j0, p0, K);
                __syncthreads();
#pragma unroll 8
                for (int p = 0; p < KC; p++) {
                    T av[4], bv[4];
#pragma unroll
                    for (int a = 0; a < 4; a++) av[a] = As[p][ty * 4 + a];
#pragma unroll
                    for (int b = 0; b < 4; b++) bv[b] = Bs[p][tx * 4 + b];
#pragma unroll
                    for (int a = 0; a < 4; a++)
#pragma unroll
                        for (int b = 0; b < 4; b++) acc[a][b] = fma(av[a], bv[b], acc[a][b]);
                }
                __syncthreads();
            }
            // every load of the output block before any store
            T cv[4][4];
#pragma unroll
            for (int b = 0; b < 4; b++)
#pragma unroll
                for (int a = 0; a < 4; a++)
                    cv[a][b] = beta == T(0) ? T(0)
                                            : ldg(C + (size_t)(i0 + ty * 4 + a) + (size_t)(j0 + tx * 4 + b) * ldc);
#pragma unroll
            for (int b = 0; b < 4; b++)
#pragma unroll
                for (int a = 0; a < 4; a++) {
                    const T v = alpha * acc[a][b];
                    C[(size_t)(i0 + ty * 4 + a) + (size_t)(j0 + tx * 4 + b) * ldc] =
                        beta == T(0) ? v : fma(beta, cv[a][b], v);
                }
        }
    }
    __syncthreads();
}

// Y[M x N] = alpha X + beta Y (column-major), loads before stores.  Ends synced.
template <class T>
__device__ void cta_axpby(int M, int N, T alpha, const T *X, int ldx, T beta, T *Y, int ldy) {
    for (int e0 = threadIdx.x; e0 < M * N; e0 += 4 * NT) {
        T xv[4], yv[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int e = e0 + q * NT;
            if (e < M * N) {
                const int i = e % M, j = e / M;
                xv[q] = ldg(X + (size_t)i + (size_t)j * ldx);
                yv[q] = beta == T(0) ? T(0) : ldg(Y + (size_t)i + (size_t)j * ldy);
            }
        }
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int e = e0 + q * NT;
            if (e < M * N) {
                const int i = e % M, j = e / M;
                Y[(size_t)i + (size_t)j * ldy] = beta == T(0) ? alpha * xv[q] : fma(alpha, xv[q], beta * yv[q]);
            }
        }
    }
    __syncthreads();
}

template <class T>
__device__ T block_sum(T *red, T v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    T s = T(0);
#pragma unroll
    for (int i = 0; i < NT / 32; i++) s += red[i];
    __syncthreads();
    return s;
}

template <class T>
__device__ T block_absmax(T *red, T v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    T s = T(0);
#pragma unroll
    for (int i = 0; i < NT / 32; i++) s = fmax(s, red[i]);
    __syncthreads();
    return s;
}

template <class T>
__device__ __forceinline__ T lapy2(T x, T y) {
    const T xa = fabs(x), ya = fabs(y);
    const T w = fmax(xa, ya), z = fmin(xa, ya);
    if (z == T(0)) return w;
    const T q = z / w;
    return w * sqrt(T(1) + q * q);
}

// ||x||_2 with scaling by max |x| (no overflow or underflow), all threads.
template <class T>
__device__ T norm2_block(T *red, const T *x, int m) {
    T mx = T(0);
    for (int r = threadIdx.x; r < m; r += NT) mx = fmax(mx, fabs(ldg(x + r)));
    const T scale = block_absmax(red, mx);
    if (scale == T(0)) return T(0);
    const T inv = T(1) / scale;
    T s = T(0);
    for (int r = threadIdx.x; r < m; r += NT) {
        const T q = ldg(x + r) * inv;
        s = fma(q, q, s);
    }
    return scale * sqrt(block_sum(red, s));
}

// Householder generation (LAPACK dlarfg): (I - tau v v^T) [alpha; x] = [beta; 0],
// beta = -sign(alpha) ||[alpha; x]||, v = [1; x / (alpha - beta)]; x overwritten by v's tail,
// beta written to *alpha_p; returns tau (0: H = I).  All threads.
template <class T>
__device__ T larfg(T *red, T *alpha_p, T *x, int m) {
    const T safmin = Lim<T>::sfmin() / Lim<T>::eps();
    T alpha = ldg(alpha_p);
    T xnorm = norm2_block(red, x, m);
    if (xnorm == T(0)) return T(0);
    T beta = -copysign(lapy2(alpha, xnorm), alpha);
    int knt = 0;
    if (fabs(beta) < safmin) {
        const T rs = T(1) / safmin;
        do {
            knt++;
            for (int r = threadIdx.x; r < m; r += NT) x[r] = ldg(x + r) * rs;
            __syncthreads();
            beta *= rs;
            alpha *= rs;
        } while (fabs(beta) < safmin && knt < 20);
        xnorm = norm2_block(red, x, m);
        beta = -copysign(lapy2(alpha, xnorm), alpha);
    }
    const T tau = (beta - alpha) / beta;
    const T sc = T(1) / (alpha - beta);
    for (int r = threadIdx.x; r < m; r += NT) x[r] = ldg(x + r) * sc;
    for (int j = 0; j < knt; j++) beta *= safmin;
    __syncthreads();
    if (threadIdx.x == 0) *alpha_p = beta;
    __syncthreads();
    return tau;
}

// One reflector on column cj by one warp: s = head + <v, cj(r0:nb)> with v = ci(r0:nb) and head
// = the column's entry at the reflector's unit position (*hj, updated too); cj(r0:nb) += (-tau
// s) v.  Up to 16 entries per lane stay in registers between the dot product and the update.
template <class T>
__device__ __forceinline__ void reflect_col(const T *ci, T *cj, T *hj, int r0, int nb, T tau, int lane) {
    constexpr int U = 16;
    T s = (lane == 0) ? ldg(hj) : T(0);
    if (nb - r0 <= 32 * U) {
        T vi[U], vj[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int r = r0 + lane + 32 * u;
            vi[u] = r < nb ? ldg(ci + r) : T(0);
            vj[u] = r < nb ? ldg(cj + r) : T(0);
        }
#pragma unroll
        for (int u = 0; u < U; u++) s = fma(vi[u], vj[u], s);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        const T f = -tau * s;
        if (lane == 0) *hj = ldg(hj) + f;
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int r = r0 + lane + 32 * u;
            if (r < nb) cj[r] = fma(f, vi[u], vj[u]);
        }
        return;
    }
    for (int b = r0 + lane; b < nb; b += 32 * U) {
        // dot product pass (columns longer than 32 U entries take several passes)
        T vi[U], vj[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int r = b + 32 * u;
            vi[u] = r < nb ? ldg(ci + r) : T(0);
            vj[u] = r < nb ? ldg(cj + r) : T(0);
        }
#pragma unroll
        for (int u = 0; u < U; u++) s = fma(vi[u], vj[u], s);
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    const T f = -tau * s;
    if (lane == 0) *hj = ldg(hj) + f;
    for (int b = r0 + lane; b < nb; b += 32 * U) {
        T vi[U], vj[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int r = b + 32 * u;
            vi[u] = r < nb ? ldg(ci + r) : T(0);
            vj[u] = r < nb ? ldg(cj + r) : T(0);
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int r = b + 32 * u;
            if (r < nb) cj[r] = fma(f, vi[u], vj[u]);
        }
    }
}

// T (upper, nb x nb, ldt) of the forward column-wise compact WY form (dlarft 'F','C'):
// T(i,i) = tau_i, T(0:i,i) = -tau_i T(0:i,0:i) z, z_j = <v_j, v_i> (j < i) from dot(j, i, lane)
// evaluated by one warp.
template <class T, class Dot>
__device__ void larft(T *red, int nb, const T *tau, T *Tm, int ldt, Dot dot) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T *z = red + 8;
    for (int i = 0; i < nb; i++) {
        const T ti = tau[i];
        for (int j = warp; j < i; j += NT / 32) {
            T s = dot(j, i, lane);
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) z[j] = -ti * s;
        }
        __syncthreads();
        for (int r = threadIdx.x; r < i; r += NT) {
            T s = T(0);
            for (int p = r; p < i; p++) s = fma(ldg(Tm + r + (size_t)p * ldt), z[p], s);
            Tm[r + (size_t)i * ldt] = s;
        }
        if (threadIdx.x == 0) Tm[i + (size_t)i * ldt] = ti;
        __syncthreads();
    }
}

// Off-diagonal 64-blocks of the full compact-WY T after the panels: for every block column
// Q (q0 = 64 Q), with the diagonal blocks T_Q already in place,
//     T(0:q0, Q) = -T(0:q0, 0:q0) (Y_{0:q0}^T Y_Q) T_Q
// (the product of two compact-WY blocks, Schreiber and Van Loan).  ytq(q0, Ys, ldy) writes
// Y_{0:q0}^T Y_Q (q0 x 64) into Ys.  scr: two nb x 64 scratch blocks.
template <class T, class YtQ>
__device__ void assemble_t(const QrSmem<T> &w, int nb, T *Tm, int ldt, T *scr, YtQ ytq) {
    T *Ys = scr, *Y2 = scr + (size_t)nb * 64;
    for (int q0 = 64; q0 < nb; q0 += 64) {
        ytq(q0, Ys, nb);
        // Y2 = Ys T_Q (T_Q upper 64 x 64)
        cta_gemm<T, false, false, M_NONE, M_UPPER>(q0, 64, 64, T(1), Ys, nb, Tm + q0 + (size_t)q0 * ldt, ldt, T(0),
                                                   Y2, nb, w.gsm);
        // T(0:q0, Q) = -T(0:q0, 0:q0) Y2 (upper)
        cta_gemm<T, false, false, M_UPPER>(q0, 64, q0, T(-1), Tm, ldt, Y2, nb, T(0), Tm + (size_t)q0 * ldt, ldt, w.gsm);
    }
}

// GEQRT of an nb x nb tile (nb a multiple of 64): Householder QR blocked by 64-column panels.
// Each panel is factored column by column (dlarfg, reflectors applied inside the panel only),
// its 64 x 64 T block built (dlarft), and the trailing columns updated by the panel's block
// reflector with CTA GEMMs (dlarfb); the full T is assembled at the end.  Output as the
// unblocked dgeqr2 + dlarft: R upper, V below the diagonal (unit implicit), T upper in Tm.
// scr: two nb x 64 scratch blocks.
template <class T>
__device__ void geqrt(const QrSmem<T> &w, T *A, int nb, int ld, T *Tm, int ldt, T *scr) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T *W = scr, *W2 = scr + (size_t)nb * 64;
    for (int p0 = 0; p0 < nb; p0 += 64) {
        for (int i = p0; i < p0 + 64; i++) {
            T *ci = A + (size_t)i * ld;
            const T ti = larfg(w.red, ci + i, ci + i + 1, nb - i - 1);
            if (threadIdx.x == 0) w.tau[i] = ti;
            if (ti != T(0)) {
                for (int j = i + 1 + warp; j < p0 + 64; j += NT / 32) {
                    T *cj = A + (size_t)j * ld;
                    reflect_col(ci, cj, cj + i, i + 1, nb, ti, lane);
                }
            }
            __syncthreads();
        }
        // panel T: z_j = <v_j, v_i> = A(i, j) + sum_{r > i} A(r, j) A(r, i), j < i (global indices)
        larft(w.red, 64, w.tau + p0, Tm + p0 + (size_t)p0 * ldt, ldt, [&](int j, int i, int ln) {
            const T *cj = A + (size_t)(p0 + j) * ld, *ci = A + (size_t)(p0 + i) * ld;
            T s = (ln == 0) ? ldg(cj + p0 + i) : T(0);
            for (int r = p0 + i + 1 + ln; r < nb; r += 32) s = fma(ldg(cj + r), ldg(ci + r), s);
            return s;
        });
        const int ncols = nb - p0 - 64;
        if (ncols > 0) {
            // C <- C - V T^T V^T C on the trailing columns (rows p0 .. nb - 1)
            const T *V = A + p0 + (size_t)p0 * ld;
            T *C = A + p0 + (size_t)(p0 + 64) * ld;
            const T *Tp = Tm + p0 + (size_t)p0 * ldt;
            cta_gemm<T, true, false, M_UNIT_LOWER>(64, ncols, nb - p0, T(1), V, ld, C, ld, T(0), W, 64, w.gsm);
            cta_gemm<T, true, false, M_UPPER>(64, ncols, 64, T(1), Tp, ldt, W, 64, T(0), W2, 64, w.gsm);
            cta_gemm<T, false, false, M_UNIT_LOWER>(nb - p0, ncols, 64, T(-1), V, ld, W2, 64, T(1), C, ld, w.gsm);
        }
    }
    // Y_a^T Y_Q: V_Q is zero above row q0 and unit on its diagonal block
    assemble_t(w, nb, Tm, ldt, scr, [&](int q0, T *Ys, int ldy) {
        cta_gemm<T, true, false, M_NONE, M_UNIT_LOWER>(q0, 64, nb - q0, T(1), A + q0, ld, A + q0 + (size_t)q0 * ld, ld,
                                                       T(0), Ys, ldy, w.gsm);
    });
}

// TSQRT: QR of [R = A1 upper; A2], blocked like geqrt: panels of 64 columns factored column
// by column (A2 becomes V, A1's upper triangle R), trailing columns of [A1; A2] updated by the
// panel's block reflector [E; V] (E: rows p0 .. p0 + 63 of A1), T assembled at the end.  A1's
// strictly lower part (the GEQRT reflectors) is neither read nor written.  scr: two nb x 64
// scratch blocks.
template <class T>
__device__ void tsqrt(const QrSmem<T> &w, T *A1, T *A2, int nb, int ld, T *Tm, int ldt, T *scr) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T *W = scr, *W2 = scr + (size_t)nb * 64;
    for (int p0 = 0; p0 < nb; p0 += 64) {
        for (int i = p0; i < p0 + 64; i++) {
            T *vi = A2 + (size_t)i * ld;
            const T ti = larfg(w.red, A1 + i + (size_t)i * ld, vi, nb);
            if (threadIdx.x == 0) w.tau[i] = ti;
            if (ti != T(0)) {
                for (int j = i + 1 + warp; j < p0 + 64; j += NT / 32)
                    reflect_col(vi, A2 + (size_t)j * ld, A1 + i + (size_t)j * ld, 0, nb, ti, lane);
            }
            __syncthreads();
        }
        // panel T: the identity parts are orthogonal, z_j = <A2(:, j), A2(:, i)>
        larft(w.red, 64, w.tau + p0, Tm + p0 + (size_t)p0 * ldt, ldt, [&](int j, int i, int ln) {
            const T *cj = A2 + (size_t)(p0 + j) * ld, *ci = A2 + (size_t)(p0 + i) * ld;
            T s = T(0);
            for (int r = ln; r < nb; r += 32) s = fma(ldg(cj + r), ldg(ci + r), s);
            return s;
        });
        const int ncols = nb - p0 - 64;
        if (ncols > 0) {
            // W = C1 + V^T C2; W2 = T^T W; C1 -= W2; C2 -= V W2
            const T *V = A2 + (size_t)p0 * ld;
            T *C1 = A1 + p0 + (size_t)(p0 + 64) * ld, *C2 = A2 + (size_t)(p0 + 64) * ld;
            const T *Tp = Tm + p0 + (size_t)p0 * ldt;
            cta_axpby<T>(64, ncols, T(1), C1, ld, T(0), W, 64);
            cta_gemm<T, true, false>(64, ncols, nb, T(1), V, ld, C2, ld, T(1), W, 64, w.gsm);
            cta_gemm<T, true, false, M_UPPER>(64, ncols, 64, T(1), Tp, ldt, W, 64, T(0), W2, 64, w.gsm);
            cta_axpby<T>(64, ncols, T(-1), W2, 64, T(1), C1, ld);
            cta_gemm<T, false, false>(nb, ncols, 64, T(-1), V, ld, W2, 64, T(1), C2, ld, w.gsm);
        }
    }
    // Y_a^T Y_Q = V_a^T V_Q (the identity parts touch disjoint rows of A1)
    assemble_t(w, nb, Tm, ldt, scr, [&](int q0, T *Ys, int ldy) {
        cta_gemm<T, true, false>(q0, 64, nb, T(1), A2, ld, A2 + (size_t)q0 * ld, ld, T(0), Ys, ldy, w.gsm);
    });
}

// UNMQR strip (dlarfb 'L','T','F','C'): C <- C - V T^T V^T C on a 64-column strip; W, W2 are
// nb x 64 scratch.
template <class T>
__device__ void unmqr_strip(const QrSmem<T> &w, const T *V, const T *Tm, T *C, int nb, int ld, T *W, T *W2) {
    cta_gemm<T, true, false, M_UNIT_LOWER>(nb, 64, nb, T(1), V, ld, C, ld, T(0), W, nb, w.gsm);
    cta_gemm<T, true, false, M_UPPER>(nb, 64, nb, T(1), Tm, ld, W, nb, T(0), W2, nb, w.gsm);
    cta_gemm<T, false, false, M_UNIT_LOWER>(nb, 64, nb, T(-1), V, ld, W2, nb, T(1), C, ld, w.gsm);
}

// TSMQR strip: Q^T = (I - [I; V] T [I; V]^T)^T applied to [A1; A2] on a 64-column strip, the
// reflectors in groups of 64, first to last, each with its 64 x 64 diagonal block of T (the T
// factor of that group in the forward column-wise compact WY form):
//   W = A1[b rows] + V[:, b]^T A2;  W2 = T_bb^T W;  A1[b rows] -= W2;  A2 -= V[:, b] W2.
// The same transformation as W = A1 + V^T A2, W2 = T^T W, A1 -= W2, A2 -= V W2 with the whole
// T, in 4 NB^2 + 64 NB instead of 5 NB^2 flops per column.  W, W2: 64 x 64 scratch.
// tc: FP32 data only, the two products with the dense V on the warp tensor cores (BF16x3); the
// triangular T product stays in FP32.
template <class T>
__device__ void tsmqr_strip(const QrSmem<T> &w, T *A1, T *A2, const T *V, const T *Tm, int nb, int ld, T *W,
                            T *W2, bool tc = false) {
    for (int b = 0; b < nb; b += 64) {
        const T *Vb = V + (size_t)b * ld;
        cta_axpby<T>(64, 64, T(1), A1 + b, ld, T(0), W, 64);
        cta_gemm<T, true, false>(64, 64, nb, T(1), Vb, ld, A2, ld, T(1), W, 64, w.gsm, tc);
        cta_gemm<T, true, false, M_UPPER>(64, 64, 64, T(1), Tm + b + (size_t)b * ld, ld, W, 64, T(0), W2, 64, w.gsm);
        cta_axpby<T>(64, 64, T(-1), W2, 64, T(1), A1 + b, ld);
        cta_gemm<T, false, false>(nb, 64, 64, T(-1), Vb, ld, W2, 64, T(1), A2, ld, w.gsm, tc);
    }
}

}  // namespace qrt
}  // namespace palial
