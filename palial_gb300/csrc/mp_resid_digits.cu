// mp_resid_digits.cu -- R = B - A X (A FP64 tile matrix, X n x 16) at FP64-level accuracy on the
// tensor cores: the refinement's full residual without the FP32 issue limit of the compensated
// FP32 kernel.
//
// Every entry of A is written as a 48-bit integer V times 2^(sigma - 47) (|a| < 2^sigma, so
// |V| < 2^47), V = round(a * 2^(47 - sigma)), and V as six 8-bit digits c_0..c_5 (two's
// complement: c_0 signed in [-128, 127], the others in [0, 255]); X's column c likewise with
// 2^(tau_c - 47) (tau_c from max |x_c|), digits d_0..d_5.  Digits are exact BF16 values, their
// products (|c_p d_q| <= 2^16) exact in FP32, and the tensor core's FP32 sums of such products
// stay integers below 2^24 as long as at most 256 of them are added -- here the products of one
// weight s = p + q over a 32-term K chunk (at most 6 pairs x 32 terms x 2^16 < 2^24).  After every
// chunk the seven weights s = 0..6 are folded into two 64-bit integer accumulators per output
// (hi: s = 0..2, lo: s = 3..6); pairs with s > 6 are dropped (< 2^-51 of max|a| max|x| per
// product).  A x = 2^(sigma + tau_c - 62) (hi * 2^32 + lo), converted to FP64 once at the end.
//
// Error per entry of A x: A's and X's rounding to 48 bits (2^-48 relative to 2^sigma and
// 2^tau_c, round to nearest, so random in sign) and the dropped pairs (below 2^-51 per product,
// one sign): far below the refinement's targets (the FP64-level backward error 1e-14 * n).
//
// Layout: warp = 16 rows of A x all 16 right-hand sides, CTA = 4 warps (64 rows).  Per K16 step
// a thread loads the 8 FP64 entries of its mma.sync m16n8k16 A fragment straight from the tile
// layout (rows g, g + 8, columns 2t, 2t + 1, 2t + 8, 2t + 9 of the step), digitises them in
// registers (integer operations on the bit pattern, no FP64 pipe) and issues the 26 digit-pair
// MMAs per 8-column half of the 16 right-hand sides.  X's digits are prepared once per call in a
// fragment-ordered buffer (one 16-byte load per digit, half and chunk).  The next chunk's A
// entries are in flight while the current chunk computes.  Row sums of |a| (FP32) give
// ||A||_inf when asked for.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"

namespace palial {
namespace mrd {

constexpr int ND = 6;        // digits per operand (48 bits)
constexpr int SMAX = 6;      // largest kept weight s = p + q
constexpr int NT = 128;      // 4 warps x 16 rows
constexpr int KC = 32;       // K chunk between integer folds

// 48-bit rounded integer of v * 2^(47 - sc) (|v| < 2^sc), from the bit pattern; *bad set for
// Inf / NaN and for |v| >= 2^sc (a value the scale does not cover: the result is then
// reported as NaN instead of a wrapped integer).
__device__ __forceinline__ long long to_v48(double v, int sc, bool &bad) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
    const int E = (int)((bits >> 52) & 0x7FF);
    if (E == 0) return 0;  // zero or subnormal: below 2^-1022, far under 2^(sc - 48)
    const unsigned long long mant = (bits & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
    const int shift = 1028 + sc - E;  // >= 6 exactly when |v| < 2^sc
    bad |= (E == 0x7FF) | (shift < 6);
    if (shift >= 64 || shift < 6) return 0;
    const long long m = (long long)((mant + (1ull << (shift - 1))) >> shift);
    return (bits >> 63) ? -m : m;
}

// Digit p of a 48-bit two's complement integer as a float (exact).
__device__ __forceinline__ float digit(long long V, int p) {
    return p == 0 ? (float)(int)(V >> 40) : (float)(int)((V >> (40 - 8 * p)) & 255);
}

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);  // .x (low half) = lo
    return *reinterpret_cast<const uint32_t *>(&h);
}

__device__ __forceinline__ void mma16816(float *d, const uint32_t *a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// X digits in fragment order: word ((chunk * ND + q) * 16 + c) * 16 + t * 4 + j holds digits q
// of x(k, c) and x(k + 1, c), k = chunk * 32 + 2 (t + 4 j), as a BF16 pair (low half: k).  tau[c]:
// exponent of max |x_c| (frexp), 0 for columns beyond nrhs (their digits are 0).
__global__ void x_digits_kernel(const double *X, int n, int nrhs, const double *colmax, uint32_t *Xd, int *tau) {
    const long long words = (long long)(n / KC) * 16 * 16;  // per digit set: chunk x column x (t, j)
    for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < words;
         w += (long long)gridDim.x * blockDim.x) {
        const int tj = (int)(w & 15), c = (int)((w >> 4) & 15);
        const long long chunk = w >> 8;
        const int t = tj >> 2, j = tj & 3;
        const long long k = chunk * KC + 2 * (t + 4 * j);
        int tc = 0;
        long long v0 = 0, v1 = 0;
        if (c < nrhs) {
            frexp(colmax[c], &tc);
            bool bad = false;
            v0 = to_v48(X[(size_t)k + (size_t)c * n], tc, bad);
            v1 = to_v48(X[(size_t)k + 1 + (size_t)c * n], tc, bad);
        }
        if (w < 16 * 16 && tj == 0) tau[c] = tc;
#pragma unroll
        for (int q = 0; q < ND; q++)
            Xd[((chunk * ND + q) * 16 + c) * 16 + tj] = pack2(digit(v0, q), digit(v1, q));
    }
}

__global__ void __launch_bounds__(NT, 2) residual_digits_kernel(const double *A, int n, int nb, const uint32_t *Xd,
                                                                const int *tau, int sigma, const double *B, double *R,
                                                                int nrhs, double *amax) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int i0 = blockIdx.x * 64 + warp * 16;  // first row of this warp
    const int mt = n / nb;
    const double *rowbase = A + (size_t)nb * nb * (size_t)(i0 / nb) + (size_t)(i0 % nb);
    // element (i0 + r, k) at rowbase + r + nb^2 mt (k / nb) + (k % nb) nb
    auto addr = [&](int r, int k) {
        return rowbase + (size_t)r + (size_t)nb * nb * (size_t)mt * (size_t)(k / nb) + (size_t)(k % nb) * nb;
    };
    long long hi[2][4], lo[2][4];
#pragma unroll
    for (int h = 0; h < 2; h++)
#pragma unroll
        for (int e = 0; e < 4; e++) hi[h][e] = lo[h][e] = 0;
    // |a| row sums of rows g and g + 8 over this thread's columns, in units of 2^(sigma - 23)
    // (from V >> 24, exact in FP32: the norm needs no more than FP32 accuracy)
    float asum0 = 0.f, asum1 = 0.f;
    const bool want_norm = amax != nullptr;
    bool bad = false;
    // a fragment entries of one K16 step: rows g, g+8 x columns 2t, 2t+1, 2t+8, 2t+9
    double cur[2][8], nxt[2][8];
    auto load_chunk = [&](int k0, double (&v)[2][8]) {
#pragma unroll
        for (int s = 0; s < 2; s++) {
            const int kk = k0 + 16 * s + 2 * t;
            v[s][0] = __ldcs(addr(g, kk));
            v[s][1] = __ldcs(addr(g, kk + 1));
            v[s][2] = __ldcs(addr(g + 8, kk));
            v[s][3] = __ldcs(addr(g + 8, kk + 1));
            v[s][4] = __ldcs(addr(g, kk + 8));
            v[s][5] = __ldcs(addr(g, kk + 9));
            v[s][6] = __ldcs(addr(g + 8, kk + 8));
            v[s][7] = __ldcs(addr(g + 8, kk + 9));
        }
    };
    load_chunk(0, cur);
    for (int k0 = 0; k0 < n; k0 += KC) {
        if (k0 + KC < n) load_chunk(k0 + KC, nxt);
        float acc[SMAX + 1][2][4];
#pragma unroll
        for (int s = 0; s <= SMAX; s++)
#pragma unroll
            for (int h = 0; h < 2; h++)
#pragma unroll
                for (int e = 0; e < 4; e++) acc[s][h][e] = 0.f;
        // X digit fragments of this chunk: per digit q and half h, words j = 0..3 (k pairs t + 4j)
        const uint4 *xq = reinterpret_cast<const uint4 *>(Xd) + ((size_t)(k0 / KC) * ND * 16) * 4;
#pragma unroll
        for (int st = 0; st < 2; st++) {
            // this step's A digit fragments
            long long V[8];
#pragma unroll
            for (int e = 0; e < 8; e++) {
                V[e] = to_v48(cur[st][e], sigma, bad);
                if (want_norm) {
                    const float m = fabsf((float)(int)(V[e] >> 24));
                    if (e == 0 || e == 1 || e == 4 || e == 5) asum0 += m;
                    else asum1 += m;
                }
            }
            uint32_t af[ND][4];
#pragma unroll
            for (int p = 0; p < ND; p++) {
                af[p][0] = pack2(digit(V[0], p), digit(V[1], p));  // row g,   k 2t, 2t+1
                af[p][1] = pack2(digit(V[2], p), digit(V[3], p));  // row g+8
                af[p][2] = pack2(digit(V[4], p), digit(V[5], p));  // row g,   k 2t+8, 2t+9
                af[p][3] = pack2(digit(V[6], p), digit(V[7], p));  // row g+8
            }
#pragma unroll
            for (int h = 0; h < 2; h++) {
#pragma unroll
                for (int q = 0; q < ND; q++) {
                    // B fragment: k pairs (t) and (t + 4) of step st -> words j = 2 st, 2 st + 1
                    const uint4 w = __ldg(xq + (size_t)(q * 16 + h * 8 + g) * 4 + t);
                    const uint32_t b0 = st == 0 ? w.x : w.z, b1 = st == 0 ? w.y : w.w;
#pragma unroll
                    for (int p = 0; p + q <= SMAX && p < ND; p++) mma16816(acc[p + q][h], af[p], b0, b1);
                }
            }
        }
        // fold the chunk's exact FP32 sums into the 64-bit accumulators
#pragma unroll
        for (int h = 0; h < 2; h++)
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const long long s0 = __float2int_rn(acc[0][h][e]), s1 = __float2int_rn(acc[1][h][e]),
                                s2 = __float2int_rn(acc[2][h][e]), s3 = __float2int_rn(acc[3][h][e]),
                                s4 = __float2int_rn(acc[4][h][e]), s5 = __float2int_rn(acc[5][h][e]),
                                s6 = __float2int_rn(acc[6][h][e]);
                hi[h][e] += (s0 << 16) + (s1 << 8) + s2;
                lo[h][e] += (s3 << 24) + (s4 << 16) + (s5 << 8) + s6;
            }
        if (k0 + KC < n) {
#pragma unroll
            for (int s = 0; s < 2; s++)
#pragma unroll
                for (int e = 0; e < 8; e++) cur[s][e] = nxt[s][e];
        }
    }
    // outputs: rows g (e = 0, 1) and g + 8 (e = 2, 3), columns h * 8 + 2t + (e & 1)
#pragma unroll
    for (int h = 0; h < 2; h++)
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int c = h * 8 + 2 * t + (e & 1);
            if (c >= nrhs) continue;
            const int row = i0 + g + (e >> 1) * 8;
            double ax = ldexp((double)hi[h][e] * 4294967296.0 + (double)lo[h][e], sigma + tau[c] - 62);
            if (bad) ax = __longlong_as_double(0x7ff8000000000000ll);
            const size_t o = (size_t)row + (size_t)c * n;
            R[o] = B ? B[o] - ax : ax;
        }
    if (amax) {
        // row sums over the 4 threads of a row group, then the warp's largest row
        for (int o = 1; o < 4; o <<= 1) {
            asum0 += __shfl_xor_sync(0xffffffffu, asum0, o);
            asum1 += __shfl_xor_sync(0xffffffffu, asum1, o);
        }
        double m = ldexp(fmax((double)asum0, (double)asum1), sigma - 23);
        for (int o = 4; o < 32; o <<= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (bad) m = __longlong_as_double(0x7ff8000000000000ll);
        if (lane == 0) atomicMax(reinterpret_cast<unsigned long long *>(amax), (unsigned long long)__double_as_longlong(m));
    }
}

}  // namespace mrd

// R = B - A X (B may be NULL: R = A X) with the digit products above; sigma: |a_ij| < 2^sigma;
// colmax = per-column max |x|; Xd (n * 48 words) and tau (16 ints) are scratch.  n % 64 == 0.
cudaError_t mrd_residual(const double *A, int n, int nb, const double *X, const double *colmax, const double *B,
                         double *R, int nrhs, int sigma, uint32_t *Xd, int *tau, double *amax, cudaStream_t s) {
    // the 64-bit accumulators hold n / 32 chunk sums of up to 2^49: n <= 2^18
    if (n % 64 || n > (1 << 18) || nrhs < 1 || nrhs > 16) return cudaErrorInvalidValue;
    note_launch();
    mrd::x_digits_kernel<<<1024, 256, 0, s>>>(X, n, nrhs, colmax, Xd, tau);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    note_launch();
    mrd::residual_digits_kernel<<<n / 64, mrd::NT, 0, s>>>(A, n, nb, Xd, tau, sigma, B, R, nrhs, amax);
    return cudaGetLastError();
}

}  // namespace palial
