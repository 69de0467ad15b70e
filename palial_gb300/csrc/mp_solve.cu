// mp_solve.cu -- FP32/FP64 kernels of the mixed-precision factorizations and of iterative
// refinement: precision conversions, panel triangular solves (FP32 SIMT), blocked triangular
// solves of the refinement corrections with the low-precision factors, the FP64 residual
// r = b - A x on the FP64 tile-layout matrix, and the norms of the backward error.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"
#include "tile_f32.cuh"

namespace palial {
namespace mps {
using namespace f32;

constexpr int SMEM_FLOATS = 2 * 64 * DP + GEMM_SMEM_FLOATS;  // Ds | Bs | gemm staging
constexpr int SMEM_BYTES = SMEM_FLOATS * 4;

__device__ __forceinline__ size_t tile_off(int n, int nb, int tm, int tn) {
    return (size_t)nb * nb * ((size_t)tm + (size_t)(n / nb) * tn);
}

// ---- conversions --------------------------------------------------------------------------
// W = float(A (+ shift on the diagonal)); amax (optional, zeroed by the caller) receives
// max |a_ij| of the unshifted A (atomicMax on the bit pattern, NaN propagating).  Work items
// are 8192-element chunks of tiles; upper_only skips the tiles below the diagonal (Cholesky
// reads only the upper triangle, which a caller may have copied in first).
constexpr int kConvChunk = 8192;
// float(d) rounded to nearest even by integer operations on the bit pattern only (the FP64 ->
// FP32 conversion instruction runs on this part's FP64 pipe, 2 per clock per SM, which would
// bound a streaming conversion): normal results keep the top 23 of the 52 mantissa bits and
// round on the 29 dropped ones (a carry reaches the exponent, and past the largest finite value
// gives infinity); results below the normal range shift the 53-bit significand into the
// subnormal field with the same rounding; Inf stays Inf, NaN becomes the quiet NaN.
__device__ __forceinline__ float d2f_rne(double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const int E = (int)((b >> 52) & 0x7FF);
    const int e32 = E - 1023 + 127;
    const unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
    // normal range
    const unsigned hi23 = (unsigned)(mant >> 29);
    const unsigned rem = (unsigned)mant & 0x1FFFFFFFu;
    unsigned fn = ((unsigned)e32 << 23) | hi23;
    fn += (rem > 0x10000000u) | ((rem == 0x10000000u) & (hi23 & 1u));
    // below it: significand >> (30 - e32) (1 + 52 bits; nothing survives a shift of 54 or more)
    const int sh = 30 - e32;
    const unsigned long long sig = mant | 0x10000000000000ull;
    unsigned fs = 0;
    if (E != 0 && e32 < 1 && sh < 54) {  // sh >= 30 here
        const unsigned long long q = sig >> sh, r = sig & ((1ull << sh) - 1), half = 1ull << (sh - 1);
        fs = (unsigned)q + ((r > half) | ((r == half) & (unsigned)(q & 1)));
    }
    unsigned f = e32 >= 1 ? fn : fs;
    if (e32 > 254) f = 0x7F800000u;                            // overflow
    if (E == 0x7FF) f = mant ? 0x7FC00000u : 0x7F800000u;      // NaN, Inf
    return __uint_as_float(f | sign);
}

__global__ void f64_to_f32_kernel(const double *__restrict__ a, float *__restrict__ w, int n, int nb,
                                  double shift_diag, int upper_only, int r0, int r1, double *amax) {
    const int mt = n / nb;
    const int te = nb * nb;
    const int chunks = (te + kConvChunk - 1) / kConvChunk;
    const long long items = (long long)mt * mt * chunks;
    // max |a| on the bit patterns (integer compares; for non-negative doubles the unsigned
    // order is the value order, and a NaN's pattern exceeds every finite one)
    unsigned long long mx = 0;
    for (long long it = blockIdx.x; it < items; it += gridDim.x) {
        const int t = (int)(it / chunks), ch = (int)(it - (long long)t * chunks);
        const int tr = t % mt, tc = t / mt;
        if ((upper_only && tr > tc) || tr < r0 || tr >= r1) continue;  // uniform per CTA
        const size_t base = (size_t)t * te;
        const int end = min(te, (ch + 1) * kConvChunk);
        const bool diag = shift_diag != 0.0 && tr == tc;
        // a symmetric matrix held as its upper triangle: the max skips the strictly lower
        // entries of the diagonal tiles (they need not hold A's values)
        const bool lower_skip = upper_only && tr == tc;
#pragma unroll 4
        for (int i = ch * kConvChunk + 2 * threadIdx.x; i < end; i += 2 * blockDim.x) {
            double2 v = *reinterpret_cast<const double2 *>(a + base + i);  // te even: 16-byte aligned
            unsigned long long b0 = (unsigned long long)__double_as_longlong(v.x) & 0x7FFFFFFFFFFFFFFFull;
            unsigned long long b1 = (unsigned long long)__double_as_longlong(v.y) & 0x7FFFFFFFFFFFFFFFull;
            if (lower_skip) {  // entries i, i + 1 share column i / nb (nb even)
                const int r = i % nb, c = i / nb;
                b0 = r > c ? 0ull : b0;
                b1 = r + 1 > c ? 0ull : b1;
            }
            mx = b0 > mx ? b0 : mx;
            mx = b1 > mx ? b1 : mx;
            if (diag) {
                if (i % (nb + 1) == 0) v.x += shift_diag;
                if ((i + 1) % (nb + 1) == 0) v.y += shift_diag;
            }
            *reinterpret_cast<float2 *>(w + base + i) = make_float2(d2f_rne(v.x), d2f_rne(v.y));
        }
    }
    if (amax) {
        for (int o = 16; o; o >>= 1) {
            const unsigned long long y = __shfl_xor_sync(0xffffffffu, mx, o);
            mx = y > mx ? y : mx;
        }
        if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<unsigned long long *>(amax), mx);
    }
}

// ---- the lower triangle of a symmetric matrix from its upper triangle ---------------------
// A(i, j) <- A(j, i) for every i > j of an n x n tile-layout matrix (nb a multiple of 32):
// host-buffer Cholesky solves copy only the upper triangle (the triangle the factorization
// reads) and rebuild the rest on the device for the residuals.  One CTA per 32 x 32 block
// (bi, bj), bi >= bj, of the lower triangle in a grid-stride loop: the mirror block (bj, bi)
// is read along its columns into shared memory and written along the destination's columns.
// On a diagonal block only the strictly lower entries are written, from the strictly upper
// ones read before the barrier.
__device__ __forceinline__ size_t sym_off(int n, int nb, int r, int c) {
    const int mt = n / nb;
    return (size_t)nb * nb * ((size_t)(r / nb) + (size_t)mt * (c / nb)) + (size_t)(r % nb) + (size_t)(c % nb) * nb;
}

__global__ void __launch_bounds__(256) mirror_upper_kernel(double *__restrict__ a, int n, int nb) {
    __shared__ double s[32][33];  // s[column][row] of the source block
    const int nbk = n / 32;
    const long long items = (long long)nbk * (nbk + 1) / 2;  // block it = bi (bi + 1) / 2 + bj
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (long long it = blockIdx.x; it < items; it += gridDim.x) {
        int bi = (int)((sqrtf(8.0f * (float)it + 1.0f) - 1.0f) * 0.5f);  // an estimate: corrected below
        while ((long long)bi * (bi + 1) / 2 > it) bi--;
        while ((long long)(bi + 1) * (bi + 2) / 2 <= it) bi++;
        const int bj = (int)(it - (long long)bi * (bi + 1) / 2);
        const int r0 = 32 * bj, c0 = 32 * bi;  // source block: rows r0.., columns c0.. (upper)
#pragma unroll
        for (int q = ty; q < 32; q += 8) s[q][tx] = a[sym_off(n, nb, r0 + tx, c0 + q)];
        __syncthreads();
        // destination (c0 + tx, r0 + q) = source (r0 + q, c0 + tx) = s[tx][q]
#pragma unroll
        for (int q = ty; q < 32; q += 8)
            if (bi != bj || tx > q) a[sym_off(n, nb, c0 + tx, r0 + q)] = s[tx][q];
        __syncthreads();
    }
}

// ---- compensated FP32 residual -------------------------------------------------------------
// Operands as pairs of FP32 numbers: v * 2^-sc = hi + lo with hi the top 24 bits of the
// significand and lo the next 29 rounded to 24 (48 bits in all), taken from the bit pattern
// with integer operations (no FP64 arithmetic).  Values below 2^-100 relative to the scale
// flush gradually (their contribution is below 2^-124 of the largest entry).  Inf/NaN -> NaN.
__device__ __forceinline__ float pow2f(int k) {  // 2^k for k >= -126 (else 0)
    return k < -126 ? 0.f : __int_as_float((k + 127) << 23);
}
__device__ __forceinline__ float2 split_df(double v, int sc) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
    const int E = (int)((bits >> 52) & 0x7FF);
    if (E == 0x7FF) return make_float2(__int_as_float(0x7fc00000), 0.f);
    const unsigned long long M = (bits & ((1ull << 52) - 1)) | (E ? (1ull << 52) : 0ull);
    const int e2 = (E ? E : 1) - 1075 - sc;  // v * 2^-sc = M * 2^e2
    float hi = __fmul_rn(__uint2float_rn((unsigned)(M >> 29)), pow2f(e2 + 29));
    float lo = __fmul_rn(__uint2float_rn((unsigned)(M & ((1ull << 29) - 1))), pow2f(e2));
    if (bits >> 63) {
        hi = -hi;
        lo = -lo;
    }
    return make_float2(hi, lo);
}

// Xs (n x 16 float2, rhs-minor: Xs[r * 16 + c]) = split(X(r, c) * 2^-tau_c), tau_c the
// exponent of the column's max |x| (colmax from mps_colmax), zero beyond nrhs.
__global__ void split_x_kernel(const double *X, long long n, int nrhs, const double *colmax, float2 *Xs, int *tau) {
    const long long total = n * 16;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e & 15);
        const long long r = e >> 4;
        int t = 0;
        if (c < nrhs) frexp(colmax[c], &t);
        Xs[e] = (c < nrhs) ? split_df(X[(size_t)r + (size_t)c * n], t) : make_float2(0.f, 0.f);
        if (r == 0) tau[c] = t;
    }
}

// R = B - A X with A and X as FP32 pairs: per product the exact FP32 product of the high parts
// (fma), the cross terms into its error, and a TwoSum accumulation (Knuth) of the pair; every
// 64 products the pair is added to an FP64 accumulator.  One CTA of 128 threads per 32-row
// block (n/32 CTAs: many resident per SM, a short last wave); thread = row x 4 right-hand
// sides (t % 32, t / 32).  amax as in residual_kernel (row sums of |a|).
__device__ __forceinline__ void df_acc(float ah, float al, float xh, float xl, float &s, float &c) {
    // explicit _rn intrinsics: no FMA contraction may touch the error-free steps
    const float pr = __fmul_rn(ah, xh);
    const float t = fmaf(ah, xl, fmaf(al, xh, fmaf(ah, xh, -pr)));
    const float sn = __fadd_rn(s, pr), bp = __fsub_rn(sn, s);
    c = __fadd_rn(c, __fadd_rn(__fadd_rn(__fsub_rn(s, __fsub_rn(sn, bp)), __fsub_rn(pr, bp)), t));
    s = sn;
}
__global__ void __launch_bounds__(128) residual_df_kernel(const double *A, int n, int nb, const float2 *Xs,
                                                          const int *tau, int sigma, const double *B, double *R,
                                                          int nrhs, double *amax) {
    __shared__ float2 As[64][33];
    __shared__ float4 Xp[64][8];  // (hi, lo) of right-hand sides 2j, 2j+1
    __shared__ float part[4][33];
    const int i0 = blockIdx.x * 32;
    const int row = threadIdx.x & 31, grp = threadIdx.x >> 5;  // right-hand sides 4 grp .. 4 grp + 3
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    float asum = 0.f;
    const int mt = n / nb;
    const double *tilerow = A + (size_t)nb * nb * (size_t)(i0 / nb) + (size_t)(i0 % nb);
    for (int p0 = 0; p0 < n; p0 += 64) {
        const double *blk = tilerow + (size_t)nb * nb * (size_t)mt * (p0 / nb) + (size_t)(p0 % nb) * nb;
        for (int e = threadIdx.x; e < 2048; e += 128) As[e >> 5][e & 31] = split_df(blk[(e & 31) + (size_t)(e >> 5) * nb], sigma);
        for (int e = threadIdx.x; e < 64 * 8; e += 128) {
            const float2 a = Xs[(size_t)(p0 + (e >> 3)) * 16 + 2 * (e & 7)];
            const float2 b = Xs[(size_t)(p0 + (e >> 3)) * 16 + 2 * (e & 7) + 1];
            Xp[e >> 3][e & 7] = make_float4(a.x, a.y, b.x, b.y);
        }
        __syncthreads();
        if (amax) {
#pragma unroll
            for (int p = grp; p < 64; p += 4) {
                const float2 a = As[p][row];
                asum += fabsf(a.x + a.y);
            }
        }
        float s[4] = {0.f, 0.f, 0.f, 0.f}, c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 4
        for (int p = 0; p < 64; p++) {
            const float2 a = As[p][row];
            const float4 x01 = Xp[p][2 * grp], x23 = Xp[p][2 * grp + 1];
            df_acc(a.x, a.y, x01.x, x01.y, s[0], c[0]);
            df_acc(a.x, a.y, x01.z, x01.w, s[1], c[1]);
            df_acc(a.x, a.y, x23.x, x23.y, s[2], c[2]);
            df_acc(a.x, a.y, x23.z, x23.w, s[3], c[3]);
        }
#pragma unroll
        for (int j = 0; j < 4; j++) acc[j] += (double)s[j] + (double)c[j];
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int cc = 4 * grp + j;
        if (cc < nrhs) {
            const size_t o = (size_t)(i0 + row) + (size_t)cc * n;
            const double ax = ldexp(acc[j], sigma + tau[cc]);
            R[o] = B ? B[o] - ax : ax;
        }
    }
    if (amax) {
        part[grp][row] = asum;
        __syncthreads();
        if (threadIdx.x < 32) {
            double t = (double)part[0][row] + (double)part[1][row] + (double)part[2][row] + (double)part[3][row];
            t = ldexp(t, sigma);
            for (int o = 16; o; o >>= 1) t = fmax(t, __shfl_xor_sync(0xffffffffu, t, o));
            if (threadIdx.x == 0)
                atomicMax(reinterpret_cast<unsigned long long *>(amax), (unsigned long long)__double_as_longlong(t));
        }
    }
}

// ---- update-form residual R <- R - A D for a small correction D ---------------------------
// After x += d with ||d|| << ||x||, the residual of the new x is r - A d, and A d needs only
// a modest relative accuracy: its error enters the backward error scaled by ||d|| / ||x||.
// Plain FP32 products then suffice and the kernel is bound by reading A once from HBM
// (8 bytes per element) instead of by the compensated residual's ~12 FP32 operations per
// product.  Error bound: A's entries and D rounded to FP32 (2^-24 each), every lane sums 64
// products with FMAs (64 roundings of at most 2^-24 of the running sum) before folding them
// into a float-float accumulator (TwoSum, error ~2^-44), so per entry
// |computed - exact| <= 67 * 2^-24 * sum_p |a_ip| |d_p| < 2^-17 * sum_p |a_ip| |d_p|
// (the caller weighs 2^-17 ||A|| ||d|| against its tolerance before choosing this form).

// float(v * 2^-sc) rounded to 24 significant bits (half-way cases away from zero), integer
// operations only (no FP64 pipe): adding half an FP32 ulp to the pattern lets a carry out of
// the significand step the exponent.  Results below 2^-126 after scaling flush to zero (|v|
// < 2^sc, so their weight is below 2^-126 of the largest entry); Inf/NaN give NaN.
__device__ __forceinline__ float f64_round_f32(unsigned long long bits, int sc) {
    const bool special = ((bits >> 52) & 0x7FF) == 0x7FF;
    bits += 1ull << 28;
    const int E = (int)((bits >> 52) & 0x7FF);
    const int e32 = E - 1023 - sc + 127;
    unsigned f = ((unsigned)(bits >> 32) & 0x80000000u) | ((unsigned)(bits >> 29) & 0x7FFFFFu) | ((unsigned)e32 << 23);
    f = e32 <= 0 ? (f & 0x80000000u) : f;
    f = special ? 0x7fc00000u : f;
    return __uint_as_float(f);
}

// Ds (n x 16 floats, rhs-minor: Ds[r * 16 + c]) = float(D(r, c) * 2^-tau_c), tau_c the exponent
// of the column's max |d| (colmax); zero beyond nrhs.
__global__ void d_to_f32_kernel(const double *D, long long n, int nrhs, const double *colmax, float *Ds, int *tau) {
    const long long total = n * 16;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e & 15);
        const long long r = e >> 4;
        int t = 0;
        if (c < nrhs) frexp(colmax[c], &t);
        float v = 0.f;
        if (c < nrhs) {
            const float2 h = split_df(D[(size_t)r + (size_t)c * n], t);
            v = __fadd_rn(h.x, h.y);
        }
        Ds[e] = v;
        if (r == 0) tau[c] = t;
    }
}

__device__ __forceinline__ void two_sum_acc(float v, float &H, float &L) {
    const float sn = __fadd_rn(H, v), bp = __fsub_rn(sn, H);
    L = __fadd_rn(L, __fadd_rn(__fsub_rn(H, __fsub_rn(sn, bp)), __fsub_rn(v, bp)));
    H = sn;
}

// One CTA of 4 warps per 32-row block: lane = row, warp w takes columns p0 + w + 4 j
// (j < 16) of every 64-column chunk, all 16 right-hand sides per lane; the chunk of D is staged
// in shared memory (read as broadcasts).  Partial sums of warps 1..3 are combined by warp 0 in
// a fixed order (deterministic).
__global__ void __launch_bounds__(128) residual_update_kernel(const double *__restrict__ A, int n, int nb,
                                                              const float *__restrict__ Ds, const int *__restrict__ tau,
                                                              int sigma, double *__restrict__ R, int nrhs) {
    __shared__ float4 Dsh[64][4];
    __shared__ double part[3][16][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int i0 = blockIdx.x * 32;
    const int mt = n / nb;
    const unsigned long long *tilerow =
        reinterpret_cast<const unsigned long long *>(A) + (size_t)nb * nb * (size_t)(i0 / nb) + (size_t)(i0 % nb) + lane;
    float s[16], H[16], L[16];
#pragma unroll
    for (int c = 0; c < 16; c++) s[c] = H[c] = L[c] = 0.f;
    int chunks = 0;
    for (int p0 = 0; p0 < n; p0 += 64) {
        const unsigned long long *blk = tilerow + (size_t)nb * nb * (size_t)mt * (p0 / nb) + (size_t)(p0 % nb) * nb;
        unsigned long long av[16];
#pragma unroll
        for (int j = 0; j < 16; j++) av[j] = __ldcs(blk + (size_t)(w + 4 * j) * nb);  // read once: streaming
        __syncthreads();  // the previous chunk's D is consumed
        for (int e = threadIdx.x; e < 256; e += 128)
            Dsh[e >> 2][e & 3] = __ldg(reinterpret_cast<const float4 *>(Ds + (size_t)p0 * 16) + e);
        __syncthreads();
#pragma unroll
        for (int j = 0; j < 16; j++) {
            const float a = f64_round_f32(av[j], sigma);
            const int p = w + 4 * j;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const float4 d = Dsh[p][q];
                s[4 * q + 0] = fmaf(a, d.x, s[4 * q + 0]);
                s[4 * q + 1] = fmaf(a, d.y, s[4 * q + 1]);
                s[4 * q + 2] = fmaf(a, d.z, s[4 * q + 2]);
                s[4 * q + 3] = fmaf(a, d.w, s[4 * q + 3]);
            }
        }
        if (++chunks == 4) {  // 64 products per lane and right-hand side
#pragma unroll
            for (int c = 0; c < 16; c++) {
                two_sum_acc(s[c], H[c], L[c]);
                s[c] = 0.f;
            }
            chunks = 0;
        }
    }
#pragma unroll
    for (int c = 0; c < 16; c++) two_sum_acc(s[c], H[c], L[c]);
    if (w > 0) {
#pragma unroll
        for (int c = 0; c < 16; c++) part[w - 1][c][lane] = (double)H[c] + (double)L[c];
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int c = 0; c < 16; c++) {
            if (c < nrhs) {
                const double v = (double)H[c] + (double)L[c] + part[0][c][lane] + part[1][c][lane] + part[2][c][lane];
                const size_t o = (size_t)(i0 + lane) + (size_t)c * n;
                R[o] -= ldexp(v, sigma + tau[c]);
            }
        }
    }
}

__global__ void tile_f32_to_f64_kernel(const float *w, double *d, int count) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < count; e += gridDim.x * blockDim.x) d[e] = (double)w[e];
}

// copy back the factored diagonal tile; mask 0: full, 1: upper triangle (row <= col)
__global__ void tile_f64_to_f32_kernel(const double *d, float *w, int nb, int mask) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nb * nb; e += gridDim.x * blockDim.x) {
        const int r = e % nb, c = e / nb;
        if (mask == 1 && r > c) continue;
        w[e] = (float)d[e];
    }
}

// ---- panel triangular solves (one CTA per 64-wide strip of one tile) -----------------------
struct Smem {
    float (*Ds)[DP];
    float (*Bs)[DP];
    float *g;
};
__device__ __forceinline__ Smem smem_parts(float *s) {
    Smem m;
    m.Ds = reinterpret_cast<float (*)[DP]>(s);
    m.Bs = reinterpret_cast<float (*)[DP]>(s + 64 * DP);
    m.g = s + 2 * 64 * DP;
    return m;
}

// ---- inverses of the 64 x 64 diagonal blocks of a factored diagonal tile -------------------
// binv[(which * (nb/64) + b) * 4096 ..]: the column-major 64 x 64 inverse of diagonal block b of
// tile (k, k): which 0 = of the upper factor U_bb (Cholesky and LU), 1 = of the unit lower
// factor L_bb (LU).  One CTA of 64 threads per block and factor; thread c computes column c,
// its 64 unknowns in registers, eliminating right-looking (the FMAs of one step are
// independent; the coefficients are shared-memory broadcasts).  The panel solves then apply
// each diagonal block as a 64 x 64 product instead of a 64-step substitution.
__global__ void __launch_bounds__(256) block_inverse_kernel(const float *W, int n, int nb, int k, float *binv) {
    __shared__ __align__(16) float Ts[64][64];  // Ts[c][r] = block(r, c)
    const int b = blockIdx.x, which = blockIdx.y;
    const float *T = W + tile_off(n, nb, k, k) + (size_t)b * 64 * ((size_t)nb + 1);
    // 256 threads load (16 independent loads each, all in flight), 64 of them solve
#pragma unroll
    for (int j = 0; j < 16; j++) {
        const int e = threadIdx.x + 256 * j;
        Ts[e >> 6][e & 63] = T[(e & 63) + (size_t)(e >> 6) * nb];
    }
    __syncthreads();
    if (threadIdx.x >= 64) return;
    const int c = threadIdx.x;
    float x[64];
#pragma unroll
    for (int i = 0; i < 64; i++) x[i] = (i == c) ? 1.f : 0.f;
    if (which == 0) {
        // U x = e_c, backward: x_p /= u_pp, then x_i -= u_ip x_p for i < p
#pragma unroll
        for (int p = 63; p >= 0; p--) {
            x[p] = x[p] / Ts[p][p];
#pragma unroll
            for (int i0 = 0; i0 < p; i0 += 4) {
                const float4 u = *reinterpret_cast<const float4 *>(&Ts[p][i0]);
                const float uv[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
                for (int j = 0; j < 4; j++)
                    if (i0 + j < p) x[i0 + j] = fmaf(-uv[j], x[p], x[i0 + j]);
            }
        }
    } else {
        // L x = e_c (unit lower), forward: x_i -= l_ip x_p for i > p
#pragma unroll
        for (int p = 0; p < 63; p++) {
#pragma unroll
            for (int i0 = (p + 1) & ~3; i0 < 64; i0 += 4) {
                const float4 l = *reinterpret_cast<const float4 *>(&Ts[p][i0]);
                const float lv[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
                for (int j = 0; j < 4; j++)
                    if (i0 + j > p) x[i0 + j] = fmaf(-lv[j], x[p], x[i0 + j]);
            }
        }
    }
    float *out = binv + ((size_t)which * (nb / 64) + b) * 4096 + (size_t)c * 64;
#pragma unroll
    for (int i = 0; i < 64; i += 4) *reinterpret_cast<float4 *>(out + i) = make_float4(x[i], x[i + 1], x[i + 2], x[i + 3]);
}

// The 64 x 64 block B (at B, ld) in place: OP 0: X^T B; 1: X B; 2: B X, with X a column-major
// 64 x 64 inverse block.  Staged through shared memory (m.Ds[c][r] = X(r, c), m.Bs[c][r] =
// B(r, c)); thread: rows 4 tr .. 4 tr + 3, columns 4 tc .. 4 tc + 3.  Ends synced.
template <int OP>
__device__ __forceinline__ void apply_inv64(const Smem &m, const float *X, float *B, int ldb,
                                            __nv_bfloat16 *ph = nullptr, __nv_bfloat16 *pl = nullptr) {
    static_assert(4096 % NT == 0, "whole staging rounds");
#pragma unroll
    for (int j = 0; j < 4096 / NT; j++) {
        const int e = threadIdx.x + NT * j;
        m.Ds[e >> 6][e & 63] = ldg(X + e);
        m.Bs[e >> 6][e & 63] = B[(e & 63) + (size_t)(e >> 6) * ldb];
    }
    __syncthreads();
    const int tr = threadIdx.x & 15, tc = threadIdx.x >> 4;
    float acc[4][4] = {};
#pragma unroll 8
    for (int p = 0; p < 64; p++) {
        float a[4], bv[4];
#pragma unroll
        for (int x = 0; x < 4; x++) {
            const int r = 4 * tr + x;
            a[x] = OP == 0 ? m.Ds[r][p] : OP == 1 ? m.Ds[p][r] : m.Bs[p][r];
        }
#pragma unroll
        for (int y = 0; y < 4; y++) {
            const int c = 4 * tc + y;
            bv[y] = OP == 2 ? m.Ds[c][p] : m.Bs[c][p];
        }
#pragma unroll
        for (int x = 0; x < 4; x++)
#pragma unroll
            for (int y = 0; y < 4; y++) acc[x][y] = fmaf(a[x], bv[y], acc[x][y]);
    }
#pragma unroll
    for (int y = 0; y < 4; y++) {
        const size_t o = (size_t)(4 * tr) + (size_t)(4 * tc + y) * ldb;
        *reinterpret_cast<float4 *>(B + o) = make_float4(acc[0][y], acc[1][y], acc[2][y], acc[3][y]);
        if (ph) {  // the packed BF16 operand (and the BF16x3 remainder) of the same elements
#pragma unroll
            for (int x = 0; x < 4; x++) {
                const __nv_bfloat16 h = __float2bfloat16_rn(acc[x][y]);
                ph[o + x] = h;
                if (pl) pl[o + x] = __float2bfloat16_rn(acc[x][y] - __bfloat162float(h));
            }
        }
    }
    __syncthreads();
}

// X = U^-T B, B = nb x 64 strip (ld), U upper nb x nb (ld_u); uinv: inverses of U's 64 x 64
// diagonal blocks
// (ph, pl: optional packed BF16 copy of the strip, same layout, written with the results)
// tc: the block updates on the warp tensor cores (BF16x3 operands, FP32 accumulation; the panels
// of a factorization whose trailing updates are BF16x3), else FP32 FMAs.
__device__ __forceinline__ void strip_lut(const Smem &m, const float *U, int ldu, float *B, int ldb, int nb,
                                          const float *uinv, __nv_bfloat16 *ph = nullptr,
                                          __nv_bfloat16 *pl = nullptr, bool tc = false) {
    for (int rb = 0; rb < nb; rb += 64) {
        if (rb > 0 && tc)
            cta_gemm<true, false, false, true>(64, 64, rb, -1.f, U + (size_t)rb * ldu, ldu, B, ldb, B + rb, ldb, m.g);
        else if (rb > 0) cta_gemm<true, false>(64, 64, rb, -1.f, U + (size_t)rb * ldu, ldu, B, ldb, B + rb, ldb, m.g);
        apply_inv64<0>(m, uinv + (size_t)(rb / 64) * 4096, B + rb, ldb, ph ? ph + rb : nullptr, pl ? pl + rb : nullptr);
    }
}
// X = L^-1 B (unit lower) with L's diagonal-block inverses linv
__device__ __forceinline__ void strip_llu_inv(const Smem &m, const float *L, int ldl, float *B, int ldb, int nb,
                                              const float *linv, __nv_bfloat16 *ph = nullptr,
                                              __nv_bfloat16 *pl = nullptr, bool tc = false) {
    for (int rb = 0; rb < nb; rb += 64) {
        if (rb > 0 && tc) cta_gemm<false, false, false, true>(64, 64, rb, -1.f, L + rb, ldl, B, ldb, B + rb, ldb, m.g);
        else if (rb > 0) cta_gemm<false, false>(64, 64, rb, -1.f, L + rb, ldl, B, ldb, B + rb, ldb, m.g);
        apply_inv64<1>(m, linv + (size_t)(rb / 64) * 4096, B + rb, ldb, ph ? ph + rb : nullptr, pl ? pl + rb : nullptr);
    }
}
// X = U^-1 B (backward), B = nb x 64 strip
__device__ __forceinline__ void strip_un(const Smem &m, const float *U, int ldu, float *B, int ldb, int nb) {
    for (int rb = nb - 64; rb >= 0; rb -= 64) {
        if (rb + 64 < nb)
            cta_gemm<false, false>(64, 64, nb - rb - 64, -1.f, U + rb + (size_t)(rb + 64) * ldu, ldu, B + rb + 64, ldb,
                                   B + rb, ldb, m.g);
        load_diag64(m.Ds, U + rb + (size_t)rb * ldu, ldu);
        solve64<3>(m.Ds, B + rb, ldb);
    }
}
// X = L^-1 B (unit lower), B = nb x 64 strip
__device__ __forceinline__ void strip_llu(const Smem &m, const float *L, int ldl, float *B, int ldb, int nb) {
    for (int rb = 0; rb < nb; rb += 64) {
        if (rb > 0) cta_gemm<false, false>(64, 64, rb, -1.f, L + rb, ldl, B, ldb, B + rb, ldb, m.g);
        load_diag64(m.Ds, L + rb + (size_t)rb * ldl, ldl);
        solve64<2>(m.Ds, B + rb, ldb);
    }
}
// X = B U^-1, B = 64 x nb row strip, with U's diagonal-block inverses uinv
__device__ __forceinline__ void strip_run(const Smem &m, const float *U, int ldu, float *B, int ldb, int nb,
                                          const float *uinv, bool tc = false) {
    for (int cb = 0; cb < nb; cb += 64) {
        if (cb > 0 && tc)
            cta_gemm<false, false, false, true>(64, 64, cb, -1.f, B, ldb, U + (size_t)cb * ldu, ldu, B + (size_t)cb * ldb,
                                                ldb, m.g);
        else if (cb > 0)
            cta_gemm<false, false>(64, 64, cb, -1.f, B, ldb, U + (size_t)cb * ldu, ldu, B + (size_t)cb * ldb, ldb, m.g);
        apply_inv64<2>(m, uinv + (size_t)(cb / 64) * 4096, B + (size_t)cb * ldb, ldb);
    }
}

// kind 0: Cholesky row panel U(k,m) <- U_kk^-T U(k,m);  1: LU row panel U(k,n) <- L_kk^-1 .;
// 2: LU column panel L(m,k) <- L(m,k) U_kk^-1.  grid (nb/64, trailing tiles).  binv: the
// diagonal-block inverses of tile k (block_inverse_kernel).
// ph, pl (row panels, optional): the packed BF16 (+ BF16x3 remainder) operand of the row panel,
// trailing tile t - k - 1 at (t - k - 1) nb^2, written together with the solved values.
__global__ void __launch_bounds__(NT, 2) panel_trsm_kernel(float *W, int n, int nb, int k, int kind,
                                                          const float *binv, __nv_bfloat16 *ph, __nv_bfloat16 *pl,
                                                          int t0, int tc) {
    extern __shared__ __align__(16) float smem[];
    const Smem m = smem_parts(smem);
    const int tt = t0 + blockIdx.y;  // trailing tile index
    const int t = k + 1 + tt, s = blockIdx.x;
    const float *T = W + tile_off(n, nb, k, k);
    const size_t po = (size_t)tt * nb * nb + (size_t)s * 64 * nb;
    __nv_bfloat16 *sh = ph ? ph + po : nullptr, *sl = pl ? pl + po : nullptr;
    if (kind == 0) strip_lut(m, T, nb, W + tile_off(n, nb, k, t) + (size_t)s * 64 * nb, nb, nb, binv, sh, sl, tc != 0);
    else if (kind == 1)
        strip_llu_inv(m, T, nb, W + tile_off(n, nb, k, t) + (size_t)s * 64 * nb, nb, nb, binv + (size_t)(nb / 64) * 4096,
                      sh, sl, tc != 0);
    else strip_run(m, T, nb, W + tile_off(n, nb, t, k) + s * 64, nb, nb, binv, tc != 0);
}

// ---- two-level factorization of a diagonal tile (NB >= 512) ---------------------------------
// The tile is factored as 2 x 2 blocks of h = NB/2: one-CTA factorization of A11, then these
// two multi-CTA steps, then one-CTA factorization of A22 (mp_diag.cu).
// Cholesky (alg 0): A12 (h x h at T + h ld) <- U11^-T A12, one CTA per 64-column strip.
// LU (alg 1): blockIdx.y = 0: U12 <- L11^-1 A12 (64-column strips), 1: L21 <- A21 U11^-1
// (64-row strips).  binv: inverses of the 64 x 64 diagonal blocks of U11 (and, for LU, of
// L11 at binv + (ld / 64) * 4096).
__global__ void __launch_bounds__(NT, 2) half_panel_kernel(float *T, int h, int ld, const float *binv, int alg) {
    extern __shared__ __align__(16) float smem[];
    const Smem m = smem_parts(smem);
    if (alg == 0) strip_lut(m, T, ld, T + (size_t)h * ld + (size_t)blockIdx.x * 64 * ld, ld, h, binv);
    else if (blockIdx.y == 0)
        strip_llu_inv(m, T, ld, T + (size_t)h * ld + (size_t)blockIdx.x * 64 * ld, ld, h, binv + (size_t)(ld / 64) * 4096);
    else strip_run(m, T, ld, T + h + (size_t)blockIdx.x * 64, ld, h, binv);
}
// Cholesky: A22 -= A12^T A12 on the 64 x 64 blocks (bi, bj), bi <= bj, of the trailing h x h
// block (one CTA each; inside diagonal blocks the strictly lower entries stay unchanged).
// LU: A22 -= L21 U12 on every 64 x 64 block.
__global__ void __launch_bounds__(NT, 2) half_update_kernel(float *T, int h, int ld, int alg) {
    extern __shared__ __align__(16) float smem[];
    const Smem m = smem_parts(smem);
    if (alg == 1) {
        const int nbl = h / 64, bi = blockIdx.x % nbl, bj = blockIdx.x / nbl;
        cta_gemm<false, false>(64, 64, h, -1.f, T + h + (size_t)bi * 64, ld, T + (size_t)(h + bj * 64) * ld, ld,
                               T + (size_t)(h + bi * 64) + (size_t)(h + bj * 64) * ld, ld, m.g);
        return;
    }
    int q = blockIdx.x, bj = 0;
    while (q > bj) {
        q -= bj + 1;
        bj++;
    }
    const int bi = q;
    const float *A12 = T + (size_t)h * ld;
    float *C = T + (size_t)(h + bi * 64) + (size_t)(h + bj * 64) * ld;
    if (bi == bj)
        cta_gemm<true, false, true>(64, 64, h, -1.f, A12 + (size_t)bi * 64 * ld, ld, A12 + (size_t)bj * 64 * ld, ld, C,
                                    ld, m.g);
    else
        cta_gemm<true, false>(64, 64, h, -1.f, A12 + (size_t)bi * 64 * ld, ld, A12 + (size_t)bj * 64 * ld, ld, C, ld,
                              m.g);
}

// ---- diagonal-tile inverses for the refinement solves --------------------------------------
// Dinv tile k (nb x nb, column-major) = T_kk^-1 with T the upper factor (kind 1) or the unit
// lower factor (kind 2) of the diagonal tile; one CTA per 64-column strip of the identity.
__global__ void __launch_bounds__(NT, 1) invert_diag_kernel(const float *W, int n, int nb, float *Dinv, int kind) {
    extern __shared__ __align__(16) float smem[];
    const Smem m = smem_parts(smem);
    const int k = blockIdx.y, s = blockIdx.x;
    float *X = Dinv + (size_t)k * nb * nb + (size_t)s * 64 * nb;   // strip of columns s*64..
    for (int e = threadIdx.x; e < nb * 64; e += NT) {
        const int r = e % nb, c = e / nb;
        X[r + (size_t)c * nb] = (r == s * 64 + c) ? 1.f : 0.f;
    }
    __syncthreads();
    const float *T = W + tile_off(n, nb, k, k);
    if (kind == 1) strip_un(m, T, nb, X, nb, nb);
    else strip_llu(m, T, nb, X, nb, nb);
}


// ---- FP64 residual R = B - A X (A: FP64 tile layout; X, B, R: n x nrhs, ld n; nrhs <= 16) ---
// One CTA per 32-row block (n/32 CTAs, several resident per SM, so the last wave is short);
// thread (row = t % 32, group g = t / 32) accumulates right-hand sides 2g and 2g + 1 over all
// columns, A staged 64 columns at a time.  The FP64 pipe is the bound (16 right-hand sides:
// 4 flop per byte of A).  With amax != nullptr the same pass also returns ||A||_inf (the row
// sums of |a_ij| in FP32 partials, combined in FP64; atomicMax on the bit pattern, amax
// zeroed by the caller).
__global__ void __launch_bounds__(256) residual_kernel(const double *A, int n, int nb, const double *X,
                                                       const double *B, double *R, int nrhs, double *amax) {
    __shared__ double As[64][33];
    __shared__ double Xs[64][17];
    __shared__ float part[8][33];
    const int i0 = blockIdx.x * 32;
    const int row = threadIdx.x & 31, grp = threadIdx.x >> 5;
    double acc0 = 0.0, acc1 = 0.0;
    float asum = 0.f;
    const int mt = n / nb;
    const double *tilerow = A + (size_t)nb * nb * (size_t)(i0 / nb) + (size_t)(i0 % nb);
    for (int p0 = 0; p0 < n; p0 += 64) {
        const double *blk = tilerow + (size_t)nb * nb * (size_t)mt * (p0 / nb) + (size_t)(p0 % nb) * nb;
        for (int e = threadIdx.x; e < 2048; e += 256) As[e >> 5][e & 31] = blk[(e & 31) + (size_t)(e >> 5) * nb];
        for (int e = threadIdx.x; e < 64 * 16; e += 256) {
            const int r = e & 63, c = e >> 6;
            Xs[r][c] = (c < nrhs) ? X[(size_t)(p0 + r) + (size_t)c * n] : 0.0;
        }
        __syncthreads();
        if (amax) {
#pragma unroll
            for (int p = grp; p < 64; p += 8) asum += fabsf((float)As[p][row]);
        }
#pragma unroll 8
        for (int p = 0; p < 64; p++) {
            const double a = As[p][row];
            acc0 = fma(a, Xs[p][2 * grp], acc0);
            acc1 = fma(a, Xs[p][2 * grp + 1], acc1);
        }
        __syncthreads();
    }
    const double accs[2] = {acc0, acc1};
#pragma unroll
    for (int j = 0; j < 2; j++) {
        const int c = 2 * grp + j;
        if (c < nrhs) {
            const size_t o = (size_t)(i0 + row) + (size_t)c * n;
            R[o] = B ? B[o] - accs[j] : accs[j];
        }
    }
    if (amax) {
        part[grp][row] = asum;
        __syncthreads();
        if (threadIdx.x < 32) {
            double t = 0.0;
#pragma unroll
            for (int g = 0; g < 8; g++) t += (double)part[g][row];
            for (int o = 16; o; o >>= 1) t = fmax(t, __shfl_xor_sync(0xffffffffu, t, o));
            if (threadIdx.x == 0)
                atomicMax(reinterpret_cast<unsigned long long *>(amax), (unsigned long long)__double_as_longlong(t));
        }
    }
}

// ||A||_inf partial: max over rows of sum |a_ij|, one CTA per 64-row block (FP64 tiles)
__global__ void rowsum_kernel(const double *A, int n, int nb, double *out_max) {
    __shared__ double part[4][64];
    const int i0 = blockIdx.x * 64;
    const int row = threadIdx.x & 63, grp = threadIdx.x >> 6;
    const int mt = n / nb;
    double s = 0.0;
    for (int j = grp; j < n; j += 4) {
        const int i = i0 + row;
        s += fabs(A[(size_t)nb * nb * ((size_t)(i / nb) + (size_t)mt * (j / nb)) + (size_t)(i % nb) + (size_t)(j % nb) * nb]);
    }
    part[grp][row] = s;
    __syncthreads();
    if (threadIdx.x < 64) {
        double t = part[0][row] + part[1][row] + part[2][row] + part[3][row];
        for (int o = 16; o; o >>= 1) t = fmax(t, __shfl_xor_sync(0xffffffffu, t, o));
        if ((threadIdx.x & 31) == 0) {
            unsigned long long *addr = reinterpret_cast<unsigned long long *>(out_max);
            atomicMax(addr, (unsigned long long)__double_as_longlong(t));  // t >= 0: bit order = value order
        }
    }
}

// per-column max |x| of dense n x cols (FP64), atomicMax on the bit patterns (values >= 0).
// NaN propagates (a NaN anywhere makes the column's maximum NaN: its bit pattern as an
// unsigned integer exceeds every finite double), so a non-finite solution can never look
// like a zero residual.
__device__ __forceinline__ double nanmax(double a, double b) { return (a > b || a != a) ? a : b; }
__global__ void colmax_kernel(const double *X, long long n, int cols, double *out) {
    const int c = blockIdx.y;
    double mx = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        mx = nanmax(mx, fabs(X[(size_t)i + (size_t)c * n]));
    for (int o = 16; o; o >>= 1) mx = nanmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0)
        atomicMax(reinterpret_cast<unsigned long long *>(out + c), (unsigned long long)__double_as_longlong(mx));
}


// R32 (n x RW, zero padded) = float(R64 / scale_c)
__global__ void to_f32_rhs_kernel(const double *R, float *R32, long long n, int cols, const double *scale) {
    const long long total = n * RW;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e / n);
        R32[e] = (c < cols) ? (float)(R[e] / scale[c]) : 0.f;
    }
}
// ---- GMRES building blocks (n x nrhs column-major blocks, one Krylov space per column) ----
// H[l*nrhs + c] += <V_l[:,c], w[:,c]> for l < count (V_l at V + l*n*nrhs)
__global__ void multi_dot_kernel(const double *V, int count, const double *w, long long n, int nrhs, double *H) {
    const int l = blockIdx.y;
    const double *v = V + (size_t)l * n * nrhs;
    double acc[16];
#pragma unroll
    for (int c = 0; c < 16; c++) acc[c] = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        for (int c = 0; c < nrhs; c++) acc[c] = fma(v[(size_t)c * n + i], w[(size_t)c * n + i], acc[c]);
    for (int c = 0; c < nrhs; c++) {
        double x = acc[c];
        for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(H + (size_t)l * nrhs + c, x);
    }
}
// w[:,c] -= sum_l H[l*nrhs + c] V_l[:,c]   (or w = sum_l H V_l when assign)
__global__ void multi_axpy_kernel(const double *V, int count, const double *H, double *w, long long n, int nrhs,
                                  int assign) {
    const long long total = n * nrhs;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e / n);
        double s = 0.0;
        for (int l = 0; l < count; l++) s = fma(H[(size_t)l * nrhs + c], V[(size_t)l * n * nrhs + e], s);
        w[e] = assign ? s : w[e] - s;
    }
}
// out = w / f[c] (f > 0) or copy with scaling; X = scale_c * D32 (assign)
__global__ void scale_cols_kernel(const double *w, double *out, long long n, int nrhs, const double *f) {
    const long long total = n * nrhs;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x)
        out[e] = w[e] / f[e / n];
}
__global__ void from_f32_rhs_kernel(double *X, const float *D32, long long n, int cols, const double *scale) {
    const long long total = n * cols;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x)
        X[e] = scale[e / n] * (double)D32[e];
}

// ---- Householder reflector application on a tile-layout FP64 matrix -----------------------
// X(i,j) -= 2 * a_i * b_j  (rank-1 update)
__global__ void rank1_kernel(double *X, int n, int nb, const double *a, const double *b) {
    const long long total = (long long)n * n;
    const int mt = n / nb;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const long long t = e / ((long long)nb * nb);
        const int in = (int)(e - t * (long long)nb * nb);
        const long long i = (t % mt) * nb + in % nb, j = (t / mt) * nb + in / nb;
        X[e] -= 2.0 * a[i] * b[j];
    }
}
// diagonal tile matrix with s_i = kappa^(-i/(n-1))
__global__ void diag_kernel(double *X, int n, int nb, double kappa) {
    const long long total = (long long)n * n;
    const int mt = n / nb;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const long long t = e / ((long long)nb * nb);
        const int in = (int)(e - t * (long long)nb * nb);
        const long long i = (t % mt) * nb + in % nb, j = (t / mt) * nb + in / nb;
        X[e] = (i == j) ? pow(kappa, -(double)i / (double)(n > 1 ? n - 1 : 1)) : 0.0;
    }
}
// y = A^T x for one vector (tile layout): one warp per output, lanes walk a tile column
// (contiguous).  y = A x: one thread per output row, a warp reads 32 consecutive rows of a
// column (contiguous) per step.
__global__ void matvec_t_kernel(const double *A, int n, int nb, const double *x, double *y) {
    const int mt = n / nb;
    const long long col = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (col >= n) return;
    double s = 0.0;
    for (int j = lane; j < n; j += 32)
        s = fma(A[(size_t)nb * nb * ((size_t)(j / nb) + (size_t)mt * (col / nb)) + (size_t)(j % nb) + (size_t)(col % nb) * nb],
                x[j], s);
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) y[col] = s;
}
__global__ void matvec_n_kernel(const double *A, int n, int nb, const double *x, double *y) {
    const int mt = n / nb;
    const long long row = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (row >= n) return;
    const double *base = A + (size_t)nb * nb * (size_t)(row / nb) + (size_t)(row % nb);
    double s = 0.0;
    for (int j = 0; j < n; j++) s = fma(base[(size_t)nb * nb * (size_t)mt * (j / nb) + (size_t)(j % nb) * nb], x[j], s);
    y[row] = s;
}

// lower triangle := upper triangle (exact symmetry of a generated SPD matrix)
__global__ void symmetrize_kernel(double *X, int n, int nb) {
    const long long total = (long long)n * n;
    const int mt = n / nb;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const long long t = e / ((long long)nb * nb);
        const int in = (int)(e - t * (long long)nb * nb);
        const long long i = (t % mt) * nb + in % nb, j = (t / mt) * nb + in / nb;
        if (i > j)
            X[e] = X[(size_t)nb * nb * ((size_t)(j / nb) + (size_t)mt * (i / nb)) + (size_t)(j % nb) + (size_t)(i % nb) * nb];
    }
}

// record the step of a diagonal-tile factorization until the first error
__global__ void mark_step_kernel(int *st, int k) {
    if (st[ST_CODE] == 0) st[6] = k;
}

}  // namespace mps

// ---------------------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------------------
cudaError_t mps_configure() {
    cudaError_t e = cudaFuncSetAttribute(mps::panel_trsm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, mps::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(mps::invert_diag_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, mps::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(mps::half_panel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, mps::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(mps::half_update_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, mps::SMEM_BYTES);
}

// (tile rows [r0, r1) only; r1 < 0: all)
cudaError_t mps_f64_to_f32(const double *A, float *W, int n, int nb, double shift, cudaStream_t s, double *amax,
                           bool upper_only, int r0, int r1) {
    const long long items = (long long)(n / nb) * (n / nb) * ((nb * nb + mps::kConvChunk - 1) / mps::kConvChunk);
    note_launch();
    mps::f64_to_f32_kernel<<<(int)std::min<long long>(items, 2048), 256, 0, s>>>(
        A, W, n, nb, shift, upper_only ? 1 : 0, r0, r1 < 0 ? n / nb : r1, amax);
    return cudaGetLastError();
}
// The lower triangle of the symmetric tile-layout matrix A from its upper triangle.
cudaError_t mps_mirror_upper(double *A, int n, int nb, cudaStream_t s) {
    if (n <= 0 || nb <= 0 || nb % 32 || n % nb) return cudaErrorInvalidValue;
    const long long blocks = (long long)(n / 32) * (n / 32 + 1) / 2;
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    note_launch();
    mps::mirror_upper_kernel<<<(int)std::min<long long>(blocks, (long long)std::max(1, sms) * 8), 256, 0, s>>>(A, n, nb);
    return cudaGetLastError();
}
// R = B - A X in compensated FP32 (see residual_df_kernel); sigma: |a_ij| < 2^sigma for all
// entries.  Xs (n x 16 float2) and tau (16 ints) are scratch; colmax = per-column max |x|.
cudaError_t mps_residual_df(const double *A, int n, int nb, const double *X, const double *colmax, const double *B,
                            double *R, int nrhs, int sigma, float2 *Xs, int *tau, double *amax, cudaStream_t s) {
    note_launch();
    mps::split_x_kernel<<<1024, 256, 0, s>>>(X, n, nrhs, colmax, Xs, tau);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    note_launch();
    mps::residual_df_kernel<<<n / 32, 128, 0, s>>>(A, n, nb, Xs, tau, sigma, B, R, nrhs, amax);
    return cudaGetLastError();
}
// R <- R - A D (update-form residual, see residual_update_kernel); colmax = per-column max
// |d|; Ds (n x 16 floats) and tau (16 ints) are scratch.
cudaError_t mps_residual_update(const double *A, int n, int nb, const double *D, const double *colmax, double *R,
                                int nrhs, int sigma, float *Ds, int *tau, cudaStream_t s) {
    note_launch();
    mps::d_to_f32_kernel<<<1024, 256, 0, s>>>(D, n, nrhs, colmax, Ds, tau);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    note_launch();
    mps::residual_update_kernel<<<n / 32, 128, 0, s>>>(A, n, nb, Ds, tau, sigma, R, nrhs);
    return cudaGetLastError();
}
cudaError_t mps_tile_to_f64(const float *w, double *d, int nb, cudaStream_t s) {
    note_launch();
    mps::tile_f32_to_f64_kernel<<<256, 256, 0, s>>>(w, d, nb * nb);
    return cudaGetLastError();
}
cudaError_t mps_tile_to_f32(const double *d, float *w, int nb, int upper_only, cudaStream_t s) {
    note_launch();
    mps::tile_f64_to_f32_kernel<<<256, 256, 0, s>>>(d, w, nb, upper_only);
    return cudaGetLastError();
}
cudaError_t mps_invert_diag(const float *W, int n, int nb, float *Dinv, int kind, cudaStream_t s) {
    dim3 grid(nb / 64, n / nb);
    note_launch();
    mps::invert_diag_kernel<<<grid, mps::NT, mps::SMEM_BYTES, s>>>(W, n, nb, Dinv, kind);
    return cudaGetLastError();
}
// binv (2 nb x 64 floats): inverses of the 64 x 64 diagonal blocks of tile k's upper factor,
// and for LU (factors = 2) of its unit lower factor
// (blocks: how many leading 64 x 64 diagonal blocks, 0 = all nb / 64)
cudaError_t mps_block_inverse(const float *W, int n, int nb, int k, int factors, float *binv, cudaStream_t s,
                              int blocks) {
    note_launch();
    mps::block_inverse_kernel<<<dim3(blocks > 0 ? blocks : nb / 64, factors), 256, 0, s>>>(W, n, nb, k, binv);
    return cudaGetLastError();
}
cudaError_t mps_half_panel(float *T, int h, int ld, const float *binv, int alg, cudaStream_t s) {
    note_launch();
    mps::half_panel_kernel<<<dim3(h / 64, alg == 0 ? 1 : 2), mps::NT, mps::SMEM_BYTES, s>>>(T, h, ld, binv, alg);
    return cudaGetLastError();
}
cudaError_t mps_half_update(float *T, int h, int ld, int alg, cudaStream_t s) {
    const int nbl = h / 64;
    note_launch();
    mps::half_update_kernel<<<alg == 0 ? nbl * (nbl + 1) / 2 : nbl * nbl, mps::NT, mps::SMEM_BYTES, s>>>(T, h, ld,
                                                                                                        alg);
    return cudaGetLastError();
}
// ph / pl: optional packed BF16 row-panel operand written by the solve (kinds 0 and 1)
cudaError_t mps_panel_trsm(float *W, int n, int nb, int k, int kind, const float *binv, cudaStream_t s, void *ph,
                           void *pl, int t0, int count, bool tc) {
    const int ntr = n / nb - k - 1;
    if (count < 0) count = ntr - t0;
    if (ntr <= 0 || count <= 0) return cudaSuccess;
    if (t0 < 0 || t0 + count > ntr) return cudaErrorInvalidValue;
    dim3 grid(nb / 64, count);
    note_launch();
    mps::panel_trsm_kernel<<<grid, mps::NT, mps::SMEM_BYTES, s>>>(W, n, nb, k, kind, binv,
                                                                   kind == 2 ? nullptr : static_cast<__nv_bfloat16 *>(ph),
                                                                   kind == 2 ? nullptr : static_cast<__nv_bfloat16 *>(pl), t0,
                                                                   tc ? 1 : 0);
    return cudaGetLastError();
}
cudaError_t mps_residual(const double *A, int n, int nb, const double *X, const double *B, double *R, int nrhs,
                         double *amax, cudaStream_t s) {
    note_launch();
    mps::residual_kernel<<<n / 32, 256, 0, s>>>(A, n, nb, X, B, R, nrhs, amax);
    return cudaGetLastError();
}
cudaError_t mps_norm_inf_matrix(const double *A, int n, int nb, double *out, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double), s);
    if (e != cudaSuccess) return e;
    note_launch();
    mps::rowsum_kernel<<<n / 64, 256, 0, s>>>(A, n, nb, out);
    return cudaGetLastError();
}
cudaError_t mps_colmax(const double *X, long long n, int cols, double *out, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double) * cols, s);
    if (e != cudaSuccess) return e;
    dim3 grid(64, cols);
    note_launch();
    mps::colmax_kernel<<<grid, 256, 0, s>>>(X, n, cols, out);
    return cudaGetLastError();
}
cudaError_t mps_to_f32_rhs(const double *R, float *R32, long long n, int cols, const double *scale, cudaStream_t s) {
    note_launch();
    mps::to_f32_rhs_kernel<<<2048, 256, 0, s>>>(R, R32, n, cols, scale);
    return cudaGetLastError();
}
cudaError_t mps_mark_step(int *status, int k, cudaStream_t s) {
    note_launch();
    mps::mark_step_kernel<<<1, 1, 0, s>>>(status, k);
    return cudaGetLastError();
}
cudaError_t mps_multi_dot(const double *V, int count, const double *w, long long n, int nrhs, double *H,
                          cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(H, 0, sizeof(double) * count * nrhs, s);
    if (e != cudaSuccess || count <= 0) return e;
    dim3 grid(128, count);
    note_launch();
    mps::multi_dot_kernel<<<grid, 256, 0, s>>>(V, count, w, n, nrhs, H);
    return cudaGetLastError();
}
cudaError_t mps_multi_axpy(const double *V, int count, const double *H, double *w, long long n, int nrhs, int assign,
                           cudaStream_t s) {
    note_launch();
    mps::multi_axpy_kernel<<<2048, 256, 0, s>>>(V, count, H, w, n, nrhs, assign);
    return cudaGetLastError();
}
cudaError_t mps_scale_cols(const double *w, double *out, long long n, int nrhs, const double *f, cudaStream_t s) {
    note_launch();
    mps::scale_cols_kernel<<<2048, 256, 0, s>>>(w, out, n, nrhs, f);
    return cudaGetLastError();
}
cudaError_t mps_from_f32_rhs(double *X, const float *D32, long long n, int cols, const double *scale, cudaStream_t s) {
    note_launch();
    mps::from_f32_rhs_kernel<<<2048, 256, 0, s>>>(X, D32, n, cols, scale);
    return cudaGetLastError();
}
cudaError_t mps_rank1(double *X, int n, int nb, const double *a, const double *b, cudaStream_t s) {
    note_launch();
    mps::rank1_kernel<<<4096, 256, 0, s>>>(X, n, nb, a, b);
    return cudaGetLastError();
}
cudaError_t mps_diag(double *X, int n, int nb, double kappa, cudaStream_t s) {
    note_launch();
    mps::diag_kernel<<<4096, 256, 0, s>>>(X, n, nb, kappa);
    return cudaGetLastError();
}
cudaError_t mps_matvec(const double *A, int n, int nb, const double *x, double *y, int trans, cudaStream_t s) {
    if (trans) {
        const long long threads = (long long)n * 32;
        note_launch();
        mps::matvec_t_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(A, n, nb, x, y);
    } else {
        note_launch();
        mps::matvec_n_kernel<<<(n + 127) / 128, 128, 0, s>>>(A, n, nb, x, y);
    }
    return cudaGetLastError();
}

cudaError_t mps_symmetrize(double *X, int n, int nb, cudaStream_t s) {
    note_launch();
    mps::symmetrize_kernel<<<4096, 256, 0, s>>>(X, n, nb);
    return cudaGetLastError();
}


}  // namespace palial
