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
// Layout: warp = 16 rows of A x all 16 right-hand sides, CTA = 4 warps (64 rows) over one range
// of K chunks (the K range of a 64-row block is split over several CTAs so that the launch fills
// whole waves).  Per K16 step a thread loads the 8 FP64 entries of its mma.sync m16n8k16 A
// fragment straight from the tile layout (rows g, g + 8, columns 2t, 2t + 1, 2t + 8, 2t + 9 of
// the step), digitises them in registers (integer operations on the bit pattern, no FP64 pipe)
// and issues the 26 digit-pair MMAs per 8-column half of the 16 right-hand sides.  X's digits
// are prepared once per call in a fragment-ordered buffer and staged per chunk in shared memory
// (cp.async, double-buffered).  The next chunk's A entries are in flight while the current chunk
// computes.  The CTAs' integer partial sums meet in global memory by integer atomics (exact, so
// the result is the same for every split and order); a last kernel converts them to FP64 and
// forms B - A X.  Integer row sums of |a| give ||A||_inf when asked for.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
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

// Magnitude form for A's fragments: |v| * 2^(47 - sc) rounded (half away from zero, as to_v48)
// split into its top and bottom 24 bits (vh, vl), and the sign bit of v; *bad as to_v48.
__device__ __forceinline__ void to_mag48(double v, int sc, bool &bad, unsigned &vh, unsigned &vl, unsigned &neg) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
    const int E = (int)((bits >> 52) & 0x7FF);
    const unsigned long long mant = (bits & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
    const int shift = 1028 + sc - E;  // >= 6 exactly when |v| < 2^sc
    bad |= (E == 0x7FF) | (E != 0 && shift < 6);
    const unsigned long long m =
        (E == 0 || shift >= 64 || shift < 6) ? 0ull : ((mant + (1ull << (shift - 1))) >> shift);
    vh = (unsigned)(m >> 24);
    vl = (unsigned)m & 0xFFFFFFu;
    neg = (unsigned)(bits >> 63);
}
// Digit p (0 = most significant) of the 48-bit magnitude (vh, vl) as a float (exact).
__device__ __forceinline__ float mdigit(unsigned vh, unsigned vl, int p) {
    return (float)(p < 3 ? (vh >> (16 - 8 * p)) & 255u : (vl >> (40 - 8 * p)) & 255u);
}

// Digit p of a 48-bit two's complement integer as a float (exact).
__device__ __forceinline__ float digit(long long V, int p) {
    return p == 0 ? (float)(int)(V >> 40) : (float)(int)((V >> (40 - 8 * p)) & 255);
}

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);  // .x (low half) = lo
    return *reinterpret_cast<const uint32_t *>(&h);
}

// Not volatile: the MMAs have no effect beyond their outputs, so the compiler may interleave them
// with the digit arithmetic of the next fragments.
__device__ __forceinline__ void mma16816(float *d, const uint32_t *a, uint32_t b0, uint32_t b1) {
    asm(
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

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

constexpr int XQ = ND * 16 * 4;  // 16-byte words of X digits per chunk (6 KB)

constexpr int AP = 66;  // pitch (doubles) of a staged A column: fragment reads of a half-warp
                        // (rows g, columns 2t) fall in 16 distinct 8-byte bank pairs
constexpr int CTAS_PER_SM = 3;

// Partial products of rows blockIdx.x * 64 .. + 63 over the K chunks [blockIdx.y * cps, + cps):
// the 64-bit integer sums (hi, lo) of every output entry and the integer |a| row sums are added
// into acc / rsum with integer atomics (exact, so the result does not depend on the order or on
// the split); a row whose entries include Inf / NaN or exceed 2^sigma is flagged in badrow.
// The next chunk's A block (64 rows x 32 columns, 512 contiguous bytes per column in the tile
// layout) and X digit fragments are copied into shared memory by cp.async while the current
// chunk multiplies, so a thread holds no prefetch registers and three CTAs fit on an SM.
__global__ void __launch_bounds__(NT, CTAS_PER_SM) residual_digits_kernel(const double *A, int n, int nb,
                                                                          const uint32_t *Xd, int sigma, int cps,
                                                                          int nrhs, unsigned long long *acc,
                                                                          unsigned long long *rsum, int *badrow,
                                                                          int want_norm) {
    __shared__ __align__(16) double sa[2][KC][AP];
    __shared__ __align__(16) uint4 sx[2][XQ];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int r0 = blockIdx.x * 64;   // first row of this CTA (inside one tile row: nb % 64 == 0)
    const int wr = warp * 16;         // first row of this warp within the CTA's 64
    const int cb = blockIdx.y * cps, ce = min(n / KC, cb + cps);
    if (cb >= ce) return;  // uniform per CTA
    const int mt = n / nb;
    const double *rowbase = A + (size_t)nb * nb * (size_t)(r0 / nb) + (size_t)(r0 % nb);
    long long hi[2][4], lo[2][4];
#pragma unroll
    for (int h = 0; h < 2; h++)
#pragma unroll
        for (int e = 0; e < 4; e++) hi[h][e] = lo[h][e] = 0;
    // |a| row sums of rows g and g + 8 over this thread's columns, in units of 2^(sigma - 23)
    // (V >> 24: the norm needs no more than that)
    long long asum0 = 0, asum1 = 0;
    bool bad = false;
    // chunk ch -> buffer buf: A columns k0 .. k0 + 31 of the CTA's rows (16-byte pieces: column
    // c = i / 32, rows 2 (i % 32) ..), and X's 6 KB of digit fragments
    auto stage = [&](int ch, int buf) {
        const int k0 = ch * KC;
        const double *src = rowbase + (size_t)nb * nb * (size_t)mt * (size_t)(k0 / nb) + (size_t)(k0 % nb) * nb;
#pragma unroll
        for (int j = 0; j < (KC * 32) / NT; j++) {
            const int i = threadIdx.x + NT * j, c = i >> 5, r = 2 * (i & 31);
            cp_async16(&sa[buf][c][r], src + (size_t)c * nb + r);
        }
        const uint4 *xs = reinterpret_cast<const uint4 *>(Xd) + (size_t)ch * XQ;
        for (int i = threadIdx.x; i < XQ; i += NT) cp_async16(&sx[buf][i], xs + i);
        cp_async_commit();
    };
    stage(cb, 0);
    for (int ch = cb; ch < ce; ch++) {
        const int buf = (ch - cb) & 1;
        if (ch + 1 < ce) {
            stage(ch + 1, buf ^ 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();  // this chunk's A block and X digits are in sa[buf], sx[buf]
        float accf[SMAX + 1][2][4];
#pragma unroll
        for (int s = 0; s <= SMAX; s++)
#pragma unroll
            for (int h = 0; h < 2; h++)
#pragma unroll
                for (int e = 0; e < 4; e++) accf[s][h][e] = 0.f;
#pragma unroll
        for (int st = 0; st < 2; st++) {
            // this step's A fragment: rows g, g+8 x columns 2t, 2t+1, 2t+8, 2t+9 of the K16 step
            const int kk = 16 * st + 2 * t, ra = wr + g;
            const double a8[8] = {sa[buf][kk][ra],     sa[buf][kk + 1][ra],     sa[buf][kk][ra + 8],
                                  sa[buf][kk + 1][ra + 8], sa[buf][kk + 8][ra], sa[buf][kk + 9][ra],
                                  sa[buf][kk + 8][ra + 8], sa[buf][kk + 9][ra + 8]};
            // digits of |a| (all in [0, 255]) with a's sign set on each BF16 digit: the same
            // integer as the two's complement digits, products and chunk sums stay below 2^16
            // and 2^24
            unsigned vh[8], vl[8], ng[8];
#pragma unroll
            for (int e = 0; e < 8; e++) to_mag48(a8[e], sigma, bad, vh[e], vl[e], ng[e]);
            if (want_norm) {  // |a| >> 24 row sums (at most 16 terms of 2^24 per chunk in 32 bits)
                asum0 += (long long)(vh[0] + vh[1] + vh[4] + vh[5]);
                asum1 += (long long)(vh[2] + vh[3] + vh[6] + vh[7]);
            }
            uint32_t sg[4];  // BF16 sign bits of the two entries of each fragment register
#pragma unroll
            for (int j = 0; j < 4; j++) sg[j] = (ng[2 * j] << 15) | (ng[2 * j + 1] << 31);
            uint32_t af[ND][4];
#pragma unroll
            for (int p = 0; p < ND; p++) {
#pragma unroll
                for (int j = 0; j < 4; j++)  // j: (row g, k 2t..), (g+8, 2t..), (g, 2t+8..), (g+8, 2t+8..)
                    af[p][j] = pack2(mdigit(vh[2 * j], vl[2 * j], p), mdigit(vh[2 * j + 1], vl[2 * j + 1], p)) ^ sg[j];
            }
            // digit q of X (both 8-column halves), then every digit p of A with p + q <= SMAX:
            // consecutive MMAs go to different accumulators (weight p + q, half h)
#pragma unroll
            for (int q = 0; q < ND; q++) {
                // B fragments: k pairs (t) and (t + 4) of step st -> words 2 st, 2 st + 1
                const uint4 w0 = sx[buf][(q * 16 + g) * 4 + t], w1 = sx[buf][(q * 16 + 8 + g) * 4 + t];
                const uint32_t b00 = st == 0 ? w0.x : w0.z, b01 = st == 0 ? w0.y : w0.w;
                const uint32_t b10 = st == 0 ? w1.x : w1.z, b11 = st == 0 ? w1.y : w1.w;
#pragma unroll
                for (int p = 0; p + q <= SMAX && p < ND; p++) {
                    mma16816(accf[p + q][0], af[p], b00, b01);
                    mma16816(accf[p + q][1], af[p], b10, b11);
                }
            }
        }
        // fold the chunk's exact FP32 sums into the 64-bit accumulators
#pragma unroll
        for (int h = 0; h < 2; h++)
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const long long s0 = __float2int_rn(accf[0][h][e]), s1 = __float2int_rn(accf[1][h][e]),
                                s2 = __float2int_rn(accf[2][h][e]), s3 = __float2int_rn(accf[3][h][e]),
                                s4 = __float2int_rn(accf[4][h][e]), s5 = __float2int_rn(accf[5][h][e]),
                                s6 = __float2int_rn(accf[6][h][e]);
                hi[h][e] += (s0 << 16) + (s1 << 8) + s2;
                lo[h][e] += (s3 << 24) + (s4 << 16) + (s5 << 8) + s6;
            }
        __syncthreads();  // every warp is done with sa[buf], sx[buf] before they are refilled
    }
    const int i0 = r0 + wr;  // first row of this warp
    // partial sums: rows g (e = 0, 1) and g + 8 (e = 2, 3), columns h * 8 + 2t + (e & 1)
#pragma unroll
    for (int h = 0; h < 2; h++)
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int c = h * 8 + 2 * t + (e & 1);
            if (c >= nrhs) continue;
            const int row = i0 + g + (e >> 1) * 8;
            unsigned long long *o = acc + ((size_t)row * 16 + c) * 2;
            atomicAdd(o, (unsigned long long)hi[h][e]);
            atomicAdd(o + 1, (unsigned long long)lo[h][e]);
        }
    if (want_norm) {
        // row sums over the 4 threads of a row group
        for (int o = 1; o < 4; o <<= 1) {
            asum0 += __shfl_xor_sync(0xffffffffu, asum0, o);
            asum1 += __shfl_xor_sync(0xffffffffu, asum1, o);
        }
        if (t == 0) {
            atomicAdd(rsum + i0 + g, (unsigned long long)asum0);
            atomicAdd(rsum + i0 + g + 8, (unsigned long long)asum1);
        }
    }
    if (bad) {
        atomicOr(badrow + i0 + g, 1);
        atomicOr(badrow + i0 + g + 8, 1);
    }
}

// R = B - A x from the integer sums: A x = 2^(sigma + tau_c - 62) (hi 2^32 + lo) in FP64, NaN for
// a flagged row; with amax the largest row sum of |a| (2^(sigma - 23) units) by atomicMax on the
// FP64 bit pattern.
__global__ void finalize_kernel(const unsigned long long *acc, const unsigned long long *rsum, const int *badrow,
                                const int *tau, int sigma, const double *B, double *R, int n, int nrhs, double *amax) {
    double m = 0.0;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < (long long)n * nrhs;
         idx += (long long)gridDim.x * blockDim.x) {
        const int row = (int)(idx % n), c = (int)(idx / n);
        const unsigned long long *a = acc + ((size_t)row * 16 + c) * 2;
        double ax = ldexp((double)(long long)a[0] * 4294967296.0 + (double)(long long)a[1], sigma + tau[c] - 62);
        const bool bad = badrow[row] != 0;
        if (bad) ax = __longlong_as_double(0x7ff8000000000000ll);
        const size_t o = (size_t)row + (size_t)c * n;
        R[o] = B ? B[o] - ax : ax;
        if (amax && c == 0) {
            const double r = bad ? __longlong_as_double(0x7ff8000000000000ll) : ldexp((double)rsum[row], sigma - 23);
            m = (r != r || r > m) ? r : m;
        }
    }
    if (amax) {
        // NaN's bit pattern exceeds every finite one: a NaN row sum wins the atomicMax
        unsigned long long bits = (unsigned long long)__double_as_longlong(m);
        for (int o = 16; o; o >>= 1) {
            const unsigned long long y = __shfl_xor_sync(0xffffffffu, bits, o);
            bits = y > bits ? y : bits;
        }
        if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<unsigned long long *>(amax), bits);
    }
}

}  // namespace mrd

// Scratch of mrd_residual (bytes): X's digits (n * 48 words), 16 exponents, the integer sums
// (n x 16 x 2), the row sums (n) and the row flags (n).
size_t mrd_scratch_bytes(int n) {
    return sizeof(uint32_t) * (size_t)n * 48 + 64 * sizeof(int) + sizeof(unsigned long long) * (size_t)n * 33 +
           sizeof(int) * (size_t)n;
}

// R = B - A X (B may be NULL: R = A X) with the digit products above; sigma: |a_ij| < 2^sigma;
// colmax = per-column max |x|; scratch: mrd_scratch_bytes(n) bytes.  n % 64 == 0.  Each 64-row
// block's K range is split over several CTAs so that the launch fills whole waves of the SMs.
cudaError_t mrd_residual(const double *A, int n, int nb, const double *X, const double *colmax, const double *B,
                         double *R, int nrhs, int sigma, void *scratch, double *amax, cudaStream_t s) {
    // the 64-bit accumulators hold n / 32 chunk sums of up to 2^49: n <= 2^18
    if (n % 64 || n > (1 << 18) || nrhs < 1 || nrhs > 16) return cudaErrorInvalidValue;
    uint32_t *Xd = static_cast<uint32_t *>(scratch);
    int *tau = reinterpret_cast<int *>(Xd + (size_t)n * 48);
    unsigned long long *acc = reinterpret_cast<unsigned long long *>(tau + 64);
    unsigned long long *rsum = acc + (size_t)n * 32;
    int *badrow = reinterpret_cast<int *>(rsum + n);
    cudaError_t e = cudaMemsetAsync(acc, 0, sizeof(unsigned long long) * (size_t)n * 33 + sizeof(int) * (size_t)n, s);
    if (e != cudaSuccess) return e;
    note_launch();
    mrd::x_digits_kernel<<<1024, 256, 0, s>>>(X, n, nrhs, colmax, Xd, tau);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // K splits: the fewest (from about three waves' worth of CTAs up) whose last wave is at
    // least 90 % full
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long slots = (long long)std::max(1, sms) * mrd::CTAS_PER_SM, rows = n / 64, chunks = n / mrd::KC;
    long long ks = std::max(1LL, (3 * slots + rows - 1) / rows);
    for (long long k2 = ks; k2 <= std::max(ks, std::min(4 * ks, chunks)); k2++) {
        const long long tot = rows * k2, waves = (tot + slots - 1) / slots;
        if (10 * tot >= 9 * waves * slots) {
            ks = k2;
            break;
        }
    }
    ks = std::min(ks, chunks);
    const int cps = (int)((chunks + ks - 1) / ks);
    ks = (chunks + cps - 1) / cps;
    note_launch();
    mrd::residual_digits_kernel<<<dim3((unsigned)rows, (unsigned)ks), mrd::NT, 0, s>>>(A, n, nb, Xd, sigma, cps, nrhs,
                                                                                       acc, rsum, badrow, amax ? 1 : 0);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    note_launch();
    mrd::finalize_kernel<<<(int)std::min<long long>(((long long)n * nrhs + 255) / 256, 4096), 256, 0, s>>>(
        acc, rsum, badrow, tau, sigma, B, R, n, nrhs, amax);
    return cudaGetLastError();
}

}  // namespace palial
