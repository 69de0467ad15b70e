// mp_gemm.cu -- tcgen05 (5th-generation tensor core) trailing update of the mixed-precision
// factorizations: C -= A_op * B_op^T on the FP32 trailing matrix, for every trailing tile of
// one k step, with low-precision operands packed from the step's panel.
//
//   Cholesky: C(n,m) -= U(k,n)^T U(k,m)    A_op = B_op = packed panel row k
//   LU:       C(m,n) -= L(m,k) U(k,n)      A_op = packed panel column k, B_op = panel row k
//
// Operands are K-major bf16 (or e4m3) matrices "rows x NB" (a packed panel: row r holds the
// K = NB values that multiply trailing row/column r).  Each CTA computes one 128 x 256 output
// block of one 512-aligned trailing tile:
//   warp 0 lane 0  TMA producer: 128B-swizzled boxes of 128 (A) and 256 (B) rows x 128 bytes
//                  of K into a 4-stage shared-memory ring (mbarrier complete_tx);
//   warp 1 lane 0  MMA issuer: tcgen05.mma (M=128, N=256, K=16 bf16 / 32 fp8) into a TMEM
//                  accumulator of 256 FP32 columns; tcgen05.commit frees ring slots;
//   all 4 warps    epilogue: tcgen05.ld 32 lanes x 16 columns at a time, C -= scale * D with
//                  coalesced FP32 loads/stores in the reference's tile layout.
// Modes: BF16 (one MMA per K slice), FP8 e4m3 (per-tile scales applied in the epilogue),
// BF16X3 (operands split x = hi + lo in bf16; hi*hi + hi*lo + lo*hi accumulated in TMEM) and
// TF32X3 (the same three products with x = hi + lo in TF32, kind::tf32: about 21 bits per
// product, the FP32-level rung of the precision ladder).
// Every mbarrier wait is bounded; on expiry the CTA records an error, drains its own TMA
// copies and frees its TMEM before returning.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"

namespace palial {
namespace mp {

constexpr int BM = 128, BN = 256;      // CTA output block
constexpr int KBYTES = 128;            // bytes of K per stage (one 128B swizzle row)
constexpr int NTHR = 128;
constexpr uint32_t TMEM_COLS = 256;
constexpr uint32_t WAIT_LIMIT = 1u << 24;  // bounded spin (about a second with back-off)

enum Mode { MODE_BF16 = 0, MODE_FP8 = 1, MODE_BF16X3 = 2, MODE_TF32X3 = 3 };

template <int MODE>
struct Cfg {
    static constexpr bool SPLIT = (MODE == MODE_BF16X3 || MODE == MODE_TF32X3);
    static constexpr int NOPS = SPLIT ? 2 : 1;   // hi (+ lo) operand copies
    // K = NB = 512 is only 8 (bf16), 4 (fp8) or 16 (tf32) stages.  2 CTAs share an SM (2 x 256
    // TMEM columns, 2 x 128 threads x 256 registers), so one CTA's epilogue overlaps the
    // other's loads and MMAs: bf16 and fp8 keep a 2-stage ring (96 KB); a split mode's stage
    // holds four operand boxes (96 KB), so it runs one stage per CTA to fit two CTAs.
    static constexpr int STAGES = SPLIT ? 1 : 2;
    static constexpr int A_BYTES = BM * KBYTES;                  // 16 KB
    static constexpr int B_BYTES = BN * KBYTES;                  // 32 KB
    static constexpr int STAGE_BYTES = NOPS * (A_BYTES + B_BYTES);
    static constexpr int SMEM = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
    static constexpr int ELEM = (MODE == MODE_FP8) ? 1 : (MODE == MODE_TF32X3) ? 4 : 2;  // bytes per element
    static constexpr int KELEMS = KBYTES / ELEM;                 // elements of K per stage
    // operand format field: e4m3 0 (kind::f8f6f4), bf16 1 (kind::f16), tf32 2 (kind::tf32)
    static constexpr uint32_t FMT = (MODE == MODE_FP8) ? 0u : (MODE == MODE_TF32X3) ? 2u : 1u;
    // instruction descriptor: D=F32, A/B format, K-major A and B, N>>3, M>>4
    static constexpr uint32_t IDESC = (1u << 4) | (FMT << 7) | (FMT << 10) | ((uint32_t)(BN >> 3) << 17) |
                                      ((uint32_t)(BM >> 4) << 24);
};

struct UpdateParams {
    float *C;                 // FP32 tile-layout matrix, n x n
    int n, nb;                // size, tile size (multiple of 256)
    int k;                    // step: trailing tiles start at tile k+1
    int ntr;                  // trailing tiles per dimension
    int upper;                // 1: only tile pairs (ti <= tj) (Cholesky), 0: all (LU)
    int part;                 // 0: every pair; 1: the next step's tiles (row 0; LU also column
                              // 0); 2: all other pairs (lookahead split); 3 (upper only): the
                              // pairs of trailing rows r0 <= ti < r1, row by row; 4: the pair
                              // (0, 0) alone; 5: part 1 without the pair (0, 0)
    int r0, r1;               // part 3 row range (trailing-relative)
    const float *scale_a;     // FP8: per trailing tile scale of A_op rows (nullptr: 1)
    const float *scale_b;     // FP8: per trailing tile scale of B_op rows
    int *status;              // error word (ST_CODE slot)
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: true when the phase of `parity` completed, false after WAIT_LIMIT tries.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    for (uint32_t i = 0; i < WAIT_LIMIT; i++) {
        if (mbar_try(bar, parity)) return true;
        if (i > 32) __nanosleep(64);
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Shared-memory matrix descriptor: K-major, rows of SWB bytes of K swizzled in SWB-byte
// atoms (128B swizzle: layout type 2, 64B: type 4), 8-row atoms 8 * SWB bytes apart.
template <int SWB = 128>
__device__ __forceinline__ uint64_t smem_desc(const void *p) {
    static_assert(SWB == 128 || SWB == 64, "swizzle width");
    const uint32_t a = smem_u32(p);
    uint64_t d = 0;
    d |= (uint64_t)((a & 0x3FFFF) >> 4);            // start address
    d |= (uint64_t)1 << 16;                         // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)((8 * SWB) >> 4) << 32;          // stride byte offset: 8 rows x SWB bytes
    d |= (uint64_t)1 << 46;                         // descriptor version (sm_100 family)
    d |= (uint64_t)(SWB == 128 ? 2 : 4) << 61;      // SWIZZLE_128B / SWIZZLE_64B
    return d;
}

template <int MODE>
__device__ __forceinline__ void mma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t accumulate) {
    if (MODE == MODE_FP8) {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
            "l"(a), "l"(b), "r"(Cfg<MODE>::IDESC), "r"(accumulate));
    } else if (MODE == MODE_TF32X3) {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
            "l"(a), "l"(b), "r"(Cfg<MODE>::IDESC), "r"(accumulate));
    } else {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
            "l"(a), "l"(b), "r"(Cfg<MODE>::IDESC), "r"(accumulate));
    }
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void decode_pair(int q, int ntr, int upper, int &ti, int &tj);
// Pair q of the launch's part (see UpdateParams::part).
__device__ __forceinline__ void decode_part(int q, int ntr, int upper, int part, int &ti, int &tj, int r0) {
    if (part == 3) {  // row ti holds ntr - ti pairs (tj >= ti)
        ti = r0;
        while (q >= ntr - ti) {
            q -= ntr - ti;
            ti++;
        }
        tj = ti + q;
        return;
    }
    if (part == 1) {
        if (upper || q < ntr) {
            ti = 0;
            tj = q;
        } else {
            ti = q - ntr + 1;
            tj = 0;
        }
        return;
    }
    if (part == 4) {  // the next step's diagonal tile alone
        ti = tj = 0;
        return;
    }
    if (part == 5) {  // the next step's row (LU: and column) without its diagonal tile
        if (upper || q < ntr - 1) {
            ti = 0;
            tj = q + 1;
        } else {
            ti = q - (ntr - 1) + 1;
            tj = 0;
        }
        return;
    }
    if (part == 2) {
        decode_pair(q, ntr - 1, upper, ti, tj);
        ti++;
        tj++;
        return;
    }
    decode_pair(q, ntr, upper, ti, tj);
}
__device__ __forceinline__ void decode_pair(int q, int ntr, int upper, int &ti, int &tj) {
    if (!upper) {
        ti = q % ntr;
        tj = q / ntr;
        return;
    }
    int j = (int)((sqrtf(8.0f * (float)q + 1.0f) - 1.0f) * 0.5f);
    while (j * (j + 1) / 2 > q) j--;
    while ((j + 1) * (j + 2) / 2 <= q) j++;
    tj = j;
    ti = q - j * (j + 1) / 2;
}

template <int MODE>
__global__ void __launch_bounds__(NTHR, 1)
    mp_update_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb,
                     const __grid_constant__ CUtensorMap ta_lo, const __grid_constant__ CUtensorMap tb_lo,
                     UpdateParams p) {
    using C = Cfg<MODE>;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(base + C::STAGES * C::STAGE_BYTES);
    uint64_t *empty = full + C::STAGES;
    uint64_t *done = empty + C::STAGES;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
    __shared__ int s_abort;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sub_m = p.nb / BM, sub_n = p.nb / BN;
    const int q = blockIdx.x / (sub_m * sub_n), sub = blockIdx.x % (sub_m * sub_n);
    int ti, tj;
    decode_part(q, p.ntr, p.upper, p.part, ti, tj, p.r0);
    const int mi = sub % sub_m, nj = sub / sub_m;
    const int arow = ti * p.nb + mi * BM;   // first row of A_op
    const int brow = tj * p.nb + nj * BN;   // first row of B_op
    const int kstages = p.nb * C::ELEM / KBYTES;

    if (threadIdx.x == 0) {
        for (int s = 0; s < C::STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        // ---- TMA producer ----
        int issued = 0;
        for (int kb = 0; kb < kstages; kb++) {
            const int s = kb % C::STAGES;
            if (kb >= C::STAGES && !mbar_wait(&empty[s], ((kb / C::STAGES) - 1) & 1)) {
                s_abort = 1;
                break;
            }
            uint8_t *st = base + s * C::STAGE_BYTES;
            mbar_expect_tx(&full[s], C::STAGE_BYTES);
            const int kx = kb * C::KELEMS;
            tma_load_2d(st, &ta, kx, arow, &full[s]);
            tma_load_2d(st + C::A_BYTES, &tb, kx, brow, &full[s]);
            if (C::NOPS == 2) {
                tma_load_2d(st + C::A_BYTES + C::B_BYTES, &ta_lo, kx, arow, &full[s]);
                tma_load_2d(st + 2 * C::A_BYTES + C::B_BYTES, &tb_lo, kx, brow, &full[s]);
            }
            issued = kb + 1;
        }
        if (s_abort) {
            // drain: wait (bounded) for this CTA's own copies that may still be landing
            for (int kb = issued - C::STAGES < 0 ? 0 : issued - C::STAGES; kb < issued; kb++)
                mbar_wait(&full[kb % C::STAGES], (kb / C::STAGES) & 1);
        }
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer ----
        bool ok = true;
        for (int kb = 0; kb < kstages; kb++) {
            const int s = kb % C::STAGES;
            if (!mbar_wait(&full[s], (kb / C::STAGES) & 1)) {
                ok = false;
                s_abort = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            uint8_t *st = base + s * C::STAGE_BYTES;
            const uint64_t da = smem_desc(st), db = smem_desc(st + C::A_BYTES);
#pragma unroll
            for (int kk = 0; kk < KBYTES / 32; kk++) {  // K slice: 32 bytes (16 bf16, 32 e4m3, 8 tf32)
                const uint32_t acc = (kb | kk) ? 1u : 0u;
                mma<MODE>(tmem, da + 2 * kk, db + 2 * kk, acc);  // +32 B per K slice
                if (C::NOPS == 2) {
                    const uint64_t dal = smem_desc(st + C::A_BYTES + C::B_BYTES);
                    const uint64_t dbl = smem_desc(st + 2 * C::A_BYTES + C::B_BYTES);
                    mma<MODE>(tmem, da + 2 * kk, dbl + 2 * kk, 1u);   // hi * lo
                    mma<MODE>(tmem, dal + 2 * kk, db + 2 * kk, 1u);   // lo * hi
                }
            }
            mma_commit(&empty[s]);
        }
        if (ok) mma_commit(done);
    }
    __syncwarp();
    // ---- epilogue: all four warps; thread = accumulator row, 64 columns per pass ----
    // The old C values of a pass are loaded as 64 independent loads before they are needed
    // (the first pass before the MMA has finished), so each pass costs one memory round trip.
    const int mt = p.n / p.nb;
    const int tr = p.k + 1 + ti, tc = p.k + 1 + tj;
    float *ct = p.C + (size_t)p.nb * p.nb * ((size_t)tr + (size_t)mt * tc) + (size_t)(mi * BM + warp * 32 + lane) +
                (size_t)(nj * BN) * p.nb;
    float cold[64];
#pragma unroll
    for (int c = 0; c < 64; c++) cold[c] = __ldcs(ct + (size_t)c * p.nb);
    bool have = false;
    if (!s_abort) have = mbar_wait(done, 0);
    if (!have) {
        if (lane == 0) atomicCAS(p.status + ST_CODE, 0, -4);
    } else {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        float sc = 1.0f;
        if (MODE == MODE_FP8 && p.scale_a) sc = p.scale_a[ti] * p.scale_b[tj];
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
        for (int c0 = 0; c0 < BN; c0 += 64) {
            float d[64];
            tmem_ld16(trow + (uint32_t)c0, d);
            tmem_ld16(trow + (uint32_t)(c0 + 16), d + 16);
            tmem_ld16(trow + (uint32_t)(c0 + 32), d + 32);
            tmem_ld16(trow + (uint32_t)(c0 + 48), d + 48);
            float nxt[64];
            if (c0 + 64 < BN) {
#pragma unroll
                for (int c = 0; c < 64; c++) nxt[c] = __ldcs(ct + (size_t)(c0 + 64 + c) * p.nb);
            }
#pragma unroll
            for (int c = 0; c < 64; c++) __stcs(ct + (size_t)(c0 + c) * p.nb, fmaf(-sc, d[c], cold[c]));
            if (c0 + 64 < BN) {
#pragma unroll
                for (int c = 0; c < 64; c++) cold[c] = nxt[c];
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
}

// ---------------------------------------------------------------------------------------
// Tile runs: one CTA per SM works through `run` consecutive 128 x 256 output blocks with
// double-buffered TMEM accumulators (2 x 256 columns), so the epilogue of one block overlaps
// the MMAs of the next, and a 192 KB shared-memory ring (2 stages for the split modes, 4 for
// BF16 / FP8) keeps TMA loads ahead of the MMAs.  Roles:
//   warp 0 lane 0   TMA producer over the run's blocks and K stages (ring slots freed by the
//                   MMA warp's tcgen05.commit on empty[s]);
//   warp 1 lane 0   MMA issuer: block j accumulates into columns (j % 2) * 256, waits until
//                   the epilogue has drained that accumulator (tempty), commits tfull;
//   warps 2..5      epilogue: warp w reads TMEM lanes 32 * (w % 4) .. + 31 (the quarter its
//                   warp index may access), C -= scale * D as in mp_update_kernel.
// The CTA retires after its run (a few tens of microseconds), so kernels of the
// high-priority stream (the factorization's critical chain) get SMs between runs.  The MMA
// sequence and epilogue arithmetic per block equal mp_update_kernel's: the same bits.
// ---------------------------------------------------------------------------------------
constexpr int RUN_THREADS = 192;
constexpr uint32_t RUN_TMEM_COLS = 512;

// Stage geometry of the run kernel: 64 bytes of K per stage (one 64B-swizzled row), so the
// 192 KB ring holds 4 stages for the split modes (8 otherwise): with 2 stages of 128 bytes the
// MMA warp waited on TMA refills (ncu: tensor pipe 50 % of active cycles, neither L2 nor DRAM
// busy); 4 shorter stages keep three refills in flight behind the one being consumed.
template <int MODE>
struct RunCfg {
    using C = Cfg<MODE>;
    static constexpr int KB = 64;                                  // bytes of K per stage
    static constexpr int A_BYTES = BM * KB;                        // 8 KB
    static constexpr int B_BYTES = BN * KB;                        // 16 KB
    static constexpr int STAGE_BYTES = C::NOPS * (A_BYTES + B_BYTES);
    static constexpr int STAGES = (192 * 1024) / STAGE_BYTES;      // 4 (split) or 8
    static constexpr int KELEMS = KB / C::ELEM;
    static constexpr int SMEM = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
};

struct RunParams {
    UpdateParams u;
    long long nblocks;        // output blocks of the launch (pairs x sub-blocks)
    int run;                  // blocks per CTA
};

__device__ __forceinline__ void block_coords(const UpdateParams &p, long long g, int &ti, int &tj, int &mi,
                                             int &nj) {
    const int sub_m = p.nb / BM, sub_n = p.nb / BN;
    const int q = (int)(g / (sub_m * sub_n)), sub = (int)(g % (sub_m * sub_n));
    decode_part(q, p.ntr, p.upper, p.part, ti, tj, p.r0);
    mi = sub % sub_m;
    nj = sub / sub_m;
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

template <int MODE>
__global__ void __launch_bounds__(RUN_THREADS, 1)
    mp_update_run_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb,
                         const __grid_constant__ CUtensorMap ta_lo, const __grid_constant__ CUtensorMap tb_lo,
                         RunParams rp) {
    using C = Cfg<MODE>;
    using R = RunCfg<MODE>;
    constexpr int S = R::STAGES;
    const UpdateParams &p = rp.u;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(base + S * R::STAGE_BYTES);
    uint64_t *empty = full + S;
    uint64_t *tfull = empty + S;   // [2] accumulator ready for the epilogue
    uint64_t *tempty = tfull + 2;  // [2] accumulator drained by the epilogue (4 warp arrivals)
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(tempty + 2);
    __shared__ int s_abort;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long g0 = (long long)blockIdx.x * rp.run;
    const int nblk = (int)min((long long)rp.run, rp.nblocks - g0);
    const int kstages = p.nb * C::ELEM / R::KB;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int a = 0; a < 2; a++) {
            mbar_init(&tfull[a], 1);
            mbar_init(&tempty[a], 4);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(RUN_TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            // ---- TMA producer ----
            int it = 0;  // K stages issued over the whole run
            for (int j = 0; j < nblk && !ld_volatile(&s_abort); j++) {
                int ti, tj, mi, nj;
                block_coords(p, g0 + j, ti, tj, mi, nj);
                const int arow = ti * p.nb + mi * BM, brow = tj * p.nb + nj * BN;
                for (int kb = 0; kb < kstages; kb++, it++) {
                    const int s = it % S;
                    if (it >= S && !mbar_wait(&empty[s], ((it / S) - 1) & 1)) {
                        s_abort = 1;
                        break;
                    }
                    uint8_t *st = base + s * R::STAGE_BYTES;
                    mbar_expect_tx(&full[s], R::STAGE_BYTES);
                    const int kx = kb * R::KELEMS;
                    tma_load_2d(st, &ta, kx, arow, &full[s]);
                    tma_load_2d(st + R::A_BYTES, &tb, kx, brow, &full[s]);
                    if (C::NOPS == 2) {
                        tma_load_2d(st + R::A_BYTES + R::B_BYTES, &ta_lo, kx, arow, &full[s]);
                        tma_load_2d(st + 2 * R::A_BYTES + R::B_BYTES, &tb_lo, kx, brow, &full[s]);
                    }
                }
            }
            if (ld_volatile(&s_abort)) {
                // drain: wait (bounded) for this CTA's own copies that may still be landing
                for (int u = it - S < 0 ? 0 : it - S; u < it; u++) mbar_wait(&full[u % S], (u / S) & 1);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---- MMA issuer ----
            int it = 0;
            for (int j = 0; j < nblk; j++) {
                const int acc = j & 1;
                if (j >= 2 && !mbar_wait(&tempty[acc], ((j >> 1) - 1) & 1)) {
                    s_abort = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t td = tmem + (uint32_t)(acc * 256);
                bool ok = true;
                for (int kb = 0; kb < kstages; kb++, it++) {
                    const int s = it % S;
                    if (ld_volatile(&s_abort) || !mbar_wait(&full[s], (it / S) & 1)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    uint8_t *st = base + s * R::STAGE_BYTES;
                    const uint64_t da = smem_desc<R::KB>(st), db = smem_desc<R::KB>(st + R::A_BYTES);
#pragma unroll
                    for (int kk = 0; kk < R::KB / 32; kk++) {
                        const uint32_t accf = (kb | kk) ? 1u : 0u;
                        mma<MODE>(td, da + 2 * kk, db + 2 * kk, accf);
                        if (C::NOPS == 2) {
                            const uint64_t dal = smem_desc<R::KB>(st + R::A_BYTES + R::B_BYTES);
                            const uint64_t dbl = smem_desc<R::KB>(st + 2 * R::A_BYTES + R::B_BYTES);
                            mma<MODE>(td, da + 2 * kk, dbl + 2 * kk, 1u);   // hi * lo
                            mma<MODE>(td, dal + 2 * kk, db + 2 * kk, 1u);   // lo * hi
                        }
                    }
                    mma_commit(&empty[s]);
                }
                if (!ok) {
                    s_abort = 1;
                    break;
                }
                mma_commit(&tfull[acc]);
            }
        }
    } else {
        // ---- epilogue: warps 2..5, thread = accumulator row of its TMEM lane quarter ----
        const int lq = warp & 3;
        const int mt = p.n / p.nb;
        for (int j = 0; j < nblk; j++) {
            const int acc = j & 1;
            int ti, tj, mi, nj;
            block_coords(p, g0 + j, ti, tj, mi, nj);
            const int tr = p.k + 1 + ti, tc = p.k + 1 + tj;
            float *ct = p.C + (size_t)p.nb * p.nb * ((size_t)tr + (size_t)mt * tc) +
                        (size_t)(mi * BM + lq * 32 + lane) + (size_t)(nj * BN) * p.nb;
            float cold[64];
#pragma unroll
            for (int c = 0; c < 64; c++) cold[c] = __ldcs(ct + (size_t)c * p.nb);
            bool have = !ld_volatile(&s_abort) && mbar_wait(&tfull[acc], (j >> 1) & 1);
            if (!have) {
                if (lane == 0) atomicCAS(p.status + ST_CODE, 0, -4);
                s_abort = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            float sc = 1.0f;
            if (MODE == MODE_FP8 && p.scale_a) sc = p.scale_a[ti] * p.scale_b[tj];
            const uint32_t trow = tmem + ((uint32_t)(lq * 32) << 16) + (uint32_t)(acc * 256);
            for (int c0 = 0; c0 < BN; c0 += 64) {
                float d[64];
                tmem_ld16(trow + (uint32_t)c0, d);
                tmem_ld16(trow + (uint32_t)(c0 + 16), d + 16);
                tmem_ld16(trow + (uint32_t)(c0 + 32), d + 32);
                tmem_ld16(trow + (uint32_t)(c0 + 48), d + 48);
                if (c0 + 64 >= BN) {
                    // the accumulator is fully read: hand it back to the MMA warp
                    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&tempty[acc]);
                }
                float nxt[64];
                if (c0 + 64 < BN) {
#pragma unroll
                    for (int c = 0; c < 64; c++) nxt[c] = __ldcs(ct + (size_t)(c0 + 64 + c) * p.nb);
                }
#pragma unroll
                for (int c = 0; c < 64; c++) __stcs(ct + (size_t)(c0 + c) * p.nb, fmaf(-sc, d[c], cold[c]));
                if (c0 + 64 < BN) {
#pragma unroll
                    for (int c = 0; c < 64; c++) cold[c] = nxt[c];
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(RUN_TMEM_COLS));
}

// ---------------------------------------------------------------------------------------
// Panel packing: K-major low-precision copies of the step's panel.
// ---------------------------------------------------------------------------------------
// TF32 rounding of an FP32 value: round half away from zero to 10 explicit mantissa bits (the
// magnitude bits are rounded by adding half a TF32 unit in the last place and clearing the 13
// low bits; a carry into the exponent is the correct result).  x - tf32_round(x) is exact in
// FP32, so x = hi + lo with both parts TF32 up to the 2 lowest bits of x.
__device__ __forceinline__ float tf32_round(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

// One packed element in mode MODE (0 bf16, 2 bf16 hi + lo, 3 tf32 hi + lo; e4m3 is handled by
// the callers with its scale).
__device__ __forceinline__ void pack_one(int mode, float x, void *hi, void *lo, size_t o) {
    if (mode == 3) {
        const float h = tf32_round(x);
        static_cast<float *>(hi)[o] = h;
        static_cast<float *>(lo)[o] = tf32_round(x - h);
        return;
    }
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    static_cast<__nv_bfloat16 *>(hi)[o] = h;
    if (mode == 2) static_cast<__nv_bfloat16 *>(lo)[o] = __float2bfloat16_rn(x - __bfloat162float(h));
}

// Row panel k (Cholesky U(k, m) / LU U(k, n), m > k): packed row (m-k-1)*nb + j, col p =
// tile (k, m) element (p, j): the tile's columns are already contiguous in p.
// MODE 0: bf16; 2: bf16 hi + lo; 3: tf32 hi + lo (FP32 containers); 1: e4m3 with per-tile
// scale (max|x| / 448).
__global__ void pack_rows_kernel(const float *W, int n, int nb, int k, int mode, void *hi, void *lo,
                                 float *scales, int t0) {
    const int t = t0 + blockIdx.y;              // trailing tile index
    const int mt = n / nb;
    const float *tile = W + (size_t)nb * nb * ((size_t)k + (size_t)mt * (k + 1 + t));
    const size_t out0 = (size_t)t * nb * nb;
    float inv = 1.0f;
    if (mode == 1) {
        __shared__ float red[32];
        float mx = 0.f;
        for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) mx = fmaxf(mx, fabsf(tile[e]));
        for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
        __syncthreads();
        if (threadIdx.x == 0) {
            float m = 0.f;
            for (int i = 0; i < (int)(blockDim.x >> 5); i++) m = fmaxf(m, red[i]);
            const float s = m > 0.f ? m / 448.0f : 1.0f;
            red[0] = s;
            scales[t] = s;
        }
        __syncthreads();
        inv = 1.0f / red[0];
    }
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nb * nb; e += gridDim.x * blockDim.x) {
        const float x = tile[e];
        if (mode == 1)
            static_cast<__nv_fp8_e4m3 *>(hi)[out0 + e] = __nv_fp8_e4m3(x * inv);
        else
            pack_one(mode, x, hi, lo, out0 + e);
    }
}

// Column panel k (LU L(m, k), m > k): packed row (m-k-1)*nb + i, col p = tile (m, k)
// element (i, p): a transpose, through shared memory 32 x 32 at a time.
__global__ void pack_cols_kernel(const float *W, int n, int nb, int k, int mode, void *hi, void *lo,
                                 const float *scales, int t0) {
    __shared__ float s[32][33];
    const int t = t0 + blockIdx.z;
    const int mt = n / nb;
    const float *tile = W + (size_t)nb * nb * ((size_t)(k + 1 + t) + (size_t)mt * k);
    const int i0 = blockIdx.x * 32, p0 = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) s[r][threadIdx.x] = tile[(size_t)(i0 + threadIdx.x) + (size_t)(p0 + r) * nb];
    __syncthreads();
    const float inv = (mode == 1) ? 1.0f / scales[t] : 1.0f;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const float x = s[threadIdx.x][r];  // element (i0 + r, p0 + tx)
        const size_t o = (size_t)t * nb * nb + (size_t)(i0 + r) * nb + p0 + threadIdx.x;
        if (mode == 1)
            static_cast<__nv_fp8_e4m3 *>(hi)[o] = __nv_fp8_e4m3(x * inv);
        else
            pack_one(mode, x, hi, lo, o);
    }
}

// per-tile max-abs scales of the column panel (FP8 mode)
__global__ void col_scales_kernel(const float *W, int n, int nb, int k, float *scales, int t0) {
    __shared__ float red[32];
    const int t = t0 + blockIdx.x;
    const int mt = n / nb;
    const float *tile = W + (size_t)nb * nb * ((size_t)(k + 1 + t) + (size_t)mt * k);
    float mx = 0.f;
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) mx = fmaxf(mx, fabsf(tile[e]));
    for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        float m = 0.f;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) m = fmaxf(m, red[i]);
        scales[t] = m > 0.f ? m / 448.0f : 1.0f;
    }
}

}  // namespace mp

// ---------------------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------------------
namespace {
using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                              const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeFn g_encode = nullptr;

cudaError_t get_encode() {
    if (g_encode) return cudaSuccess;
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) return cudaErrorNotSupported;
    g_encode = reinterpret_cast<EncodeFn>(fn);
    return cudaSuccess;
}

// K-major packed operand: rows x nb elements, box = box_rows x swb bytes, swb-byte swizzle
// (128 or 64).
cudaError_t make_map(CUtensorMap *m, const void *base, long long rows, int nb, int elem_bytes, int box_rows,
                     int swb = 128) {
    cudaError_t e = get_encode();
    if (e != cudaSuccess) return e;
    const cuuint64_t dims[2] = {(cuuint64_t)nb, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)nb * elem_bytes};
    const cuuint32_t box[2] = {(cuuint32_t)(swb / elem_bytes), (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    const CUtensorMapDataType dt = elem_bytes == 1   ? CU_TENSOR_MAP_DATA_TYPE_UINT8
                                   : elem_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                                     : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    const CUresult r = g_encode(m, dt, 2,
                                const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                swb == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B,
                                CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// Which update kernel runs: 0 one output block per CTA (mp_update_kernel), 2 tile runs
// (mp_update_run_kernel) for every launch, 1 (default) tile runs for the split modes (three
// products per K slice: tensor-bound, where overlapping the epilogue with the next block's
// MMAs pays) and one block per CTA for BF16 / FP8 (HBM-bound on the C traffic, where two
// CTAs' epilogues per SM keep more loads in flight).
int g_update_kernel = 1;
// SMs the rest update (part 2) leaves free for the high-priority chain and the panel solves
// beside it: 24 of 152 measured best at N = 32768, NB = 512 (0: none held back)
int g_update_reserve = 24;
int g_update_reserve_below = 0;  // ... only for trailing matrices of fewer tile rows (0: always)

int sm_count() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 148;
    }
    return sms;
}

template <int MODE>
cudaError_t launch_mode(const void *a_hi, const void *a_lo, const void *b_hi, const void *b_lo,
                        const mp::UpdateParams &p, cudaStream_t s) {
    using C = mp::Cfg<MODE>;
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(mp::mp_update_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             C::SMEM);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(mp::mp_update_run_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 mp::RunCfg<MODE>::SMEM);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    const long long rows = (long long)p.ntr * p.nb;
    const int eb = C::ELEM;
    CUtensorMap ta, tb, tal, tbl;
    cudaError_t e;
    if ((e = make_map(&ta, a_hi, rows, p.nb, eb, mp::BM)) != cudaSuccess) return e;
    if ((e = make_map(&tb, b_hi, rows, p.nb, eb, mp::BN)) != cudaSuccess) return e;
    if (C::NOPS == 2) {
        if ((e = make_map(&tal, a_lo, rows, p.nb, eb, mp::BM)) != cudaSuccess) return e;
        if ((e = make_map(&tbl, b_lo, rows, p.nb, eb, mp::BN)) != cudaSuccess) return e;
    } else {
        tal = ta;
        tbl = tb;
    }
    const long long nt = p.ntr, ns = nt - 1;
    long long pairs = p.part == 1   ? (p.upper ? nt : 2 * nt - 1)
                      : p.part == 2 ? (p.upper ? ns * (ns + 1) / 2 : ns * ns)
                      : p.part == 4 ? 1
                      : p.part == 5 ? (p.upper ? ns : 2 * ns)
                                    : (p.upper ? nt * (nt + 1) / 2 : nt * nt);
    if (p.part == 3) {
        if (!p.upper || p.r0 < 0 || p.r1 > p.ntr) return cudaErrorInvalidValue;
        pairs = 0;
        for (int r = p.r0; r < p.r1; r++) pairs += nt - r;
    }
    const long long blocks = pairs * (p.nb / mp::BM) * (p.nb / mp::BN);
    if (blocks <= 0) return cudaSuccess;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
    // blocks per CTA of the tile-run kernel: 8 (one 512 tile pair) down to 2, keeping at least
    // two waves of CTAs over the SMs
    const long long sms = sm_count();
    int run = 8;
    while (run > 1 && blocks < sms * run * 2) run /= 2;
    if (g_update_kernel == 0 || (g_update_kernel == 1 && !C::SPLIT)) {
        note_launch();
        mp::mp_update_kernel<MODE><<<(unsigned)blocks, mp::NTHR, C::SMEM, s>>>(ta, tb, tal, tbl, p);
        return cudaGetLastError();
    }
    if (run < 2) run = 2;  // small launches too: two blocks per CTA beat one block per CTA (measured)
    // the rest update (part 2, or its row ranges while row groups arrive: part 3) with SMs held
    // back for the critical chain's kernels: at most sms - reserve CTAs, each taking a longer
    // run of consecutive blocks
    if ((p.part == 2 || p.part == 3) && g_update_reserve > 0 && g_update_reserve < sms &&
        (g_update_reserve_below <= 0 || p.ntr < g_update_reserve_below)) {
        const long long cap = sms - g_update_reserve;
        if ((blocks + run - 1) / run > cap) run = (int)((blocks + cap - 1) / cap);
    }
    constexpr int KB = mp::RunCfg<MODE>::KB;
    if ((e = make_map(&ta, a_hi, rows, p.nb, eb, mp::BM, KB)) != cudaSuccess) return e;
    if ((e = make_map(&tb, b_hi, rows, p.nb, eb, mp::BN, KB)) != cudaSuccess) return e;
    if (C::NOPS == 2) {
        if ((e = make_map(&tal, a_lo, rows, p.nb, eb, mp::BM, KB)) != cudaSuccess) return e;
        if ((e = make_map(&tbl, b_lo, rows, p.nb, eb, mp::BN, KB)) != cudaSuccess) return e;
    } else {
        tal = ta;
        tbl = tb;
    }
    mp::RunParams rp{p, blocks, run};
    note_launch();
    mp::mp_update_run_kernel<MODE><<<(unsigned)((blocks + run - 1) / run), mp::RUN_THREADS, mp::RunCfg<MODE>::SMEM, s>>>(
        ta, tb, tal, tbl, rp);
    return cudaGetLastError();
}
}  // namespace

// mode: 0 bf16, 1 fp8, 2 bf16x3, 3 tf32x3.  a_*/b_*: packed operands (ntr*nb rows x nb), scales: per
// trailing tile (fp8).  C: FP32 tile-layout matrix.
cudaError_t mp_update(int mode, int upper, float *C, int n, int nb, int k, const void *a_hi, const void *a_lo,
                      const void *b_hi, const void *b_lo, const float *scale_a, const float *scale_b, int *status,
                      cudaStream_t s, int part, int r0, int r1) {
    if (nb % 256 || n % nb) return cudaErrorInvalidValue;
    mp::UpdateParams p{};
    p.C = C;
    p.n = n;
    p.nb = nb;
    p.k = k;
    p.ntr = n / nb - k - 1;
    p.upper = upper;
    p.scale_a = scale_a;
    p.scale_b = scale_b;
    p.status = status;
    p.part = part;
    p.r0 = r0;
    p.r1 = r1;
    if (p.ntr <= 0) return cudaSuccess;
    if (mode == mp::MODE_BF16) return launch_mode<mp::MODE_BF16>(a_hi, nullptr, b_hi, nullptr, p, s);
    if (mode == mp::MODE_FP8) return launch_mode<mp::MODE_FP8>(a_hi, nullptr, b_hi, nullptr, p, s);
    if (mode == mp::MODE_TF32X3) return launch_mode<mp::MODE_TF32X3>(a_hi, a_lo, b_hi, b_lo, p, s);
    if (mode != mp::MODE_BF16X3) return cudaErrorInvalidValue;
    return launch_mode<mp::MODE_BF16X3>(a_hi, a_lo, b_hi, b_lo, p, s);
}

// Update-kernel choice (palial_gpu_set_update_kernel): returns the previous setting.
int set_update_kernel(int kind) {
    const int old = g_update_kernel;
    if (kind >= 0 && kind <= 2) g_update_kernel = kind;
    return old;
}

// SMs the rest update leaves to the critical chain (palial_gpu_set_update_reserve): returns the
// previous setting.
int set_update_reserve(int sms, int below_rows) {
    const int old = g_update_reserve;
    if (sms >= 0) g_update_reserve = sms;
    g_update_reserve_below = below_rows;
    return old;
}

// Pack the row panel k (tiles (k, m), m > k) of the FP32 tile matrix W: trailing tiles
// [t0, t0 + count) (count < 0: to the end).
cudaError_t mp_pack_rows(int mode, const float *W, int n, int nb, int k, void *hi, void *lo, float *scales,
                         cudaStream_t s, int t0, int count) {
    const int ntr = n / nb - k - 1;
    if (count < 0) count = ntr - t0;
    if (ntr <= 0 || count <= 0) return cudaSuccess;
    if (t0 < 0 || t0 + count > ntr) return cudaErrorInvalidValue;
    dim3 grid(mode == 1 ? 1 : 16, count);
    note_launch();
    mp::pack_rows_kernel<<<grid, 1024, 0, s>>>(W, n, nb, k, mode, hi, lo, scales, t0);
    return cudaGetLastError();
}

// Pack the column panel k (tiles (m, k), m > k), transposed to K-major: trailing tiles
// [t0, t0 + count) (count < 0: to the end).
cudaError_t mp_pack_cols(int mode, const float *W, int n, int nb, int k, void *hi, void *lo, float *scales,
                         cudaStream_t s, int t0, int count) {
    const int ntr = n / nb - k - 1;
    if (count < 0) count = ntr - t0;
    if (ntr <= 0 || count <= 0) return cudaSuccess;
    if (t0 < 0 || t0 + count > ntr) return cudaErrorInvalidValue;
    if (mode == 1) {
        note_launch();
        mp::col_scales_kernel<<<count, 1024, 0, s>>>(W, n, nb, k, scales, t0);
    }
    dim3 grid(nb / 32, nb / 32, count), block(32, 8);
    note_launch();
    mp::pack_cols_kernel<<<grid, block, 0, s>>>(W, n, nb, k, mode, hi, lo, scales, t0);
    return cudaGetLastError();
}

}  // namespace palial
