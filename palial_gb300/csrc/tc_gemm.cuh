// tc_gemm.cuh -- the tensor-core form of the FP32 CTA GEMMs (tile_f32.cuh, tile_qr.cuh): a staged
// K chunk of 32 multiplied on the warp tensor cores with BF16x3 operands (x = hi + lo in BF16,
// hi*hi + hi*lo + lo*hi accumulated in FP32, about 2^-16 per product), for the batched
// factorizations' "BF16-update" form and the FP32 QR's UNMQR / TSMQR.  The 256 threads of the
// CTA are 8 warps; warp w computes rows 16 (w % 4) .. + 15 and columns 32 (w / 4) .. + 31 of the
// 64 x 64 output block as four m16n8k16 tiles.  The operands are the staged chunks the SIMT
// GEMMs use: As[p][i] = op(A)(i, p) and Bs[p][j] = op(B)(p, j), p < 32, pitch SP (reads
// As[k][row] by lanes (g, t) fall in 32 distinct banks for SP = 68).
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

namespace palial {
namespace tcg {

struct Frag {
    float acc[4][4];  // [n8 tile][m16n8 accumulator register]
};

__device__ __forceinline__ void zero(Frag &f) {
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) f.acc[a][b] = 0.f;
}

__device__ __forceinline__ void split2(float x0, float x1, uint32_t &hi, uint32_t &lo) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);  // .x (low half) = x0
    const __nv_bfloat162 l = __floats2bfloat162_rn(x0 - __low2float(h), x1 - __high2float(h));
    hi = *reinterpret_cast<const uint32_t *>(&h);
    lo = *reinterpret_cast<const uint32_t *>(&l);
}

__device__ __forceinline__ void mma16816(float *d, const uint32_t *a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// acc += op(A)[rows] op(B)[cols] over one staged chunk of KC = 32.
template <int SP>
__device__ __forceinline__ void bf16x3_chunk(const float *As, const float *Bs, Frag &f) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int m0 = (warp & 3) * 16, n0 = (warp >> 2) * 32;
#pragma unroll
    for (int ks = 0; ks < 32; ks += 16) {
        const float *a0 = As + (ks + 2 * t) * SP + m0 + g;   // (row g, k 2t), next k one row below
        uint32_t ah[4], al[4];
        split2(a0[0], a0[SP], ah[0], al[0]);                   // row g,     k 2t, 2t+1
        split2(a0[8], a0[SP + 8], ah[1], al[1]);               // row g + 8
        split2(a0[8 * SP], a0[9 * SP], ah[2], al[2]);          // row g,     k 2t+8, 2t+9
        split2(a0[8 * SP + 8], a0[9 * SP + 8], ah[3], al[3]);  // row g + 8
#pragma unroll
        for (int nt = 0; nt < 4; nt++) {
            const float *b0 = Bs + (ks + 2 * t) * SP + n0 + nt * 8 + g;
            uint32_t bh0, bl0, bh1, bl1;
            split2(b0[0], b0[SP], bh0, bl0);            // k 2t, 2t+1, column g
            split2(b0[8 * SP], b0[9 * SP], bh1, bl1);   // k 2t+8, 2t+9
            mma16816(f.acc[nt], ah, bh0, bh1);
            mma16816(f.acc[nt], ah, bl0, bl1);
            mma16816(f.acc[nt], al, bh0, bh1);
        }
    }
}

// Output coordinates (within the 64 x 64 block) of accumulator register e of n8 tile nt.
__device__ __forceinline__ void frag_coord(int nt, int e, int &r, int &c) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    r = (warp & 3) * 16 + (lane >> 2) + (e >> 1) * 8;
    c = (warp >> 2) * 32 + nt * 8 + 2 * (lane & 3) + (e & 1);
}

}  // namespace tcg
}  // namespace palial
