// rbt.cuh -- depth-2 random butterflies (Parker 1995, see rbt.cu): the per-group transforms
// shared by the single-matrix path (rbt.cu) and the batched solves (batch_solve.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace palial {
namespace rbt {

constexpr float kInvSqrt2f = 0.70710678118654752f;

struct Rand {  // device pointers into one transform's 2n randoms
    const float *a0, *a1, *b0, *b1;  // b0, b1: [2][n/4]
};
__host__ __device__ inline Rand rand_view(const float *base, int n) {
    Rand r;
    r.a0 = base;
    r.a1 = base + n / 2;
    r.b0 = base + n;
    r.b1 = base + n + n / 2;
    return r;
}

// W^T applied to the group {i, i + q, i + 2q, i + 3q}, q = n / 4 (level 2, then level 1)
__device__ __forceinline__ void wt4(const Rand &R, int i, int q, float &x0, float &x1, float &x2, float &x3) {
    const float y0 = R.b0[i] * (x0 + x1) * kInvSqrt2f, y1 = R.b1[i] * (x0 - x1) * kInvSqrt2f;
    const float y2 = R.b0[q + i] * (x2 + x3) * kInvSqrt2f, y3 = R.b1[q + i] * (x2 - x3) * kInvSqrt2f;
    x0 = R.a0[i] * (y0 + y2) * kInvSqrt2f;
    x2 = R.a1[i] * (y0 - y2) * kInvSqrt2f;
    x1 = R.a0[q + i] * (y1 + y3) * kInvSqrt2f;
    x3 = R.a1[q + i] * (y1 - y3) * kInvSqrt2f;
}
// W applied to the group (level 1, then level 2)
__device__ __forceinline__ void w4(const Rand &R, int i, int q, float &x0, float &x1, float &x2, float &x3) {
    const float y0 = (R.a0[i] * x0 + R.a1[i] * x2) * kInvSqrt2f, y2 = (R.a0[i] * x0 - R.a1[i] * x2) * kInvSqrt2f;
    const float y1 = (R.a0[q + i] * x1 + R.a1[q + i] * x3) * kInvSqrt2f;
    const float y3 = (R.a0[q + i] * x1 - R.a1[q + i] * x3) * kInvSqrt2f;
    x0 = (R.b0[i] * y0 + R.b1[i] * y1) * kInvSqrt2f;
    x1 = (R.b0[i] * y0 - R.b1[i] * y1) * kInvSqrt2f;
    x2 = (R.b0[q + i] * y2 + R.b1[q + i] * y3) * kInvSqrt2f;
    x3 = (R.b0[q + i] * y2 - R.b1[q + i] * y3) * kInvSqrt2f;
}

}  // namespace rbt

// The 4n randoms of size n for seed (U's 2n, then V's 2n; host, splitmix64 counter-based).
void rbt_randoms(int n, uint64_t seed, float *h);
// W = float(U^T A V) (tile layout, tile nb) with the 4n randoms at rnd (device).
cudaError_t rbt_transform_matrix_with(const double *A, float *W, int n, int nb, const float *rnd, cudaStream_t s);

}  // namespace palial
