// rbt.cu -- random butterfly transformation (opt-in stabilised LU without pivoting).
//
// Published method: D. S. Parker, "Random butterfly transformations with applications in
// computational linear algebra" (UCLA CSD-950023, 1995), and M. Baboulin, J. Dongarra,
// J. Herrmann, S. Tomov, "Accelerating linear system solutions using randomization
// techniques" (ACM TOMS 39(2), 2013).  A butterfly of size m is
//     B = (1/sqrt 2) [[R0, R1], [R0, -R1]],   R0, R1 diagonal with entries exp(r / 10),
// r uniform in [-1/2, 1/2]; a depth-2 recursive butterfly is W = diag(B', B'') * B with two
// half-size butterflies.  No-pivot LU is applied to Ar = U^T A V (U, V independent depth-2
// butterflies), which removes the need for pivoting with high probability; A x = b is then
// Ar y = U^T b, x = V y.  The refinement keeps the original A for its residuals and uses
// z = V (L_r U_r)^-1 U^T r as the preconditioner.
//
// Index groups: for i < n/4 the four indices {i, i + n/4, i + n/2, i + 3n/4} mix only among
// themselves.  Random vectors per transform (2n doubles): a0, a1 (level 1, n/2 each) and
// b0[h], b1[h] (level 2, half h, n/4 each).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <vector>

#include "host_state.hpp"
#include "rbt.cuh"

namespace palial {
namespace {

using rbt::Rand;
using rbt::rand_view;
using rbt::w4;
using rbt::wt4;

__device__ __forceinline__ size_t toff(int n, int nb, int r, int c) {
    return (size_t)nb * nb * ((size_t)(r / nb) + (size_t)(n / nb) * (c / nb)) + (size_t)(r % nb) + (size_t)(c % nb) * nb;
}

// W = float(U^T A): every column of the FP64 tile matrix A transformed by U^T; amax (optional,
// zeroed) receives max |a_ij| of A (bit patterns, as in the plain conversion).
__global__ void rbt_left_kernel(const double *__restrict__ A, float *__restrict__ W, int n, int nb, Rand U,
                                double *amax) {
    const int q = n / 4;
    const long long total = (long long)q * n;
    unsigned long long mx = 0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % q), c = (int)(e / q);  // consecutive threads: consecutive rows
        double v[4];
#pragma unroll
        for (int g = 0; g < 4; g++) {
            v[g] = A[toff(n, nb, i + g * q, c)];
            const unsigned long long ab = (unsigned long long)__double_as_longlong(v[g]) & 0x7FFFFFFFFFFFFFFFull;
            mx = ab > mx ? ab : mx;
        }
        float x0 = (float)v[0], x1 = (float)v[1], x2 = (float)v[2], x3 = (float)v[3];
        wt4(U, i, q, x0, x1, x2, x3);
        W[toff(n, nb, i, c)] = x0;
        W[toff(n, nb, i + q, c)] = x1;
        W[toff(n, nb, i + 2 * q, c)] = x2;
        W[toff(n, nb, i + 3 * q, c)] = x3;
    }
    if (amax) {
        for (int o = 16; o; o >>= 1) {
            const unsigned long long y = __shfl_xor_sync(0xffffffffu, mx, o);
            mx = y > mx ? y : mx;
        }
        if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<unsigned long long *>(amax), mx);
    }
}

// W <- W V in place: every row of W transformed by V^T (as a row vector, W V = (V^T W^T)^T).
__global__ void rbt_right_kernel(float *__restrict__ W, int n, int nb, Rand V) {
    const int q = n / 4;
    const long long total = (long long)q * n;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(e % n), j = (int)(e / n);  // consecutive threads: consecutive rows
        float x0 = W[toff(n, nb, r, j)], x1 = W[toff(n, nb, r, j + q)];
        float x2 = W[toff(n, nb, r, j + 2 * q)], x3 = W[toff(n, nb, r, j + 3 * q)];
        wt4(V, j, q, x0, x1, x2, x3);
        W[toff(n, nb, r, j)] = x0;
        W[toff(n, nb, r, j + q)] = x1;
        W[toff(n, nb, r, j + 2 * q)] = x2;
        W[toff(n, nb, r, j + 3 * q)] = x3;
    }
}

// right-hand sides (n x cols, ld n, FP32): trans ? W^T X : W X
__global__ void rbt_vec_kernel(float *__restrict__ X, int n, int cols, Rand R, int trans) {
    const int q = n / 4;
    const long long total = (long long)q * cols;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % q), c = (int)(e / q);
        float *x = X + (size_t)c * n;
        float x0 = x[i], x1 = x[i + q], x2 = x[i + 2 * q], x3 = x[i + 3 * q];
        if (trans) wt4(R, i, q, x0, x1, x2, x3);
        else w4(R, i, q, x0, x1, x2, x3);
        x[i] = x0;
        x[i + q] = x1;
        x[i + 2 * q] = x2;
        x[i + 3 * q] = x3;
    }
}

DevBuf g_rand;  // U randoms (2n floats) then V randoms (2n floats)
int g_rand_n = 0;
uint64_t g_rand_seed = ~0ull;

uint64_t mix(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int grid_for(long long elems) {
    const long long b = (elems + 255) / 256;
    return (int)std::max(1LL, std::min<long long>(b, (long long)std::max(1, g.sms) * 16));
}

}  // namespace

// The 4n randoms of size n from seed: exp(r / 10), r uniform [-1/2, 1/2) (splitmix64).
void rbt_randoms(int n, uint64_t seed, float *h) {
    const uint64_t key = mix(seed * 0xD1B54A32D192ED03ull + 11ull);
    for (size_t i = 0; i < (size_t)4 * n; i++) {
        const double u = (double)(mix(key + i) >> 11) * 0x1.0p-53 - 0.5;  // uniform [-1/2, 1/2)
        h[i] = (float)std::exp(u / 10.0);
    }
}

// The randoms for size n from seed (host generated; cached).
cudaError_t rbt_prepare(int n, uint64_t seed) {
    if (n % 4) return cudaErrorInvalidValue;
    if (g_rand_n == n && g_rand_seed == seed && g_rand.ptr) return cudaSuccess;
    std::vector<float> h((size_t)4 * n);
    rbt_randoms(n, seed, h.data());
    cudaError_t e = g_rand.ensure(sizeof(float) * h.size());
    if (e != cudaSuccess) return e;
    e = cudaMemcpy(g_rand.ptr, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    g_rand_n = n;
    g_rand_seed = seed;
    return cudaSuccess;
}

void rbt_release() {
    g_rand.release();
    g_rand_n = 0;
}

// W = float(U^T A V) with the randoms at rnd (4n floats).
cudaError_t rbt_transform_matrix_with(const double *A, float *W, int n, int nb, const float *rnd, cudaStream_t s) {
    if (n % 4 || n % nb) return cudaErrorInvalidValue;
    note_launch();
    rbt_left_kernel<<<grid_for((long long)n / 4 * n), 256, 0, s>>>(A, W, n, nb, rand_view(rnd, n), nullptr);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    note_launch();
    rbt_right_kernel<<<grid_for((long long)n / 4 * n), 256, 0, s>>>(W, n, nb, rand_view(rnd + 2 * n, n));
    return cudaGetLastError();
}

// W = float(U^T A V) (tile layout), amax of A as for the plain conversion.
cudaError_t rbt_transform_matrix(const double *A, float *W, int n, int nb, double *amax, cudaStream_t s) {
    const float *base = g_rand.as<float>();
    note_launch();
    rbt_left_kernel<<<grid_for((long long)n / 4 * n), 256, 0, s>>>(A, W, n, nb, rand_view(base, n), amax);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    note_launch();
    rbt_right_kernel<<<grid_for((long long)n / 4 * n), 256, 0, s>>>(W, n, nb, rand_view(base + 2 * n, n));
    return cudaGetLastError();
}

// Right-hand sides (n x cols, ld n, FP32): which = 0: X <- U^T X; 1: X <- V X.
cudaError_t rbt_transform_vectors(float *X, int n, int cols, int which, cudaStream_t s) {
    const float *base = g_rand.as<float>();
    note_launch();
    rbt_vec_kernel<<<grid_for((long long)n / 4 * cols), 256, 0, s>>>(X, n, cols,
                                                                    rand_view(base + (which ? 2 * n : 0), n), which ? 0 : 1);
    return cudaGetLastError();
}

}  // namespace palial
