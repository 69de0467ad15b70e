// mp_solve.cu -- FP32/FP64 kernels of the mixed-precision factorizations and of iterative
// refinement: precision conversions, panel triangular solves (FP32 SIMT), blocked triangular
// solves of the refinement corrections with the low-precision factors, the FP64 residual
// r = b - A x on the FP64 tile-layout matrix, and the norms of the backward error.
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
__global__ void f64_to_f32_kernel(const double *a, float *w, long long len, double shift_diag, int n, int nb) {
    const int mt = n / nb;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < len; e += (long long)gridDim.x * blockDim.x) {
        double v = a[e];
        if (shift_diag != 0.0) {
            const long long t = e / ((long long)nb * nb);
            const int in = (int)(e - t * (long long)nb * nb);
            if ((t % mt) == (t / mt) && (in % nb) == (in / nb)) v += shift_diag;
        }
        w[e] = (float)v;
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

// X = U^-T B, B = nb x 64 strip (ld), U upper nb x nb (ld_u)
__device__ void strip_lut(const Smem &m, const float *U, int ldu, float *B, int ldb, int nb) {
    for (int rb = 0; rb < nb; rb += 64) {
        if (rb > 0) cta_gemm<true, false>(64, 64, rb, -1.f, U + (size_t)rb * ldu, ldu, B, ldb, B + rb, ldb, m.g);
        load_diag64(m.Ds, U + rb + (size_t)rb * ldu, ldu);
        solve64<0>(m.Ds, m.Bs, B + rb, ldb);
    }
}
// X = U^-1 B (backward), B = nb x 64 strip
__device__ void strip_un(const Smem &m, const float *U, int ldu, float *B, int ldb, int nb) {
    for (int rb = nb - 64; rb >= 0; rb -= 64) {
        if (rb + 64 < nb)
            cta_gemm<false, false>(64, 64, nb - rb - 64, -1.f, U + rb + (size_t)(rb + 64) * ldu, ldu, B + rb + 64, ldb,
                                   B + rb, ldb, m.g);
        load_diag64(m.Ds, U + rb + (size_t)rb * ldu, ldu);
        solve64<3>(m.Ds, m.Bs, B + rb, ldb);
    }
}
// X = L^-1 B (unit lower), B = nb x 64 strip
__device__ void strip_llu(const Smem &m, const float *L, int ldl, float *B, int ldb, int nb) {
    for (int rb = 0; rb < nb; rb += 64) {
        if (rb > 0) cta_gemm<false, false>(64, 64, rb, -1.f, L + rb, ldl, B, ldb, B + rb, ldb, m.g);
        load_diag64(m.Ds, L + rb + (size_t)rb * ldl, ldl);
        solve64<2>(m.Ds, m.Bs, B + rb, ldb);
    }
}
// X = B U^-1, B = 64 x nb row strip
__device__ void strip_run(const Smem &m, const float *U, int ldu, float *B, int ldb, int nb) {
    for (int cb = 0; cb < nb; cb += 64) {
        if (cb > 0)
            cta_gemm<false, false>(64, 64, cb, -1.f, B, ldb, U + (size_t)cb * ldu, ldu, B + (size_t)cb * ldb, ldb, m.g);
        load_diag64(m.Ds, U + cb + (size_t)cb * ldu, ldu);
        solve64<1>(m.Ds, m.Bs, B + (size_t)cb * ldb, ldb);
    }
}

// kind 0: Cholesky row panel U(k,m) <- U_kk^-T U(k,m);  1: LU row panel U(k,n) <- L_kk^-1 .;
// 2: LU column panel L(m,k) <- L(m,k) U_kk^-1.  grid (nb/64, trailing tiles).
__global__ void __launch_bounds__(NT, 1) panel_trsm_kernel(float *W, int n, int nb, int k, int kind) {
    extern __shared__ __align__(16) float smem[];
    const Smem m = smem_parts(smem);
    const int t = k + 1 + blockIdx.y, s = blockIdx.x;
    const float *T = W + tile_off(n, nb, k, k);
    if (kind == 0) strip_lut(m, T, nb, W + tile_off(n, nb, k, t) + (size_t)s * 64 * nb, nb, nb);
    else if (kind == 1) strip_llu(m, T, nb, W + tile_off(n, nb, k, t) + (size_t)s * 64 * nb, nb, nb);
    else strip_run(m, T, nb, W + tile_off(n, nb, t, k) + s * 64, nb, nb);
}

// ---- blocked triangular solves of the refinement right-hand sides (R: n x 64, ld n) ---------
// diag step: one CTA solves tile row k of R with the diagonal tile; kind as below.
//   0: U^T y = r (forward, Cholesky)   1: U z = y (backward)   2: L y = r (forward, unit)
__global__ void __launch_bounds__(NT, 1) rhs_diag_kernel(const float *W, int n, int nb, int k, float *R, int kind) {
    extern __shared__ __align__(16) float smem[];
    const Smem m = smem_parts(smem);
    const float *T = W + tile_off(n, nb, k, k);
    float *B = R + (size_t)k * nb;
    if (kind == 0) strip_lut(m, T, nb, const_cast<float *>(B), n, nb);
    else if (kind == 1) strip_un(m, T, nb, B, n, nb);
    else strip_llu(m, T, nb, B, n, nb);
}

// update step: for every other tile row t (blockIdx.x) in the active range:
//   kind 0: R_t -= U(k,t)^T R_k  (t > k)     kind 1: R_t -= U(t,k) R_k (t < k)
//   kind 2: R_t -= L(t,k) R_k    (t > k)
__global__ void __launch_bounds__(NT, 1) rhs_update_kernel(const float *W, int n, int nb, int k, float *R, int kind) {
    extern __shared__ __align__(16) float smem[];
    const Smem m = smem_parts(smem);
    const int t = (kind == 1) ? (int)blockIdx.x : k + 1 + (int)blockIdx.x;
    const float *Rk = R + (size_t)k * nb;
    float *Rt = R + (size_t)t * nb;
    if (kind == 0) cta_gemm<true, false>(nb, 64, nb, -1.f, W + tile_off(n, nb, k, t), nb, Rk, n, Rt, n, m.g);
    else cta_gemm<false, false>(nb, 64, nb, -1.f, W + tile_off(n, nb, t, k), nb, Rk, n, Rt, n, m.g);
}

// ---- FP64 residual R = B - A X (A: FP64 tile layout; X, B, R: n x nrhs, ld n; nrhs <= 16) ---
__global__ void __launch_bounds__(256) residual_kernel(const double *A, int n, int nb, const double *X,
                                                       const double *B, double *R, int nrhs) {
    __shared__ double As[64][65];
    __shared__ double Xs[64][17];
    const int i0 = blockIdx.x * 64;
    const int row = threadIdx.x & 63, grp = threadIdx.x >> 6;   // 4 groups x 4 right-hand sides
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const int mt = n / nb;
    for (int p0 = 0; p0 < n; p0 += 64) {
        const double *blk = A + (size_t)nb * nb * ((size_t)(i0 / nb) + (size_t)mt * (p0 / nb)) + (size_t)(i0 % nb) +
                            (size_t)(p0 % nb) * nb;
        for (int e = threadIdx.x; e < 4096; e += 256) As[e >> 6][e & 63] = blk[(e & 63) + (size_t)(e >> 6) * nb];
        for (int e = threadIdx.x; e < 64 * 16; e += 256) {
            const int r = e & 63, c = e >> 6;
            Xs[r][c] = (c < nrhs) ? X[(size_t)(p0 + r) + (size_t)c * n] : 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int p = 0; p < 64; p++) {
            const double a = As[p][row];
#pragma unroll
            for (int j = 0; j < 4; j++) acc[j] = fma(a, Xs[p][grp * 4 + j], acc[j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int c = grp * 4 + j;
        if (c < nrhs) {
            const size_t o = (size_t)(i0 + row) + (size_t)c * n;
            R[o] = B[o] - acc[j];
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

// per-column max |x| of dense n x cols (FP64), atomicMax on the bit patterns (values >= 0)
__global__ void colmax_kernel(const double *X, long long n, int cols, double *out) {
    const int c = blockIdx.y;
    double mx = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        mx = fmax(mx, fabs(X[(size_t)i + (size_t)c * n]));
    for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0)
        atomicMax(reinterpret_cast<unsigned long long *>(out + c), (unsigned long long)__double_as_longlong(mx));
}

// R32 (n x 64, zero padded) = float(R64 / scale_c) ; X64 += scale_c * D32
__global__ void to_f32_rhs_kernel(const double *R, float *R32, long long n, int cols, const double *scale) {
    const long long total = n * 64;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e / n);
        R32[e] = (c < cols) ? (float)(R[e] / scale[c]) : 0.f;
    }
}
__global__ void add_correction_kernel(double *X, const float *D32, long long n, int cols, const double *scale) {
    const long long total = n * cols;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x)
        X[e] += scale[e / n] * (double)D32[e];
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
    e = cudaFuncSetAttribute(mps::rhs_diag_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, mps::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(mps::rhs_update_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, mps::SMEM_BYTES);
}

cudaError_t mps_f64_to_f32(const double *A, float *W, int n, int nb, double shift, cudaStream_t s) {
    mps::f64_to_f32_kernel<<<4096, 256, 0, s>>>(A, W, (long long)n * n, shift, n, nb);
    return cudaGetLastError();
}
cudaError_t mps_tile_to_f64(const float *w, double *d, int nb, cudaStream_t s) {
    mps::tile_f32_to_f64_kernel<<<256, 256, 0, s>>>(w, d, nb * nb);
    return cudaGetLastError();
}
cudaError_t mps_tile_to_f32(const double *d, float *w, int nb, int upper_only, cudaStream_t s) {
    mps::tile_f64_to_f32_kernel<<<256, 256, 0, s>>>(d, w, nb, upper_only);
    return cudaGetLastError();
}
cudaError_t mps_panel_trsm(float *W, int n, int nb, int k, int kind, cudaStream_t s) {
    const int ntr = n / nb - k - 1;
    if (ntr <= 0) return cudaSuccess;
    dim3 grid(nb / 64, ntr);
    mps::panel_trsm_kernel<<<grid, mps::NT, mps::SMEM_BYTES, s>>>(W, n, nb, k, kind);
    return cudaGetLastError();
}
cudaError_t mps_rhs_diag(const float *W, int n, int nb, int k, float *R, int kind, cudaStream_t s) {
    mps::rhs_diag_kernel<<<1, mps::NT, mps::SMEM_BYTES, s>>>(W, n, nb, k, R, kind);
    return cudaGetLastError();
}
cudaError_t mps_rhs_update(const float *W, int n, int nb, int k, float *R, int kind, cudaStream_t s) {
    const int mt = n / nb;
    const int cnt = (kind == 1) ? k : mt - k - 1;
    if (cnt <= 0) return cudaSuccess;
    mps::rhs_update_kernel<<<cnt, mps::NT, mps::SMEM_BYTES, s>>>(W, n, nb, k, R, kind);
    return cudaGetLastError();
}
cudaError_t mps_residual(const double *A, int n, int nb, const double *X, const double *B, double *R, int nrhs,
                         cudaStream_t s) {
    mps::residual_kernel<<<n / 64, 256, 0, s>>>(A, n, nb, X, B, R, nrhs);
    return cudaGetLastError();
}
cudaError_t mps_norm_inf_matrix(const double *A, int n, int nb, double *out, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double), s);
    if (e != cudaSuccess) return e;
    mps::rowsum_kernel<<<n / 64, 256, 0, s>>>(A, n, nb, out);
    return cudaGetLastError();
}
cudaError_t mps_colmax(const double *X, long long n, int cols, double *out, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double) * cols, s);
    if (e != cudaSuccess) return e;
    dim3 grid(64, cols);
    mps::colmax_kernel<<<grid, 256, 0, s>>>(X, n, cols, out);
    return cudaGetLastError();
}
cudaError_t mps_to_f32_rhs(const double *R, float *R32, long long n, int cols, const double *scale, cudaStream_t s) {
    mps::to_f32_rhs_kernel<<<2048, 256, 0, s>>>(R, R32, n, cols, scale);
    return cudaGetLastError();
}
cudaError_t mps_mark_step(int *status, int k, cudaStream_t s) {
    mps::mark_step_kernel<<<1, 1, 0, s>>>(status, k);
    return cudaGetLastError();
}
cudaError_t mps_add_correction(double *X, const float *D32, long long n, int cols, const double *scale,
                               cudaStream_t s) {
    mps::add_correction_kernel<<<2048, 256, 0, s>>>(X, D32, n, cols, scale);
    return cudaGetLastError();
}

}  // namespace palial
