// gen_check.cu -- seeded input generators and normwise residual probes on device buffers.
//
// Generators are counter-based: entry (i, j) of an n x cols matrix is a function of
// (seed, stream, i + j*n) only (splitmix64), so any thread layout -- and the CPU oracle's
// numpy generator -- yields the same bytes.  The SPD generator A = B B^T + n I uses
// B = K / 128 with K integer in [-128, 127]: K K^T is computed exactly in int32 (dp4a), so
// the device and the CPU produce identical matrices.
#include <cstdint>

#include "common.cuh"

namespace palial {

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ uint64_t stream_key(uint64_t seed, uint64_t stream) {
    return mix64(seed * 0xD1B54A32D192ED03ull + stream);
}
__device__ __forceinline__ double uniform_pm1(uint64_t r) {
    return (double)(r >> 11) * 0x1.0p-52 - 1.0;
}

enum { STREAM_UNIFORM = 0, STREAM_SPD = 1, STREAM_RHS = 2, STREAM_HOUSE = 3 };

// Tile-layout uniform matrix.  One thread per element, consecutive threads walk rows of a
// tile column (coalesced writes).
__global__ void gen_uniform_kernel(double *A, int n, int nb, uint64_t key) {
    const long long total = (long long)n * n;
    const int mt = n / nb;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        // e indexes the tile-layout buffer: tile t = e / nb^2, inside r + c*nb
        const long long t = e / ((long long)nb * nb);
        const int in = (int)(e - t * (long long)nb * nb);
        const int r = in % nb, c = in / nb;
        const int tm = (int)(t % mt), tn = (int)(t / mt);
        const long long i = (long long)tm * nb + r, j = (long long)tn * nb + c;
        A[e] = uniform_pm1(mix64(key + (uint64_t)(i + j * n)));
    }
}

// The reference generator's pattern (reference include/populate.h:36-67) with a seeded
// diagonal: 0.5 everywhere, diagonal 173 * u + 173 with u = (x_i + 1) / 2, x_i the uniform
// [-1, 1) number of index i.  Explicit _rn operations keep the bytes equal to numpy's.
__global__ void gen_refpattern_kernel(double *A, int n, int nb, uint64_t key) {
    const long long total = (long long)n * n;
    const int mt = n / nb;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long t = e / ((long long)nb * nb);
        const int in = (int)(e - t * (long long)nb * nb);
        const int r = in % nb, c = in / nb;
        const long long i = (long long)(t % mt) * nb + r, j = (long long)(t / mt) * nb + c;
        double v = 0.5;
        if (i == j) {
            const double u = __dmul_rn(__dadd_rn(uniform_pm1(mix64(key + (uint64_t)i)), 1.0), 0.5);
            v = __dadd_rn(__dmul_rn(173.0, u), 173.0);
        }
        A[e] = v;
    }
}

// Dense column-major n x cols uniform block (right-hand sides, probe vectors).
__global__ void gen_uniform_dense_kernel(double *X, long long rows, int cols, uint64_t key) {
    const long long total = rows * cols;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x)
        X[e] = uniform_pm1(mix64(key + (uint64_t)e));
}

// K (int8, row-major [i][p]) for the SPD generator: K(i,p) from index i + p*n.
__global__ void gen_k8_kernel(int8_t *K, int n, uint64_t key) {
    const long long total = (long long)n * n;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long i = e / n, p = e - i * n;
        K[e] = (int8_t)((int)(mix64(key + (uint64_t)(i + p * n)) >> 56) - 128);
    }
}

// A(i,j) = (K K^T)(i,j) * 2^-14 + n*[i==j], 128x128 output tile per CTA (256 threads, 8x8
// each), K chunk of 64 bytes staged in shared memory as packed int32 words.
__global__ void __launch_bounds__(256) spd_from_k8_kernel(const int8_t *K, double *A, int n, int nb, double diag) {
    __shared__ int As[16][128 + 4];
    __shared__ int Bs[16][128 + 4];
    const int i0 = blockIdx.y * 128, j0 = blockIdx.x * 128;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    int acc[8][8];
#pragma unroll
    for (int a = 0; a < 8; a++)
#pragma unroll
        for (int b = 0; b < 8; b++) acc[a][b] = 0;
    const int *K32 = reinterpret_cast<const int *>(K);
    const int nw = n / 4;  // words per row
    for (int p0 = 0; p0 < nw; p0 += 16) {
        // 128 rows x 16 words for each operand: 2048 words, 8 per thread
        for (int e = threadIdx.x; e < 2048; e += 256) {
            const int r = e >> 4, q = e & 15;
            As[q][r] = (i0 + r < n) ? K32[(size_t)(i0 + r) * nw + p0 + q] : 0;
            Bs[q][r] = (j0 + r < n) ? K32[(size_t)(j0 + r) * nw + p0 + q] : 0;
        }
        __syncthreads();
#pragma unroll 4
        for (int q = 0; q < 16; q++) {
            int av[8], bv[8];
#pragma unroll
            for (int a = 0; a < 8; a++) av[a] = As[q][ty + 16 * a];
#pragma unroll
            for (int b = 0; b < 8; b++) bv[b] = Bs[q][tx + 16 * b];
#pragma unroll
            for (int a = 0; a < 8; a++)
#pragma unroll
                for (int b = 0; b < 8; b++) acc[a][b] = __dp4a(av[a], bv[b], acc[a][b]);
        }
        __syncthreads();
    }
    const int mt = n / nb;
#pragma unroll
    for (int a = 0; a < 8; a++)
#pragma unroll
        for (int b = 0; b < 8; b++) {
            const int i = i0 + ty + 16 * a, j = j0 + tx + 16 * b;
            if (i >= n || j >= n) continue;
            double v = (double)acc[a][b] * 0x1.0p-14;
            if (i == j) v += diag;
            const size_t off = (size_t)nb * nb * ((size_t)(i / nb) + (size_t)mt * (j / nb)) + (size_t)(i % nb) +
                               (size_t)(j % nb) * nb;
            A[off] = v;
        }
}

// One matrix of a batch, n_true x n_true embedded in an n_pad x n_pad tile-layout buffer:
//   kind 0 (LU): uniform [-1, 1) from index i + j*n_true, identity padding;
//   kind 1 (Cholesky): A = K K^T / 2^14 + n_true I, K int8 (index i + p*n_true), computed
//   exactly per element, padding n_true * I (block diagonal: the leading factor is exact).
__global__ void gen_batch_uniform_kernel(double *A, int nt, int np, int nb, uint64_t key) {
    const long long total = (long long)np * np;
    const int mt = np / nb;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const long long t = e / ((long long)nb * nb);
        const int in = (int)(e - t * (long long)nb * nb);
        const long long i = (t % mt) * nb + in % nb, j = (t / mt) * nb + in / nb;
        A[e] = (i < nt && j < nt) ? uniform_pm1(mix64(key + (uint64_t)(i + j * nt))) : (i == j ? 1.0 : 0.0);
    }
}
// K of a batched SPD matrix: np x np row-major int8, zero outside the leading nt x nt block
__global__ void gen_batch_k8_kernel(int8_t *K, int nt, int np, uint64_t key) {
    const long long total = (long long)np * np;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const long long i = e / np, p = e - i * np;
        K[e] = (i < nt && p < nt) ? (int8_t)((int)(mix64(key + (uint64_t)(i + p * nt)) >> 56) - 128) : (int8_t)0;
    }
}

// ---------------------------------------------------------------------------------------
// Y = op(tri(A)) X for a tile-layout A and dense column-major X, Y (n x r, r <= 64).
// mode: 0 full, 1 upper (incl. diagonal), 2 unit lower (strict lower + unit diagonal).
// trans: use A^T.  One CTA per 64-row block of Y, FP64.
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) tiled_mm_kernel(const double *A, const double *X, double *Y, int n,
                                                       int nb, int r, int mode, int trans) {
    __shared__ double Xs[64][65];
    __shared__ double As[64][65];
    const int i0 = blockIdx.x * 64;
    const int t = threadIdx.x;
    const int col = t & 63;        // Y column handled (r <= 64)
    const int rg = t >> 6;         // 4 row groups of 16 rows
    double acc[16];
#pragma unroll
    for (int a = 0; a < 16; a++) acc[a] = 0.0;
    const int mt = n / nb;
    for (int p0 = 0; p0 < n; p0 += 64) {
        // skip blocks that the triangle zeroes
        if (mode == 1) {
            if (!trans && p0 + 63 < i0) continue;  // A(i,p) nonzero for p >= i
            if (trans && p0 > i0 + 63) continue;   // A(p,i) nonzero for p <= i
        } else if (mode == 2) {
            if (!trans && p0 > i0 + 63) continue;  // L(i,p) for p <= i
            if (trans && p0 + 63 < i0) continue;   // L(p,i) for p >= i
        }
        for (int e = t; e < 64 * 64; e += 256) {
            const int rr = e & 63, cc = e >> 6;
            // As[cc][rr] = op(A)(i0+rr, p0+cc)
            const int gi = trans ? p0 + cc : i0 + rr;
            const int gj = trans ? i0 + rr : p0 + cc;
            double v = A[(size_t)nb * nb * ((size_t)(gi / nb) + (size_t)mt * (gj / nb)) + (size_t)(gi % nb) +
                         (size_t)(gj % nb) * nb];
            if (mode == 1 && gi > gj) v = 0.0;
            if (mode == 2) v = (gi < gj) ? 0.0 : (gi == gj ? 1.0 : v);
            As[cc][rr] = v;
            Xs[cc][rr] = (cc < r) ? X[(size_t)(p0 + rr) + (size_t)cc * n] : 0.0;
        }
        __syncthreads();
        if (col < r) {
            for (int p = 0; p < 64; p++) {
                const double x = Xs[col][p];
#pragma unroll
                for (int a = 0; a < 16; a++) acc[a] = fma(As[p][rg * 16 + a], x, acc[a]);
            }
        }
        __syncthreads();
    }
    if (col < r) {
#pragma unroll
        for (int a = 0; a < 16; a++) Y[(size_t)(i0 + rg * 16 + a) + (size_t)col * n] = acc[a];
    }
}

// sum of squares of a dense array (partials per block, finished on the host)
__global__ void sumsq_kernel(const double *X, long long len, double *partial) {
    __shared__ double red[8];
    double s = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < len; e += (long long)gridDim.x * blockDim.x)
        s = fma(X[e], X[e], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < (int)(blockDim.x / 32); i++) t += red[i];
        partial[blockIdx.x] = t;
    }
}

__global__ void sub_kernel(const double *X, const double *Y, double *Z, long long len) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < len; e += (long long)gridDim.x * blockDim.x)
        Z[e] = X[e] - Y[e];
}

// ---------------------------------------------------------------------------------------
// host wrappers
// ---------------------------------------------------------------------------------------
cudaError_t launch_gen_uniform(double *A, int n, int nb, uint64_t seed, cudaStream_t s) {
    note_launch();
    gen_uniform_kernel<<<4096, 256, 0, s>>>(A, n, nb, stream_key(seed, STREAM_UNIFORM));
    return cudaGetLastError();
}

cudaError_t launch_gen_refpattern(double *A, int n, int nb, uint64_t seed, cudaStream_t s) {
    note_launch();
    gen_refpattern_kernel<<<4096, 256, 0, s>>>(A, n, nb, stream_key(seed, STREAM_UNIFORM));
    return cudaGetLastError();
}

cudaError_t launch_gen_dense(double *X, long long rows, int cols, uint64_t seed, int stream, cudaStream_t s) {
    note_launch();
    gen_uniform_dense_kernel<<<2048, 256, 0, s>>>(X, rows, cols, stream_key(seed, (uint64_t)stream));
    return cudaGetLastError();
}

cudaError_t launch_gen_spd(double *A, int n, int nb, uint64_t seed, int8_t *kbuf, cudaStream_t s) {
    note_launch();
    gen_k8_kernel<<<4096, 256, 0, s>>>(kbuf, n, stream_key(seed, STREAM_SPD));
    dim3 grid((n + 127) / 128, (n + 127) / 128);  // n % 64 == 0 (checked by the caller)
    note_launch();
    spd_from_k8_kernel<<<grid, 256, 0, s>>>(kbuf, A, n, nb, (double)n);
    return cudaGetLastError();
}

cudaError_t launch_gen_batch(double *A, int kind, int nt, int np, int nb, uint64_t seed, int8_t *kbuf,
                             cudaStream_t s) {
    if (kind == 0) {
        note_launch();
        gen_batch_uniform_kernel<<<1024, 256, 0, s>>>(A, nt, np, nb, stream_key(seed, STREAM_UNIFORM));
        return cudaGetLastError();
    }
    note_launch();
    gen_batch_k8_kernel<<<1024, 256, 0, s>>>(kbuf, nt, np, stream_key(seed, STREAM_SPD));
    dim3 grid((np + 127) / 128, (np + 127) / 128);
    note_launch();
    spd_from_k8_kernel<<<grid, 256, 0, s>>>(kbuf, A, np, nb, (double)nt);
    return cudaGetLastError();
}

cudaError_t launch_tiled_mm(const double *A, const double *X, double *Y, int n, int nb, int r, int mode, int trans,
                            cudaStream_t s) {
    note_launch();
    tiled_mm_kernel<<<n / 64, 256, 0, s>>>(A, X, Y, n, nb, r, mode, trans);
    return cudaGetLastError();
}

cudaError_t launch_sumsq(const double *X, long long len, double *partial, int blocks, cudaStream_t s) {
    note_launch();
    sumsq_kernel<<<blocks, 256, 0, s>>>(X, len, partial);
    return cudaGetLastError();
}

cudaError_t launch_sub(const double *X, const double *Y, double *Z, long long len, cudaStream_t s) {
    note_launch();
    sub_kernel<<<1024, 256, 0, s>>>(X, Y, Z, len);
    return cudaGetLastError();
}

}  // namespace palial
