// layout.cu -- bridges between LAPACK column-major matrices and the reference's tile layout
// (reference include/tile_address.h:9-17), padding for any N, the column-major solve front end,
// and the tiled-matrix file format.
//
// Padding: a column-major n x n matrix goes into an npad x npad tile matrix (npad the next
// multiple of nb, at least n); the padding is zero except its diagonal, which holds `pad_diag`
// (1 for LU, for Cholesky a value comparable to the matrix' diagonal).  The leading n x n block
// of the factors of the padded matrix is then the factor of the original one, and a solve with
// zero-padded right-hand sides returns the original solution in its first n rows.
//
// File format (little-endian): 8-byte magic "PALTILE1", int64 n, int64 nb, int64 flags (0),
// then the n*n doubles of the tile layout in memory order (tile (m, k) at element
// nb*nb*(m + (n/nb)*k), column-major inside a tile).
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstring>

#include "host_state.hpp"

namespace palial {
namespace {

__global__ void col_to_tiles_kernel(const double *__restrict__ C, long long ldc, int n, double *__restrict__ T,
                                    int npad, int nb, double pad_diag) {
    const long long total = (long long)npad * npad;
    const int mt = npad / nb;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        // e walks the tile layout in memory order: coalesced writes
        const long long tile = e / ((long long)nb * nb);
        const int in = (int)(e - tile * (long long)nb * nb);
        const int tm = (int)(tile % mt), tk = (int)(tile / mt);
        const int r = tm * nb + in % nb, c = tk * nb + in / nb;
        double v;
        if (r < n && c < n) v = C[(size_t)r + (size_t)c * ldc];
        else v = (r == c) ? pad_diag : 0.0;
        T[e] = v;
    }
}

__global__ void tiles_to_col_kernel(const double *__restrict__ T, int npad, int nb, double *__restrict__ C,
                                    long long ldc, int n) {
    const long long total = (long long)n * n;
    const int mt = npad / nb;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        // e walks the column-major output: coalesced writes
        const int r = (int)(e % n), c = (int)(e / n);
        const int tm = r / nb, tk = c / nb;
        C[(size_t)r + (size_t)c * ldc] =
            T[(size_t)nb * nb * ((size_t)tm + (size_t)mt * tk) + (size_t)(r % nb) + (size_t)(c % nb) * nb];
    }
}

// rows [0, n) of each of nrhs columns copied between leading dimensions, zero rows [n, npad)
__global__ void copy_cols_kernel(const double *__restrict__ S, long long lds, int nrows_src, double *__restrict__ D,
                                 long long ldd, int nrows_dst, int nrhs) {
    const long long total = (long long)nrows_dst * nrhs;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(e % nrows_dst), c = (int)(e / nrows_dst);
        D[(size_t)r + (size_t)c * ldd] = r < nrows_src ? S[(size_t)r + (size_t)c * lds] : 0.0;
    }
}

int grid_of(long long elems) {
    const long long b = (elems + 255) / 256;
    return (int)std::max(1LL, std::min<long long>(b, (long long)std::max(1, g.sms) * 16));
}

DevBuf lay_a, lay_b, lay_x;

}  // namespace

void layout_release() {
    lay_a.release();
    lay_b.release();
    lay_x.release();
}

}  // namespace palial

using namespace palial;

extern "C" {

int palial_gpu_padded_size(int n, int nb) { return (n <= 0 || nb <= 0) ? 0 : ((n + nb - 1) / nb) * nb; }

int palial_gpu_colmajor_to_tiles(const double *dC, long long ldc, int n, double *dT, int npad, int nb,
                                 double pad_diag, void *stream) {
    if (!dC || !dT || n <= 0 || nb <= 0 || npad < n || npad % nb || ldc < n) return PALIAL_ERR_ARG;
    palial_status st0;
    int rc = ensure_init(&st0);
    if (rc) return rc;
    note_launch();
    col_to_tiles_kernel<<<grid_of((long long)npad * npad), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        dC, ldc, n, dT, npad, nb, pad_diag);
    return cudaGetLastError() == cudaSuccess ? PALIAL_OK : PALIAL_ERR_CUDA;
}

int palial_gpu_tiles_to_colmajor(const double *dT, int npad, int nb, double *dC, long long ldc, int n, void *stream) {
    if (!dC || !dT || n <= 0 || nb <= 0 || npad < n || npad % nb || ldc < n) return PALIAL_ERR_ARG;
    palial_status st0;
    int rc = ensure_init(&st0);
    if (rc) return rc;
    note_launch();
    tiles_to_col_kernel<<<grid_of((long long)n * n), 256, 0, static_cast<cudaStream_t>(stream)>>>(dT, npad, nb, dC,
                                                                                                   ldc, n);
    return cudaGetLastError() == cudaSuccess ? PALIAL_OK : PALIAL_ERR_CUDA;
}

// A X = B for a column-major n x n A of ANY n (device): padded to the next multiple of nb in
// the tile layout (identity padding for LU, max|a_ii|-scaled identity for Cholesky), solved by
// palial_gpu_solve_ir (mixed precision + refinement, or FP64 by opts), X = the first n rows.
int palial_gpu_solve_colmajor(int alg, int n, const double *dA, long long lda, const double *dB, long long ldb,
                              double *dX, long long ldx, int nrhs, int nb, const palial_opts *opts, palial_status *st,
                              void *stream) {
    if (st) memset(st, 0, sizeof *st);
    if ((alg != 0 && alg != 1) || n <= 0 || !dA || !dB || !dX || lda < n || ldb < n || ldx < n || nrhs < 1 ||
        nrhs > 16 || nb <= 0 || nb % 256)
        return set_status(st, PALIAL_ERR_ARG, "solve_colmajor: Cholesky/LU, NB a multiple of 256, 1 <= nrhs <= 16");
    int rc = ensure_init(st);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int npad = palial_gpu_padded_size(n, nb);
    PALIAL_CK(lay_a.ensure(sizeof(double) * (size_t)npad * npad), "alloc padded A");
    PALIAL_CK(lay_b.ensure(sizeof(double) * (size_t)npad * nrhs), "alloc padded B");
    PALIAL_CK(lay_x.ensure(sizeof(double) * (size_t)npad * nrhs), "alloc padded X");
    double pad = 1.0;
    if (alg == 0 && npad > n) {
        // Cholesky padding: a diagonal value of the matrix' own scale keeps the padded matrix'
        // norm and the refinement's scaling unchanged (the padded block is factored exactly)
        double dg = 0.0;
        PALIAL_CK(cudaMemcpyAsync(&dg, dA, sizeof(double), cudaMemcpyDeviceToHost, s), "diag");
        PALIAL_CK(cudaStreamSynchronize(s), "diag");
        pad = dg > 0 ? dg : 1.0;
    }
    note_launch();
    col_to_tiles_kernel<<<grid_of((long long)npad * npad), 256, 0, s>>>(dA, lda, n, lay_a.as<double>(), npad, nb, pad);
    PALIAL_CK(cudaGetLastError(), "pad A");
    note_launch();
    copy_cols_kernel<<<grid_of((long long)npad * nrhs), 256, 0, s>>>(dB, ldb, n, lay_b.as<double>(), npad, npad, nrhs);
    PALIAL_CK(cudaGetLastError(), "pad B");
    rc = palial_gpu_solve_ir(alg, lay_a.as<double>(), npad, nb, lay_b.as<double>(), lay_x.as<double>(), nrhs, opts, st,
                             stream);
    if (rc < 0 && rc != PALIAL_ERR_NOT_CONVERGED) return rc;
    note_launch();
    copy_cols_kernel<<<grid_of((long long)n * nrhs), 256, 0, s>>>(lay_x.as<double>(), npad, npad, dX, ldx, n, nrhs);
    PALIAL_CK(cudaGetLastError(), "unpad X");
    PALIAL_CK(cudaStreamSynchronize(s), "unpad X");
    return rc;
}

// ---- tiled-matrix files (host) ---------------------------------------------------------------
static const char kMagic[8] = {'P', 'A', 'L', 'T', 'I', 'L', 'E', '1'};

int palial_tiles_write(const char *path, const palial_desc *A) {
    if (!path || !A || !A->matrix || A->tile_size <= 0 || A->matrix_size <= 0 || A->matrix_size % A->tile_size)
        return PALIAL_ERR_ARG;
    FILE *f = fopen(path, "wb");
    if (!f) return PALIAL_ERR_ARG;
    const long long hdr[3] = {A->matrix_size, A->tile_size, 0};
    const size_t count = (size_t)A->matrix_size * A->matrix_size;
    const bool ok = fwrite(kMagic, 1, 8, f) == 8 && fwrite(hdr, sizeof hdr, 1, f) == 1 &&
                    fwrite(A->matrix, sizeof(double), count, f) == count;
    return (fclose(f) == 0 && ok) ? PALIAL_OK : PALIAL_ERR_ARG;
}

// Reads the header (n, nb into *n_out, *nb_out) and, if dst is not NULL, the n*n doubles into
// dst (the caller allocates n*n doubles after a first call with dst = NULL).
int palial_tiles_read(const char *path, int *n_out, int *nb_out, double *dst) {
    if (!path) return PALIAL_ERR_ARG;
    FILE *f = fopen(path, "rb");
    if (!f) return PALIAL_ERR_ARG;
    char magic[8];
    long long hdr[3];
    int rc = PALIAL_ERR_ARG;
    if (fread(magic, 1, 8, f) == 8 && memcmp(magic, kMagic, 8) == 0 && fread(hdr, sizeof hdr, 1, f) == 1 &&
        hdr[0] > 0 && hdr[1] > 0 && hdr[0] % hdr[1] == 0 && hdr[0] <= (1LL << 20) && hdr[2] == 0) {
        if (n_out) *n_out = (int)hdr[0];
        if (nb_out) *nb_out = (int)hdr[1];
        rc = PALIAL_OK;
        if (dst) {
            const size_t count = (size_t)hdr[0] * (size_t)hdr[0];
            if (fread(dst, sizeof(double), count, f) != count) rc = PALIAL_ERR_ARG;
        }
    }
    fclose(f);
    return rc;
}

}  // extern "C"
