// batch_solve.cu -- batched solves A_i x_i = b_i of many independent matrices to FP64-level
// backward error, the factorization precision chosen per matrix.
//
// Matrix i (tile layout, tile nb_i = scheduler block, n_i <= 4096) is factored either in FP32
// (a copy of A_i rounded to FP32; all FP32 matrices in ONE persistent launch of the FP32 task
// scheduler, sched_f32.cu) or in FP64 (a copy of A_i; one launch of the FP64 scheduler), then
// refined in FP64:
//     r = b - A x (FP64, every matrix's rows in one launch),  d = F^-1 (r / |r|)  (factor
//     precision, one CTA per matrix),  x += |r| d,
// until the normwise backward error |r| / (|A| |x| + |b|) (infinity norms) is at most the
// tolerance.  A matrix whose FP32 factorization breaks down, whose refinement stalls (less than
// 2x per step), produces a non-finite residual or runs out of steps is refactored in FP64 and
// refined again (the fallback phase), so every result is FP64-level or reported as not
// converged.  Cholesky uses the upper factor U (A = U^T U), LU the unit-lower L and upper U of
// the no-pivot factorization (the reference's src/lu.h rule).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "rbt.cuh"
#include "host_state.hpp"

namespace palial {
cudaError_t launch_gen_dense(double *X, long long rows, int cols, uint64_t seed, int stream, cudaStream_t s);

namespace {

constexpr int NTS = 256;           // threads of the solve kernels
constexpr int COPY_CHUNK = 16384;  // elements per CTA of the copy kernel
constexpr int MAX_N = 4096;        // the correction solve keeps the vector in shared memory
constexpr int PART_ROWS = 16;      // partial-sum groups of the row-oriented updates

struct SolveMat {
    const double *A;  // FP64 matrix (tile layout, tile nb), read only
    const double *b;  // right-hand side
    double *x;        // solution
    double *r;        // residual
    const void *F;    // factors (float or double), same layout as A
    const float *rnd; // LU of the random-butterfly transform U^T A V: the 4n randoms (else null)
    int n, nb, alg, f32;
};

struct CopyJob {
    const double *src;
    void *dst;
    long long elems;
    int to_f32;
};

// largest j with first[j] <= bid (first ascending, first[0] = 0)
__device__ __forceinline__ int find_job(const int *first, int njobs, int bid) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (first[mid] <= bid) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Every job's FP64 matrix copied (or rounded to FP32) into its factor buffer; COPY_CHUNK
// elements per CTA, first[j] = the first CTA of job j.
__global__ void __launch_bounds__(NTS) copy_kernel(const CopyJob *jobs, const int *first, int njobs) {
    __shared__ int s_j;
    if (threadIdx.x == 0) s_j = find_job(first, njobs, (int)blockIdx.x);
    __syncthreads();
    const CopyJob jb = jobs[s_j];
    const long long base = (long long)((int)blockIdx.x - first[s_j]) * COPY_CHUNK;
    const long long end = min(jb.elems, base + COPY_CHUNK);
    if (jb.to_f32) {
        float *d = static_cast<float *>(jb.dst);
        for (long long e = base + threadIdx.x; e < end; e += NTS) d[e] = (float)__ldcs(jb.src + e);
    } else {
        double *d = static_cast<double *>(jb.dst);
        for (long long e = base + threadIdx.x; e < end; e += NTS) d[e] = __ldcs(jb.src + e);
    }
}

__device__ __forceinline__ unsigned long long abs_bits(double v) {
    return (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;  // NaN sorts above inf
}

__device__ __forceinline__ unsigned long long block_max(unsigned long long v, unsigned long long *red) {
    for (int o = 16; o; o >>= 1) {
        const unsigned long long y = __shfl_xor_sync(0xffffffffu, v, o);
        v = y > v ? y : v;
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    unsigned long long m = 0;
#pragma unroll
    for (int i = 0; i < NTS / 32; i++) m = red[i] > m ? red[i] : m;
    return m;
}

// r = b - A x for 256 rows of one matrix per CTA (jobs: {matrix, first row}); first: x = 0
// (r = b) and the row sums |A| are taken.  norms[4m + 0..3] = |r|, |x|, |A| (first), |b|
// (first), infinity norms as bit patterns (atomicMax; a NaN dominates).
__global__ void __launch_bounds__(NTS) residual_kernel(const SolveMat *mats, const int2 *jobs, int first,
                                                       unsigned long long *norms) {
    __shared__ unsigned long long red[NTS / 32];
    const int2 jb = jobs[blockIdx.x];
    const SolveMat M = mats[jb.x];
    const int i = jb.y + (int)threadIdx.x;
    unsigned long long rmax = 0, xmax = 0, amax = 0, bmax = 0;
    if (i < M.n) {
        const int nb = M.nb, mt = M.n / nb;
        const double bi = M.b[i];
        const double *row = M.A + (size_t)nb * nb * (size_t)(i / nb) + (i % nb);  // tile column 0
        const size_t tstride = (size_t)nb * nb * mt;                              // next tile column
        double r;
        if (first) {
            double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
            for (int jt = 0; jt < mt; jt++) {
                const double *tp = row + tstride * jt;
#pragma unroll 4
                for (int jj = 0; jj < nb; jj += 4) {
                    s0 += fabs(tp[(size_t)jj * nb]);
                    s1 += fabs(tp[(size_t)(jj + 1) * nb]);
                    s2 += fabs(tp[(size_t)(jj + 2) * nb]);
                    s3 += fabs(tp[(size_t)(jj + 3) * nb]);
                }
            }
            amax = abs_bits((s0 + s1) + (s2 + s3));
            bmax = abs_bits(bi);
            r = bi;
        } else {
            double a0 = bi, a1 = 0, a2 = 0, a3 = 0;
            for (int jt = 0; jt < mt; jt++) {
                const double *tp = row + tstride * jt;
                const double *xp = M.x + (size_t)jt * nb;
#pragma unroll 4
                for (int jj = 0; jj < nb; jj += 4) {
                    a0 = fma(-tp[(size_t)jj * nb], __ldg(xp + jj), a0);
                    a1 = fma(-tp[(size_t)(jj + 1) * nb], __ldg(xp + jj + 1), a1);
                    a2 = fma(-tp[(size_t)(jj + 2) * nb], __ldg(xp + jj + 2), a2);
                    a3 = fma(-tp[(size_t)(jj + 3) * nb], __ldg(xp + jj + 3), a3);
                }
            }
            r = (a0 + a1) + (a2 + a3);
            xmax = abs_bits(M.x[i]);
        }
        M.r[i] = r;
        rmax = abs_bits(r);
    }
    unsigned long long *out = norms + 4 * (size_t)jb.x;
    rmax = block_max(rmax, red);
    if (threadIdx.x == 0) atomicMax(out + 0, rmax);
    xmax = block_max(xmax, red);
    if (threadIdx.x == 0 && !first) atomicMax(out + 1, xmax);
    if (first) {
        amax = block_max(amax, red);
        if (threadIdx.x == 0) atomicMax(out + 2, amax);
        bmax = block_max(bmax, red);
        if (threadIdx.x == 0) atomicMax(out + 3, bmax);
    }
}

template <class T>
struct Vec;
template <>
struct Vec<float> {
    static constexpr int W = 4;
    __device__ static void load(const float *p, float (&v)[4]) {
        const float4 q = __ldg(reinterpret_cast<const float4 *>(p));
        v[0] = q.x, v[1] = q.y, v[2] = q.z, v[3] = q.w;
    }
};
template <>
struct Vec<double> {
    static constexpr int W = 2;
    __device__ static void load(const double *p, double (&v)[2]) {
        const double2 q = __ldg(reinterpret_cast<const double2 *>(p));
        v[0] = q.x, v[1] = q.y;
    }
};

template <class T>
struct Fac {
    const T *F;
    int nb, mt;
    // element (r, c) of the factor matrix (tile layout)
    __device__ const T *at(int r, int c) const {
        return F + (size_t)nb * nb * ((size_t)(r / nb) + (size_t)mt * (c / nb)) + (r % nb) + (size_t)(c % nb) * nb;
    }
};

// v[rb + c] -= sum_{p < rb} U(p, rb + c) v[p], c < 64 (columns of U: warp per column, lanes
// along p, vector loads).
template <class T>
__device__ void column_update(const Fac<T> &f, int rb, T *v) {
    constexpr int W = Vec<T>::W;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int c = warp; c < 64; c += NTS / 32) {
        const int q = rb + c;
        T s = 0;
        for (int p0 = 0; p0 < rb; p0 += f.nb) {
            const int len = min(f.nb, rb - p0);  // a multiple of 64
            const T *col = f.at(p0, q);
#pragma unroll 2
            for (int e = lane * W; e < len; e += 32 * W) {
                T a[W];
                Vec<T>::load(col + e, a);
#pragma unroll
                for (int k = 0; k < W; k++) s += a[k] * v[p0 + e + k];
            }
        }
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) v[q] -= s;
    }
    __syncthreads();
}

// v[rb + u] -= sum_{plo <= p < phi} F(rb + u, p) v[p], u < 64 (rows of F: 64 / W threads
// cover the 64 rows with vector loads, PART groups split p; partial sums reduced in part).
template <class T>
__device__ void row_update(const Fac<T> &f, int rb, int plo, int phi, T *v, T *part) {
    constexpr int W = Vec<T>::W, RT = 64 / W, G = NTS / RT;
    static_assert(G <= PART_ROWS, "partial-sum rows");
    const int rg = threadIdx.x % RT, pg = threadIdx.x / RT;
    T acc[W];
#pragma unroll
    for (int k = 0; k < W; k++) acc[k] = 0;
#pragma unroll 4
    for (int p = plo + pg; p < phi; p += G) {
        T a[W];
        Vec<T>::load(f.at(rb + rg * W, p), a);
        const T vp = v[p];
#pragma unroll
        for (int k = 0; k < W; k++) acc[k] += a[k] * vp;
    }
#pragma unroll
    for (int k = 0; k < W; k++) part[pg * 64 + rg * W + k] = acc[k];
    __syncthreads();
    if (threadIdx.x < 64) {
        T s = 0;
        for (int g2 = 0; g2 < G; g2++) s += part[g2 * 64 + threadIdx.x];
        v[rb + threadIdx.x] -= s;
    }
    __syncthreads();
}

// The 64 x 64 diagonal block of the factor at rb, one warp, unknowns in registers (lane owns
// j = lane and lane + 32):  KIND 0: U^T y = v;  KIND 2: L y = v (unit lower);  KIND 3: U x = v.
template <class T, int KIND>
__device__ void diag_solve(const Fac<T> &f, int rb, T *v, T (*Ds)[65]) {
    for (int e = threadIdx.x; e < 64 * 64; e += NTS) {
        const int r = e & 63, c = e >> 6;
        Ds[c][r] = *f.at(rb + r, rb + c);  // Ds[c][r] = F(rb + r, rb + c)
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        T a0 = v[rb + lane], a1 = v[rb + lane + 32];
        for (int s = 0; s < 64; s++) {
            const int i = (KIND == 3) ? 63 - s : s;
            T yi = __shfl_sync(0xffffffffu, i < 32 ? a0 : a1, i & 31);
            if (KIND != 2) yi = yi / Ds[i][i];
            if (lane == (i & 31)) {
                if (i < 32) a0 = yi;
                else a1 = yi;
            }
            const int j0 = lane, j1 = lane + 32;
            if (KIND == 0) {  // a_j -= U(i, j) y_i, j > i
                if (j0 > i) a0 -= Ds[j0][i] * yi;
                if (j1 > i) a1 -= Ds[j1][i] * yi;
            } else if (KIND == 2) {  // a_j -= L(j, i) y_i, j > i
                if (j0 > i) a0 -= Ds[i][j0] * yi;
                if (j1 > i) a1 -= Ds[i][j1] * yi;
            } else {  // a_j -= U(j, i) x_i, j < i
                if (j0 < i) a0 -= Ds[i][j0] * yi;
                if (j1 < i) a1 -= Ds[i][j1] * yi;
            }
        }
        v[rb + lane] = a0;
        v[rb + lane + 32] = a1;
    }
    __syncthreads();
}

// One CTA per matrix (jobs: {matrix, assign}): v = r / |r| in the factor's precision, forward
// and backward substitution with the factors, x = (assign ? 0 : x) + |r| v.  Dynamic shared
// memory: v (nmax) | Ds[64][65] | part[PART_ROWS][64], all of type T.
template <class T>
__global__ void __launch_bounds__(NTS) correction_kernel(const SolveMat *mats, const int2 *jobs,
                                                         const unsigned long long *norms, int nmax) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *v = reinterpret_cast<T *>(smem_raw);
    T(*Ds)[65] = reinterpret_cast<T(*)[65]>(v + nmax);
    T *part = reinterpret_cast<T *>(Ds + 64);
    const int2 jb = jobs[blockIdx.x];
    const SolveMat M = mats[jb.x];
    const int n = M.n;
    const double scale = __longlong_as_double((long long)norms[4 * (size_t)jb.x]);
    if (!(scale > 0.0) || isinf(scale)) {  // r = 0: x stays (0 if new); non-finite: NaN
        if (jb.y)
            for (int i = threadIdx.x; i < n; i += NTS) M.x[i] = scale == 0.0 ? 0.0 : __longlong_as_double(-1LL);
        return;
    }
    Fac<T> f;
    f.F = static_cast<const T *>(M.F);
    f.nb = M.nb;
    f.mt = n / M.nb;
    const double inv = 1.0 / scale;
    for (int i = threadIdx.x; i < n; i += NTS) v[i] = (T)(M.r[i] * inv);
    __syncthreads();
    if constexpr (sizeof(T) == 4) {
        if (M.rnd) {  // factors of U^T A V: v <- U^T v
            const int q = n / 4;
            const rbt::Rand U = rbt::rand_view(M.rnd, n);
            for (int i = threadIdx.x; i < q; i += NTS) rbt::wt4(U, i, q, v[i], v[i + q], v[i + 2 * q], v[i + 3 * q]);
            __syncthreads();
        }
    }
    for (int rb = 0; rb < n; rb += 64) {  // forward
        if (M.alg == 0) {
            if (rb) column_update<T>(f, rb, v);
            diag_solve<T, 0>(f, rb, v, Ds);
        } else {
            if (rb) row_update<T>(f, rb, 0, rb, v, part);
            diag_solve<T, 2>(f, rb, v, Ds);
        }
    }
    for (int rb = n - 64; rb >= 0; rb -= 64) {  // backward: U x = y
        if (rb + 64 < n) row_update<T>(f, rb, rb + 64, n, v, part);
        diag_solve<T, 3>(f, rb, v, Ds);
    }
    if constexpr (sizeof(T) == 4) {
        if (M.rnd) {  // z = V y
            __syncthreads();
            const int q = n / 4;
            const rbt::Rand Vr = rbt::rand_view(M.rnd + 2 * n, n);
            for (int i = threadIdx.x; i < q; i += NTS) rbt::w4(Vr, i, q, v[i], v[i + q], v[i + 2 * q], v[i + 3 * q]);
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < n; i += NTS) M.x[i] = (jb.y ? 0.0 : M.x[i]) + scale * (double)v[i];
}

template <class T>
size_t correction_smem(int nmax) {
    return sizeof(T) * ((size_t)nmax + 64 * 65 + (size_t)PART_ROWS * 64);
}

// ---- host ---------------------------------------------------------------------------------
DevBuf w32, w64, w64b, wr, wnorm, wmats, wjobs, wfirst, wcopy, wrand;

bool g_configured = false;
cudaError_t configure() {
    if (g_configured) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(correction_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)correction_smem<float>(MAX_N));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(correction_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)correction_smem<double>(MAX_N));
    g_configured = e == cudaSuccess;
    return e;
}

size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

struct Solver {
    int count;
    std::vector<SolveMat> mats;
    std::vector<double> anorm, bnorm, berr, tol, eta_prev;
    std::vector<int> iters, state;  // state: 0 active, 1 converged, 2 failed
    std::vector<int> tc;            // 1: FP32 factorization with its updates on the tensor cores (BF16x3)
    cudaStream_t s;
    palial_status *st;
    double factor_s = 0;

    int upload_table() {
        PALIAL_CK(wmats.ensure(sizeof(SolveMat) * (size_t)count), "alloc table");
        PALIAL_CK(cudaMemcpyAsync(wmats.ptr, mats.data(), sizeof(SolveMat) * (size_t)count, cudaMemcpyHostToDevice, s),
                  "upload table");
        return PALIAL_OK;
    }

    // copy (to_f32: round) A into the factor buffers of the listed matrices
    int copy(const std::vector<int> &ms) {
        std::vector<CopyJob> jobs;
        std::vector<int> first;
        long long ctas = 0;
        for (int m : ms) {
            const long long el = (long long)mats[m].n * mats[m].n;
            jobs.push_back(CopyJob{mats[m].A, const_cast<void *>(mats[m].F), el, mats[m].f32});
            first.push_back((int)ctas);
            ctas += (el + COPY_CHUNK - 1) / COPY_CHUNK;
        }
        if (jobs.empty()) return PALIAL_OK;
        if (ctas > 0x7fffffff) return set_status(st, PALIAL_ERR_ARG, "batch too large");
        PALIAL_CK(wcopy.ensure(sizeof(CopyJob) * jobs.size()), "alloc copy jobs");
        PALIAL_CK(wfirst.ensure(sizeof(int) * first.size()), "alloc copy jobs");
        PALIAL_CK(cudaMemcpyAsync(wcopy.ptr, jobs.data(), sizeof(CopyJob) * jobs.size(), cudaMemcpyHostToDevice, s),
                  "upload copy jobs");
        PALIAL_CK(cudaMemcpyAsync(wfirst.ptr, first.data(), sizeof(int) * first.size(), cudaMemcpyHostToDevice, s),
                  "upload copy jobs");
        note_launch();
        copy_kernel<<<(unsigned)ctas, NTS, 0, s>>>(wcopy.as<CopyJob>(), wfirst.as<int>(), (int)jobs.size());
        PALIAL_CK(cudaGetLastError(), "copy");
        // the job tables are reused by the next call: finish before returning
        PALIAL_CK(cudaStreamSynchronize(s), "copy");
        return PALIAL_OK;
    }

    // factor the listed matrices (all of one precision) in one batched launch; FP32
    // breakdowns are marked failed.  FP32 tasks run on the matrix's tile as the block; FP64
    // tasks on 64-blocks inside it (the FP64 scheduler's fastest block on every size class of
    // the synthetic batch: its FP64 pipe favours more, shorter tasks)
    int factor(const std::vector<int> &ms, bool f32) {
        if (ms.empty()) return PALIAL_OK;
        std::vector<int> algs, ns, nbs, bss, tcs;
        std::vector<void *> bufs;
        for (int m : ms) {
            algs.push_back(mats[m].alg);
            ns.push_back(mats[m].n);
            nbs.push_back(mats[m].nb);
            bss.push_back(f32 ? mats[m].nb : 64);
            bufs.push_back(const_cast<void *>(mats[m].F));
            tcs.push_back(tc[m]);
        }
        std::vector<int> flags(ms.size(), 0);
        palial_opts o;
        palial_opts_default(&o);
        palial_status s2;
        memset(&s2, 0, sizeof s2);
        const int rc = batched_run((int)ms.size(), algs.data(), ns.data(), nbs.data(), bss.data(), bufs.data(), f32,
                                   flags.data(), &o, &s2, nullptr, s, tcs.data());
        factor_s += s2.seconds;
        if (rc < 0) return set_status(st, rc, "batched factorization: %s", s2.message);
        for (size_t j = 0; j < ms.size(); j++)
            if (flags[j]) state[ms[j]] = 2;
        return PALIAL_OK;
    }

    // residuals of the listed matrices; fills rn[m], xn[m] (and anorm/bnorm when first)
    int residual(const std::vector<int> &ms, bool first, std::vector<double> &rn, std::vector<double> &xn) {
        std::vector<int2> jobs;
        for (int m : ms)
            for (int r0 = 0; r0 < mats[m].n; r0 += NTS) jobs.push_back(make_int2(m, r0));
        if (jobs.empty()) return PALIAL_OK;
        PALIAL_CK(wjobs.ensure(sizeof(int2) * jobs.size()), "alloc jobs");
        PALIAL_CK(wnorm.ensure(sizeof(unsigned long long) * 4 * (size_t)count), "alloc norms");
        PALIAL_CK(cudaMemcpyAsync(wjobs.ptr, jobs.data(), sizeof(int2) * jobs.size(), cudaMemcpyHostToDevice, s),
                  "upload jobs");
        PALIAL_CK(cudaMemsetAsync(wnorm.ptr, 0, sizeof(unsigned long long) * 4 * (size_t)count, s), "clear norms");
        note_launch();
        residual_kernel<<<(unsigned)jobs.size(), NTS, 0, s>>>(wmats.as<SolveMat>(), wjobs.as<int2>(), first ? 1 : 0,
                                                              wnorm.as<unsigned long long>());
        PALIAL_CK(cudaGetLastError(), "residual");
        std::vector<double> h(4 * (size_t)count);
        PALIAL_CK(cudaMemcpyAsync(h.data(), wnorm.ptr, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s), "norms");
        PALIAL_CK(cudaStreamSynchronize(s), "residual");
        for (int m : ms) {
            rn[m] = h[4 * (size_t)m];
            xn[m] = h[4 * (size_t)m + 1];
            if (first) {
                anorm[m] = h[4 * (size_t)m + 2];
                bnorm[m] = h[4 * (size_t)m + 3];
            }
        }
        return PALIAL_OK;
    }

    // corrections of the listed matrices (assign: x was not set yet)
    int correct(const std::vector<int> &ms, const std::vector<char> &assign) {
        for (int prec = 0; prec < 2; prec++) {
            std::vector<int2> jobs;
            int nmax = 64;
            for (int m : ms)
                if (mats[m].f32 == prec) {
                    jobs.push_back(make_int2(m, assign[m] ? 1 : 0));
                    nmax = std::max(nmax, mats[m].n);
                }
            if (jobs.empty()) continue;
            // larger matrices first: the longest CTAs start in the first wave
            std::stable_sort(jobs.begin(), jobs.end(), [&](int2 a, int2 b) { return mats[a.x].n > mats[b.x].n; });
            PALIAL_CK(wjobs.ensure(sizeof(int2) * jobs.size()), "alloc jobs");
            PALIAL_CK(cudaMemcpyAsync(wjobs.ptr, jobs.data(), sizeof(int2) * jobs.size(), cudaMemcpyHostToDevice, s),
                      "upload jobs");
            note_launch();
            if (prec)
                correction_kernel<float><<<(unsigned)jobs.size(), NTS, correction_smem<float>(nmax), s>>>(
                    wmats.as<SolveMat>(), wjobs.as<int2>(), wnorm.as<unsigned long long>(), nmax);
            else
                correction_kernel<double><<<(unsigned)jobs.size(), NTS, correction_smem<double>(nmax), s>>>(
                    wmats.as<SolveMat>(), wjobs.as<int2>(), wnorm.as<unsigned long long>(), nmax);
            PALIAL_CK(cudaGetLastError(), "correction");
            PALIAL_CK(cudaStreamSynchronize(s), "correction");  // wjobs is reused
        }
        return PALIAL_OK;
    }

    // Refinement of the listed matrices from x = 0 until each converges or fails.
    int refine(std::vector<int> ms, int max_iter) {
        std::vector<double> rn(count, 0), xn(count, 0);
        std::vector<char> assign(count, 0);
        int rc = residual(ms, true, rn, xn);
        if (rc) return rc;
        for (int m : ms) {
            assign[m] = 1;
            eta_prev[m] = INFINITY;
            iters[m] = 0;
        }
        for (int it = 1; it <= max_iter && !ms.empty(); it++) {
            rc = correct(ms, assign);
            if (rc) return rc;
            for (int m : ms) assign[m] = 0;
            rc = residual(ms, false, rn, xn);
            if (rc) return rc;
            std::vector<int> next;
            for (int m : ms) {
                iters[m] = it;
                const double den = anorm[m] * xn[m] + bnorm[m];
                const double eta = rn[m] == 0.0 ? 0.0 : rn[m] / den;
                berr[m] = eta;
                if (eta <= tol[m]) state[m] = 1;
                else if (!std::isfinite(eta) || (it >= 2 && eta > 0.5 * eta_prev[m]) || it == max_iter) state[m] = 2;
                else next.push_back(m);
                eta_prev[m] = eta;
            }
            ms.swap(next);
        }
        return PALIAL_OK;
    }
};

}  // namespace

void batch_solve_release() {
    for (DevBuf *b : {&w32, &w64, &w64b, &wr, &wnorm, &wmats, &wjobs, &wfirst, &wcopy, &wrand}) b->release();
    g_configured = false;  // a later init (possibly another device) sets the attributes again
}

int batched_solve_run(int count, const int *algs, const int *ns, const int *nbs, const double *const *dA,
                      const double *const *dB, double *const *dX, const int *precs, const palial_opts *opts,
                      palial_status *st, int *iters, double *berr, double *phases, void *stream) {
    if (st) memset(st, 0, sizeof *st);
    double ph[3] = {0, 0, 0};
    if (!phases) phases = ph;
    for (int i = 0; i < 3; i++) phases[i] = 0;
    if (count <= 0 || !algs || !ns || !nbs || !dA || !dB || !dX) return set_status(st, PALIAL_ERR_ARG, "empty batch");
    for (int i = 0; i < count; i++) {
        const int p = precs ? precs[i] : PALIAL_PREC_FP32;
        if ((algs[i] != 0 && algs[i] != 1) || ns[i] <= 0 || ns[i] > MAX_N || nbs[i] <= 0 || nbs[i] % 64 ||
            ns[i] % nbs[i] || !dA[i] || !dB[i] || !dX[i] ||
            (p != PALIAL_PREC_FP32 && p != PALIAL_PREC_FP64 && p != PALIAL_PREC_BF16X3) ||
            (reinterpret_cast<uintptr_t>(dA[i]) & 15))
            return set_status(st, PALIAL_ERR_ARG, "matrix %d: alg %d n %d nb %d precision %d (n <= %d, nb | n, 64 | nb)",
                              i, algs[i], ns[i], nbs[i], p, MAX_N);
    }
    int rc = ensure_init(st);
    if (rc) return rc;
    PALIAL_CK(configure(), "configure");
    palial_opts o;
    palial_opts_default(&o);
    if (opts) o = *opts;
    const int max_iter = o.ir_max_iter > 0 ? o.ir_max_iter : 30;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const auto t0 = std::chrono::steady_clock::now();

    // workspace: FP32 factors, FP64 factors, residuals (offsets in elements, 16-byte aligned)
    std::vector<size_t> off(count), offr(count);
    size_t n32 = 0, n64 = 0, nr = 0;
    for (int i = 0; i < count; i++) {
        const size_t el = (size_t)ns[i] * ns[i];
        const bool f32 = !precs || precs[i] != PALIAL_PREC_FP64;
        off[i] = f32 ? n32 : n64;
        (f32 ? n32 : n64) += round_up(el, 4);
        offr[i] = nr;
        nr += round_up((size_t)ns[i], 2);
    }
    PALIAL_CK(w32.ensure(sizeof(float) * std::max<size_t>(4, n32)), "alloc FP32 factors");
    PALIAL_CK(w64.ensure(sizeof(double) * std::max<size_t>(2, n64)), "alloc FP64 factors");
    PALIAL_CK(wr.ensure(sizeof(double) * nr), "alloc residuals");

    Solver sv;
    sv.count = count;
    sv.s = s;
    sv.st = st;
    sv.mats.resize(count);
    sv.anorm.assign(count, 0);
    sv.bnorm.assign(count, 0);
    sv.berr.assign(count, INFINITY);
    sv.eta_prev.assign(count, INFINITY);
    sv.tol.resize(count);
    sv.iters.assign(count, 0);
    sv.state.assign(count, 0);
    sv.tc.assign(count, 0);
    std::vector<int> all(count), m32, m64;
    std::iota(all.begin(), all.end(), 0);
    for (int i = 0; i < count; i++) {
        const bool f32 = !precs || precs[i] != PALIAL_PREC_FP64;
        sv.tc[i] = (precs && precs[i] == PALIAL_PREC_BF16X3) ? 1 : 0;
        SolveMat &m = sv.mats[i];
        m.A = dA[i];
        m.b = dB[i];
        m.x = dX[i];
        m.r = wr.as<double>() + offr[i];
        m.F = f32 ? (const void *)(w32.as<float>() + off[i]) : (const void *)(w64.as<double>() + off[i]);
        m.rnd = nullptr;
        m.n = ns[i];
        m.nb = nbs[i];
        m.alg = algs[i];
        m.f32 = f32 ? 1 : 0;
        sv.tol[i] = o.ir_tol > 0 ? o.ir_tol : 1e-14 * ns[i];
        (f32 ? m32 : m64).push_back(i);
    }
    // U^T A V (float) into the FP32 factor buffers of the listed matrices, each with its own 4n
    // randoms (seed 1)
    std::vector<float> hq;
    const auto butterfly = [&](const std::vector<int> &ms) -> int {
        std::vector<size_t> offq(ms.size());
        size_t nq = 0;
        for (size_t j = 0; j < ms.size(); j++) {
            offq[j] = nq;
            nq += 4 * (size_t)ns[ms[j]];
        }
        hq.assign(nq, 0.f);
        for (size_t j = 0; j < ms.size(); j++) rbt_randoms(ns[ms[j]], 1, hq.data() + offq[j]);
        PALIAL_CK(wrand.ensure(sizeof(float) * nq), "alloc butterflies");
        PALIAL_CK(cudaMemcpyAsync(wrand.ptr, hq.data(), sizeof(float) * nq, cudaMemcpyHostToDevice, s), "butterflies");
        for (size_t j = 0; j < ms.size(); j++) {
            SolveMat &m = sv.mats[ms[j]];
            m.rnd = wrand.as<float>() + offq[j];
            PALIAL_CK(rbt_transform_matrix_with(m.A, static_cast<float *>(const_cast<void *>(m.F)), m.n, m.nb, m.rnd, s),
                      "butterfly transform");
            sv.state[ms[j]] = 0;
        }
        PALIAL_CK(cudaStreamSynchronize(s), "butterflies");  // hq is reused
        return PALIAL_OK;
    };
    rc = sv.upload_table();
    if (rc) return rc;
    rc = sv.copy(all);
    if (rc) return rc;
    // opts.reserved[6] = 1: every FP32 LU matrix on its butterfly transform from the start
    if (o.reserved[6] == 1) {
        std::vector<int> lu32;
        for (int i : m32)
            if (algs[i] == 1) lu32.push_back(i);
        if (!lu32.empty()) {
            rc = butterfly(lu32);
            if (rc) return rc;
            rc = sv.upload_table();
            if (rc) return rc;
        }
    }
    rc = sv.factor(m32, true);
    if (rc) return rc;
    rc = sv.factor(m64, false);
    if (rc) return rc;
    const auto t1 = std::chrono::steady_clock::now();
    phases[0] = std::chrono::duration<double>(t1 - t0).count();
    std::vector<int> run;
    for (int i = 0; i < count; i++)
        if (sv.state[i] == 0) run.push_back(i);
    rc = sv.refine(run, max_iter);
    if (rc) return rc;
    const auto t2 = std::chrono::steady_clock::now();
    phases[1] = std::chrono::duration<double>(t2 - t1).count();

    // fallback phase.  First the no-pivot LU matrices FP32 could not handle (pivot growth):
    // FP32 LU of their random-butterfly transform U^T A V (Parker 1995: no pivoting needed with
    // high probability), refined against A with z = V (LU)^-1 U^T r.  Then every FP32 matrix
    // still failing is refactored in FP64.  opts.reserved[6] = -1 skips the butterfly stage (and
    // matrices already on their butterfly transform go straight to FP64).
    std::vector<int> rb;
    for (int i = 0; i < count; i++)
        if (sv.state[i] == 2 && sv.mats[i].f32 && algs[i] == 1 && !sv.mats[i].rnd && o.reserved[6] != -1)
            rb.push_back(i);
    int butterflies = 0;
    if (!rb.empty()) {
        rc = butterfly(rb);
        if (rc) return rc;
        rc = sv.upload_table();
        if (rc) return rc;
        rc = sv.factor(rb, true);
        if (rc) return rc;
        std::vector<int> again;
        for (int i : rb)
            if (sv.state[i] == 0) again.push_back(i);
        rc = sv.refine(again, max_iter);
        if (rc) return rc;
    }
    for (int i = 0; i < count; i++)
        if (sv.state[i] == 1 && sv.mats[i].rnd) butterflies++;
    std::vector<int> fb;
    for (int i = 0; i < count; i++)
        if (sv.state[i] == 2 && sv.mats[i].f32) fb.push_back(i);
    if (!fb.empty()) {
        size_t nfb = 0;
        std::vector<size_t> offb(fb.size());
        for (size_t j = 0; j < fb.size(); j++) {
            offb[j] = nfb;
            nfb += round_up((size_t)ns[fb[j]] * ns[fb[j]], 2);
        }
        PALIAL_CK(w64b.ensure(sizeof(double) * nfb), "alloc fallback factors");
        for (size_t j = 0; j < fb.size(); j++) {
            SolveMat &m = sv.mats[fb[j]];
            m.F = w64b.as<double>() + offb[j];
            m.f32 = 0;
            m.rnd = nullptr;
            sv.state[fb[j]] = 0;
        }
        rc = sv.upload_table();
        if (rc) return rc;
        rc = sv.copy(fb);
        if (rc) return rc;
        rc = sv.factor(fb, false);
        if (rc) return rc;
        std::vector<int> again;
        for (int i : fb)
            if (sv.state[i] == 0) again.push_back(i);
        rc = sv.refine(again, max_iter);
        if (rc) return rc;
    }
    PALIAL_CK(cudaStreamSynchronize(s), "batched solve");
    const auto t3 = std::chrono::steady_clock::now();
    phases[2] = std::chrono::duration<double>(t3 - t2).count();
    const double wall = std::chrono::duration<double>(t3 - t0).count();

    int not_conv = 0, max_it = 0;
    double worst = 0, flops = 0;
    for (int i = 0; i < count; i++) {
        if (sv.state[i] != 1) not_conv++;
        max_it = std::max(max_it, sv.iters[i]);
        worst = std::max(worst, std::isfinite(sv.berr[i]) ? sv.berr[i] : INFINITY);
        flops += algorithmic_flops(algs[i], ns[i]);
        if (iters) iters[i] = std::find(fb.begin(), fb.end(), i) != fb.end() ? -sv.iters[i] - 1 : sv.iters[i];
        if (berr) berr[i] = sv.berr[i];
    }
    if (st) {
        st->seconds = wall;
        st->total_seconds = wall;
        st->factor_seconds = sv.factor_s;
        st->tflops = flops / std::max(1e-12, wall) * 1e-12;
        st->ir_iters = max_it;
        st->backward_error = worst;
        st->fallbacks = (int)fb.size();  // matrices refactored in FP64
        st->butterflies = butterflies;    // LU matrices solved on their butterfly transform
    }
    if (not_conv)
        return set_status(st, PALIAL_ERR_NOT_CONVERGED, "%d of %d matrices above their tolerance (worst %.3g)",
                          not_conv, count, worst);
    return set_status(st, PALIAL_OK);
}

}  // namespace palial

using namespace palial;

extern "C" {

int palial_gpu_batched_solve(int count, const int *algs, const int *ns, const int *nbs, const double *const *dA,
                             const double *const *dB, double *const *dX, const int *precs, const palial_opts *opts,
                             palial_status *st, int *iters, double *berr, void *stream) {
    return batched_solve_run(count, algs, ns, nbs, dA, dB, dX, precs, opts, st, iters, berr, nullptr, stream);
}

}  // extern "C"
