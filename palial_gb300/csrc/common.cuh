// common.cuh -- types shared by the host runtime and the device kernels of libpalial_gpu.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace palial {

// ----------------------------------------------------------------------------------------
// Task record of the persistent scheduler.  The host builds one record per unit of work in
// dispatch order; CTAs take records in that order with an atomic ticket.  A record waits
// until every wait object's completion counter reaches its target, runs, then increments
// the counters of its signal objects.  Every target refers to signals of records EARLIER
// in dispatch order, so the smallest unfinished taken record can always proceed: the
// dispatch cannot deadlock whatever the number of resident CTAs.
// ----------------------------------------------------------------------------------------
enum TaskType : uint8_t {
    // Cholesky (upper, A = U^T U), on blocks of size bs
    T_POTRF = 0,   // block (k,k)
    T_TRSM_LUT,    // block (k,m) <- U(k,k)^-T block(k,m); part = column strip
    T_SYRK,        // block (m,m) -= block(k,m)^T block(k,m), upper; part = column strip
    T_GEMM_TN,     // block (n,m) -= block(k,n)^T block(k,m); part = column strip
    // LU, no pivoting
    T_GETRF,       // block (k,k)
    T_TRSM_RUN,    // block (m,k) <- block(m,k) U(k,k)^-1; part = row strip
    T_TRSM_LLU,    // block (k,n) <- L(k,k)^-1 block(k,n) (unit); part = column strip
    T_GEMM_NN,     // block (m,n) -= block(m,k) block(k,n); part = column strip
    // QR (flat tree, on NB tiles)
    T_GEQRT,       // tile (k,k) -> S(k,k)
    T_UNMQR,       // tile (k,n) <- (I - V T V^T)^T tile(k,n); part = column strip
    T_TSQRT,       // tiles (k,k) upper + (m,k) -> S(m,k)
    T_TSMQR,       // tiles (k,n), (m,n) with V = A(m,k), T = S(m,k); part = column strip
    // QR solve back-substitution
    T_TRSM_LUN,    // block (k,n) <- R(k,k)^-1 block(k,n) (R upper, non-unit); part = column strip
    T_NUM_TYPES
};

struct alignas(16) Task {
    uint8_t type;
    uint8_t part;      // strip index
    uint8_t nparts;    // strips of this task
    uint8_t nwait;     // 0..3
    uint16_t k, m, n;  // block / tile coordinates (meaning per type)
    uint8_t nsig;      // 1..2
    uint8_t pad0;
    uint32_t wait_obj[3];
    uint32_t wait_cnt[3];
    uint32_t sig_obj[2];
    uint32_t mat;      // matrix of a batched run (index into SchedParams::mats)
};
static_assert(sizeof(Task) == 48, "Task record layout");

// One matrix of a batched run: its own tile-layout buffer, sizes and counter range.  The FP64
// scheduler reads A; the FP32 scheduler (batched mixed-precision solves) reads Af.
struct MatInfo {
    union {
        double *A;
        float *Af;
    };
    int n, nb, bs;
    int tc;                     // FP32 scheduler: update tasks on the warp tensor cores (BF16x3)
};

struct TraceRec {
    unsigned long long t0, t1;  // %globaltimer ns
    unsigned int smid;
    unsigned int task;          // dispatch index
    long long clk;              // clock64 delta of the task (SM clock estimate)
};

// Device status word layout (int[8]): [0] code, [1] task, [2] tile m, [3] tile n, [4] column,
// [5] zero-pivot flag.
enum StatusSlot { ST_CODE = 0, ST_TASK, ST_M, ST_N, ST_COL, ST_ZEROPIV, ST_NSLOTS = 8 };

struct SchedParams {
    const Task *tasks;
    int ntasks;
    unsigned int *ticket;       // dispatch counter
    unsigned int *counters;     // per object completion counters
    int *status;                // ST_NSLOTS ints
    TraceRec *trace;            // nullptr = no trace
    double *A;                  // tile-layout matrix (device)
    double *S;                  // QR T factors (tile layout) or nullptr
    double *scratch;            // per-worker scratch
    long long scratch_per_worker;  // doubles
    int n, nb, bs;              // matrix size, tile size, block size
    unsigned long long timeout_ns;
    const MatInfo *mats;        // batched run: per-matrix buffers and sizes (else nullptr)
    int *mat_status;            // FP32 batched run: per-matrix breakdown flags (else nullptr)
    float *Af, *Sf;             // FP32 scheduler on one matrix: factors and QR T factors
    float *scratch_f;           // FP32 scheduler: per-worker scratch (scratch_per_worker floats)
    int tc;                     // FP32 QR: TSMQR's products on the warp tensor cores (BF16x3)
};

// Host: count of kernel launches made by the library (every launch wrapper calls this).
void note_launch();

#ifdef __CUDACC__
__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ unsigned int smid() {
    unsigned int r;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned int ld_acquire(const unsigned int *p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_volatile(const int *p) { return *(volatile const int *)p; }

// Element (r, c) of the N x N tile-layout matrix: tile (r/nb, c/nb), offset inside the tile
// (r%nb) + (c%nb)*nb.  A block of size bs | nb lies inside one tile with leading dim nb.
__device__ __forceinline__ double *block_ptr(double *A, int n, int nb, int bs, int bi, int bj) {
    const long long r0 = (long long)bi * bs, c0 = (long long)bj * bs;
    const long long tm = r0 / nb, tn = c0 / nb;
    const long long mt = n / nb;
    return A + (size_t)nb * nb * (size_t)(tm + mt * tn) + (size_t)(r0 % nb) + (size_t)(c0 % nb) * nb;
}
#endif

}  // namespace palial
