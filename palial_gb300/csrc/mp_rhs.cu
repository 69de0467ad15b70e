// mp_rhs.cu -- the refinement's blocked triangular solves with the FP32 factors, one
// persistent launch per direction.
//
// Solve T Y = R (16 right-hand sides, R and Y n x 16 FP32, ld n) by tile rows of the factor:
//   APPLY(k, b):     Y_k[b] = op(D_k^-1)[b rows] R_k      (D_k^-1 the stored inverse of the
//                                                           diagonal factor tile, 32-row block b)
//   UPDATE(k, t, b): R_t[b] -= op(W_kt)[b rows] Y_k       (t after k in the solve order)
// with, per kind: 0 = Cholesky forward U^T y = r (op = transpose, W_kt = U(k,t), t > k);
// 1 = backward U x = y (op = none, W_kt = U(t,k), t < k, k descending); 2 = LU forward
// L y = r (unit L, op = none, W_kt = L(t,k), t > k).
// Tasks run in one launch of persistent CTAs that take records in a fixed order (right-looking:
// step k's applies, then its updates) with an atomic ticket and wait on completion
// counters: per tile t the updates applied to it (APPLY waits for all of them), per 32-row
// block the updates applied to it (updates into one block run in k order: deterministic
// results), per tile k its applies (UPDATE(k, ..) waits for all of Y_k).  Every wait refers to
// earlier records, so the dispatch cannot deadlock; every wait has a deadline and reports
// PALIAL_ERR_TIMEOUT in the status words instead of hanging.
#include <cuda_runtime.h>

#include <map>
#include <tuple>
#include <vector>

#include "host_state.hpp"
#include "tile_f32.cuh"

namespace palial {
namespace mpr {
using namespace f32;

struct alignas(16) RhsTask {
    int type;  // 0 apply, 1 update
    int k, t, b;
    int wobj[2], wcnt[2];
    int sobj[2];
    int nwait, nsig;
};

struct RhsParams {
    const RhsTask *tasks;
    int ntasks;
    unsigned *ticket, *counters;
    int *status;
    const float *W, *Dinv;
    float *R, *Y;
    int n, nb, kind;
    unsigned long long timeout_ns;
};

// Task body: a 32-row block of output rows against all K = NB of one factor tile.  The factor
// slice (32 x NB FP32, read-only) is requested with cp.async BEFORE the task's dependency wait,
// so its latency hides behind the wait; the right-hand-side block (NB x 16) follows once the
// wait is met.  Both land in shared memory in one round trip each.  Thread (r = lane, g = warp)
// accumulates row r over the K range g * NB/8 .. + NB/8 for all 16 columns (float4 reads of the
// factor row and of each column, the columns broadcast across the warp); the 8 partial sums of
// each output are then added in fixed order (deterministic).
constexpr int RB = 32;                 // rows per task
constexpr int KMAX = 512;              // largest NB
constexpr int AP = KMAX + 4;           // pitch of a factor row [r][p] (float4-aligned, conflict-free)
constexpr int BP = KMAX + 4;           // pitch of a right-hand-side column [j][p]
constexpr int RED_P = RW + 1;          // pitch of the partial sums [g][r][j]
// the partial sums reuse the factor slice's space once the products are done: 99 KB per CTA,
// two CTAs per SM (one computes while the other waits or loads)
constexpr int SMEM_FLOATS = RB * AP + RW * BP;
constexpr int SMEM_BYTES = SMEM_FLOATS * 4;
static_assert(RB * AP >= KMAX * RB, "factor slice fits either layout");
static_assert(RB * AP >= (NT / 32) * RB * RED_P, "partial sums fit in the factor slice's space");

__device__ __forceinline__ size_t tile_off(int n, int nb, int tm, int tn) {
    return (size_t)nb * nb * ((size_t)tm + (size_t)(n / nb) * tn);
}

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// op(A)(i, p), i < 32, p < nb: TA: A[p + i * lda] (rows contiguous in p) -> As[i][p];
// else A[i + p * lda] (32 contiguous rows per p) -> As[p][i] (pitch RB).
template <bool TA>
__device__ __forceinline__ void load_factor(float *As, const float *A, int lda, int nb) {
    if (TA) {
        const int per_row = nb / 4;  // 16-byte chunks per row
        for (int c = threadIdx.x; c < RB * per_row; c += NT) {
            const int i = c / per_row, q = c % per_row;
            cp_async16(As + i * AP + q * 4, A + (size_t)q * 4 + (size_t)i * lda);
        }
    } else {
        for (int c = threadIdx.x; c < nb * (RB / 4); c += NT) {
            const int p = c / (RB / 4), q = c % (RB / 4);
            cp_async16(As + p * RB + q * 4, A + (size_t)q * 4 + (size_t)p * lda);
        }
    }
}

// Bs[j][p] = B[p + j * ldb], j < 16, p < nb.
__device__ __forceinline__ void load_rhs(float *Bs, const float *B, int ldb, int nb) {
    const int per_col = nb / 4;
    for (int c = threadIdx.x; c < RW * per_col; c += NT) {
        const int j = c / per_col, q = c % per_col;
        cp_async16(Bs + j * BP + q * 4, B + (size_t)q * 4 + (size_t)j * ldb);
    }
}

// res[r][j] = sum_p op(A)(r, p) Bs[j][p] for the task's 32 rows: partial sums per warp, then
// thread t adds the 8 partials of outputs (r, j) = (t % 32, t / 32) and (t % 32, t / 32 + 8).
template <bool TA>
__device__ __forceinline__ void block_product(const float *As, const float *Bs, float *red, int nb, float out[2]) {
    const int r = threadIdx.x & 31, g = threadIdx.x >> 5;
    const int kq = nb / (NT / 32);  // K per warp
    float acc[RW];
#pragma unroll
    for (int j = 0; j < RW; j++) acc[j] = 0.f;
    for (int p = g * kq; p < (g + 1) * kq; p += 4) {
        float4 a;
        if (TA) {
            a = *reinterpret_cast<const float4 *>(As + r * AP + p);
        } else {
            a.x = As[(p + 0) * RB + r];
            a.y = As[(p + 1) * RB + r];
            a.z = As[(p + 2) * RB + r];
            a.w = As[(p + 3) * RB + r];
        }
#pragma unroll
        for (int j = 0; j < RW; j++) {
            const float4 b = *reinterpret_cast<const float4 *>(Bs + j * BP + p);
            acc[j] = fmaf(a.x, b.x, acc[j]);
            acc[j] = fmaf(a.y, b.y, acc[j]);
            acc[j] = fmaf(a.z, b.z, acc[j]);
            acc[j] = fmaf(a.w, b.w, acc[j]);
        }
    }
    __syncthreads();  // every warp is done with the factor slice: its space takes the partial sums
#pragma unroll
    for (int j = 0; j < RW; j++) red[(g * RB + r) * RED_P + j] = acc[j];
    __syncthreads();
    const int j0 = threadIdx.x >> 5;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int j = j0 + 8 * h;
        float v = 0.f;
#pragma unroll
        for (int q = 0; q < NT / 32; q++) v += red[(q * RB + r) * RED_P + j];
        out[h] = v;
    }
}

__global__ void __launch_bounds__(NT, 2) rhs_solve_kernel(RhsParams p) {
    extern __shared__ __align__(16) float smem[];
    float *As = smem, *Bs = smem + RB * AP, *red = smem;
    __shared__ int s_task, s_abort;
    const int n = p.n, nb = p.nb;
    for (;;) {
        if (threadIdx.x == 0) {
            int tk = p.ntasks;
            if (ld_volatile(p.status + ST_CODE) == 0) tk = (int)atomicAdd(p.ticket, 1u);
            s_task = tk;
            s_abort = 0;
        }
        __syncthreads();
        const int id = s_task;
        if (id >= p.ntasks) break;
        const RhsTask t = p.tasks[id];
        const int rb = t.b * RB;
        // the factor slice does not depend on the wait: request it first
        const float *A;
        bool ta = p.kind == 0;
        if (t.type == 0) {
            const float *D = p.Dinv + (size_t)t.k * nb * nb;
            A = ta ? D + (size_t)rb * nb : D + rb;
        } else {
            A = ta ? p.W + tile_off(n, nb, t.k, t.t) + (size_t)rb * nb : p.W + tile_off(n, nb, t.t, t.k) + rb;
        }
        if (ta)
            load_factor<true>(As, A, nb, nb);
        else
            load_factor<false>(As, A, nb, nb);
        cp_async_commit();
        if (threadIdx.x == 0) {
            const unsigned long long start = globaltimer_ns();
            for (int i = 0; i < t.nwait && !s_abort; i++) {
                const unsigned *c = p.counters + t.wobj[i];
                while (ld_acquire(c) < (unsigned)t.wcnt[i]) {
                    if (ld_volatile(p.status + ST_CODE) != 0) { s_abort = 1; break; }
                    if (globaltimer_ns() - start > p.timeout_ns) {
                        if (atomicCAS(p.status + ST_CODE, 0, -4 /*PALIAL_ERR_TIMEOUT*/) == 0) {
                            p.status[ST_TASK] = id;
                            p.status[ST_COL] = t.wobj[i];
                        }
                        s_abort = 1;
                        break;
                    }
                    __nanosleep(64);
                }
            }
        }
        __syncthreads();
        if (s_abort) {
            cp_async_wait_all();  // no copy of this CTA left landing in shared memory
            break;
        }
        // APPLY reads R_k, UPDATE reads Y_k (both n x 16, column-major)
        load_rhs(Bs, (t.type == 0 ? p.R : p.Y) + (size_t)t.k * nb, n, nb);
        cp_async_commit();
        cp_async_wait_all();
        __syncthreads();
        float v[2];
        if (ta)
            block_product<true>(As, Bs, red, nb, v);
        else
            block_product<false>(As, Bs, red, nb, v);
        const int r = threadIdx.x & 31, j0 = threadIdx.x >> 5;
        if (t.type == 0) {
            // Y_k[rb] = op(D_k^-1)[rb rows] R_k
            float *out = p.Y + (size_t)t.k * nb + rb + r;
            out[(size_t)j0 * n] = v[0];
            out[(size_t)(j0 + 8) * n] = v[1];
        } else {
            // R_t[rb] -= op(W_kt)[rb rows] Y_k
            float *out = p.R + (size_t)t.t * nb + rb + r;
            out[(size_t)j0 * n] = __ldcg(out + (size_t)j0 * n) - v[0];
            out[(size_t)(j0 + 8) * n] = __ldcg(out + (size_t)(j0 + 8) * n) - v[1];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            for (int i = 0; i < t.nsig; i++) atomicAdd(p.counters + t.sobj[i], 1u);
        }
    }
}

// Task list of one direction, right-looking with a lookahead of one tile: step k's updates of
// the next tile come first, then that tile's applies (the critical path: they need only those
// updates and the earlier steps'), then step k's updates of the remaining tiles.  Updates into
// one row block run in k order (deterministic sums).  Every wait refers to earlier records,
// so the in-order dispatch cannot deadlock.
// Objects: [0, mt) updates into tile t; [mt, 2 mt) applies of tile k; [2 mt, 2 mt + mt * nbl)
// updates into row block (t, b).
std::vector<RhsTask> build_tasks(int mt, int nbl, int kind) {
    std::vector<RhsTask> v;
    const auto order = [&](int i) { return kind == 1 ? mt - 1 - i : i; };  // solve order
    std::vector<int> upd_tile(mt, 0), upd_blk((size_t)mt * nbl, 0);
    const auto add_applies = [&](int k) {
        for (int b = 0; b < nbl; b++) {
            RhsTask r{};
            r.type = 0;
            r.k = k;
            r.t = k;
            r.b = b;
            if (upd_tile[k] > 0) {
                r.wobj[0] = k;
                r.wcnt[0] = upd_tile[k];
                r.nwait = 1;
            }
            r.sobj[0] = mt + k;
            r.nsig = 1;
            v.push_back(r);
        }
    };
    const auto add_updates = [&](int k, int t) {
        for (int b = 0; b < nbl; b++) {
            RhsTask r{};
            r.type = 1;
            r.k = k;
            r.t = t;
            r.b = b;
            const int blk = 2 * mt + t * nbl + b;
            r.wobj[0] = mt + k;
            r.wcnt[0] = nbl;  // Y_k complete
            r.nwait = 1;
            if (upd_blk[(size_t)t * nbl + b] > 0) {  // the previous step's update of this block
                r.wobj[1] = blk;
                r.wcnt[1] = upd_blk[(size_t)t * nbl + b];
                r.nwait = 2;
            }
            r.sobj[0] = t;
            r.sobj[1] = blk;
            r.nsig = 2;
            upd_blk[(size_t)t * nbl + b]++;
            upd_tile[t]++;
            v.push_back(r);
        }
    };
    add_applies(order(0));
    for (int ik = 0; ik < mt; ik++) {
        const int k = order(ik);
        if (ik + 1 < mt) {
            add_updates(k, order(ik + 1));
            add_applies(order(ik + 1));
        }
        for (int it = ik + 2; it < mt; it++) add_updates(k, order(it));
    }
    return v;
}

struct Cached {
    DevBuf tasks;
    int ntasks = 0;
};
std::map<std::tuple<int, int, int>, Cached> g_cache;
DevBuf g_counters, g_ticket;

}  // namespace mpr

cudaError_t mpr_configure() {
    return cudaFuncSetAttribute(mpr::rhs_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, mpr::SMEM_BYTES);
}

void mpr_release() {
    for (auto &kv : mpr::g_cache) kv.second.tasks.release();
    mpr::g_cache.clear();
    mpr::g_counters.release();
    mpr::g_ticket.release();
}

// One direction of the blocked triangular solve: R (input, overwritten) -> Y (output), on
// stream s.  status: the factorization's status words (a timed-out wait is reported there).
cudaError_t mpr_solve(const float *W, const float *Dinv, int n, int nb, int kind, float *R, float *Y, int *status,
                      cudaStream_t s) {
    if (nb % mpr::RB || nb > mpr::KMAX || nb % (4 * (f32::NT / 32))) return cudaErrorInvalidValue;
    const int mt = n / nb, nbl = nb / mpr::RB;
    auto key = std::make_tuple(mt, nbl, kind);
    auto it = mpr::g_cache.find(key);
    if (it == mpr::g_cache.end()) {
        const auto tasks = mpr::build_tasks(mt, nbl, kind);
        mpr::Cached c;
        cudaError_t e = c.tasks.ensure(sizeof(mpr::RhsTask) * tasks.size());
        if (e != cudaSuccess) return e;
        e = cudaMemcpy(c.tasks.ptr, tasks.data(), sizeof(mpr::RhsTask) * tasks.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return e;
        c.ntasks = (int)tasks.size();
        it = mpr::g_cache.emplace(key, c).first;
    }
    const int nobj = 2 * mt + mt * nbl;
    cudaError_t e = mpr::g_counters.ensure(sizeof(unsigned) * (size_t)nobj);
    if (e == cudaSuccess) e = mpr::g_ticket.ensure(64);
    if (e == cudaSuccess) e = cudaMemsetAsync(mpr::g_counters.ptr, 0, sizeof(unsigned) * (size_t)nobj, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(mpr::g_ticket.ptr, 0, 64, s);
    if (e != cudaSuccess) return e;
    mpr::RhsParams p;
    p.tasks = it->second.tasks.as<mpr::RhsTask>();
    p.ntasks = it->second.ntasks;
    p.ticket = mpr::g_ticket.as<unsigned>();
    p.counters = mpr::g_counters.as<unsigned>();
    p.status = status;
    p.W = W;
    p.Dinv = Dinv;
    p.R = R;
    p.Y = Y;
    p.n = n;
    p.nb = nb;
    p.kind = kind;
    p.timeout_ns = 30ull * 1000000000ull;
    note_launch();
    mpr::rhs_solve_kernel<<<2 * g.sms, f32::NT, mpr::SMEM_BYTES, s>>>(p);  // two per SM
    return cudaGetLastError();
}

}  // namespace palial

// Checks the task list of one solve direction: every wait must be met by signals of earlier
// records (in-order dispatch cannot deadlock) and every object receives exactly the signals
// its waiters count.  Returns 0, or 1 + the index of the first bad record.  Host only.
extern "C" int palial_gpu_check_solve_tasks(int mt, int nbl, int kind) {
    if (mt <= 0 || nbl <= 0 || kind < 0 || kind > 2) return -1;
    const auto v = palial::mpr::build_tasks(mt, nbl, kind);
    std::vector<int> sig((size_t)(2 * mt + mt * nbl), 0);
    for (size_t i = 0; i < v.size(); i++) {
        const auto &t = v[i];
        for (int w = 0; w < t.nwait; w++)
            if (t.wobj[w] < 0 || t.wobj[w] >= (int)sig.size() || sig[t.wobj[w]] < t.wcnt[w]) return (int)i + 1;
        for (int q = 0; q < t.nsig; q++) sig[t.sobj[q]]++;
    }
    const size_t expect = (size_t)mt * nbl + (size_t)mt * (mt - 1) / 2 * nbl;
    return v.size() == expect ? 0 : (int)v.size() + 1;
}
