// mp_driver.cu -- mixed-precision Cholesky / LU with iterative refinement (host driver).
//
// Factorization (right-looking, one k step at a time on one stream), on an FP32 working
// copy W of A in the reference's tile layout:
//   1. the diagonal tile W(k,k) is factored in FP32 by one CTA (mp_diag.cu): POTRF for
//      Cholesky, no-pivot GETRF with the reference's pivot rule for LU;
//   2. the panel is solved in FP32 (substitution against the diagonal factor);
//   3. the panel is packed into K-major low-precision operands (BF16, FP8 e4m3 with per-tile
//      scales, or BF16 hi + lo) and the whole trailing matrix is updated by the tcgen05
//      kernel with FP32 accumulation.
// Refinement: x0 = 0, r = b; repeat: solve with the FP32 factors (blocked triangular
// solves), x += d (FP64), r = b - A x with the original FP64 matrix, until the normwise
// backward error max_j ||r_j||_inf / (||A||_inf ||x_j||_inf + ||b_j||_inf) meets the
// tolerance.  When plain refinement stagnates (or gmres = 1), the correction equation is
// solved by GMRES preconditioned with the low-precision factors, in FP64 (GMRES-IR).
// A Cholesky breakdown in low precision is retried with a diagonal shift (A + s I, s a small
// multiple of the unit roundoff of the update precision times max a_ii); refinement still
// targets the unshifted A.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "host_state.hpp"

namespace palial {
cudaError_t mp_update(int mode, int upper, float *C, int n, int nb, int k, const void *a_hi, const void *a_lo,
                      const void *b_hi, const void *b_lo, const float *scale_a, const float *scale_b, int *status,
                      cudaStream_t s, int part = 0, int r0 = 0, int r1 = 0);
cudaError_t mp_pack_rows(int mode, const float *W, int n, int nb, int k, void *hi, void *lo, float *scales,
                         cudaStream_t s, int t0 = 0, int count = -1);
cudaError_t mp_pack_cols(int mode, const float *W, int n, int nb, int k, void *hi, void *lo, float *scales,
                         cudaStream_t s, int t0 = 0, int count = -1);
cudaError_t mps_f64_to_f32(const double *A, float *W, int n, int nb, double shift, cudaStream_t s,
                           double *amax = nullptr, bool upper_only = false, int r0 = 0, int r1 = -1);
cudaError_t mps_residual_df(const double *A, int n, int nb, const double *X, const double *colmax, const double *B,
                            double *R, int nrhs, int sigma, float2 *Xs, int *tau, double *amax, cudaStream_t s);
cudaError_t mps_residual_update(const double *A, int n, int nb, const double *D, const double *colmax, double *R,
                                int nrhs, int sigma, float *Ds, int *tau, cudaStream_t s);
cudaError_t mps_tile_to_f64(const float *w, double *d, int nb, cudaStream_t s);
cudaError_t mps_mirror_upper(double *A, int n, int nb, cudaStream_t s);
cudaError_t mps_tile_to_f32(const double *d, float *w, int nb, int upper_only, cudaStream_t s);
cudaError_t mps_panel_trsm(float *W, int n, int nb, int k, int kind, const float *binv, cudaStream_t s,
                           void *ph = nullptr, void *pl = nullptr, int t0 = 0, int count = -1, bool tc = false);
cudaError_t mps_block_inverse(const float *W, int n, int nb, int k, int factors, float *binv, cudaStream_t s,
                              int blocks = 0);
cudaError_t mps_residual(const double *A, int n, int nb, const double *X, const double *B, double *R, int nrhs,
                         double *amax, cudaStream_t s);
cudaError_t mps_norm_inf_matrix(const double *A, int n, int nb, double *out, cudaStream_t s);
cudaError_t mps_colmax(const double *X, long long n, int cols, double *out, cudaStream_t s);
cudaError_t mps_to_f32_rhs(const double *R, float *R32, long long n, int cols, const double *scale, cudaStream_t s);
cudaError_t mps_mark_step(int *status, int k, cudaStream_t s);
cudaError_t mpr_solve(const float *W, const float *Dinv, int n, int nb, int kind, float *R, float *Y, int *status,
                      cudaStream_t s);
cudaError_t rbt_prepare(int n, uint64_t seed);
cudaError_t rbt_transform_matrix(const double *A, float *W, int n, int nb, double *amax, cudaStream_t s);
cudaError_t rbt_transform_vectors(float *X, int n, int cols, int which, cudaStream_t s);
cudaError_t mpd_factor_tile(int alg, float *W, int n, int nb, int k, int *status, float *binv, cudaStream_t s);
cudaError_t mps_invert_diag(const float *W, int n, int nb, float *Dinv, int kind, cudaStream_t s);
cudaError_t mps_multi_dot(const double *V, int count, const double *w, long long n, int nrhs, double *H,
                          cudaStream_t s);
cudaError_t mps_multi_axpy(const double *V, int count, const double *H, double *w, long long n, int nrhs, int assign,
                           cudaStream_t s);
cudaError_t mps_scale_cols(const double *w, double *out, long long n, int nrhs, const double *f, cudaStream_t s);
cudaError_t mps_from_f32_rhs(double *X, const float *D32, long long n, int cols, const double *scale, cudaStream_t s);
cudaError_t mps_rank1(double *X, int n, int nb, const double *a, const double *b, cudaStream_t s);
cudaError_t mps_diag(double *X, int n, int nb, double kappa, cudaStream_t s);
cudaError_t mps_matvec(const double *A, int n, int nb, const double *x, double *y, int trans, cudaStream_t s);
cudaError_t mps_symmetrize(double *X, int n, int nb, cudaStream_t s);
cudaError_t launch_gen_dense(double *X, long long rows, int cols, uint64_t seed, int stream, cudaStream_t s);
cudaError_t launch_sumsq(const double *X, long long len, double *partial, int blocks, cudaStream_t s);
void mp_release();
int set_update_kernel(int kind);
int set_diag_kernel(int kind);
int set_update_reserve(int sms, int below_rows);
size_t mrd_scratch_bytes(int n);
cudaError_t mrd_residual(const double *A, int n, int nb, const double *X, const double *colmax, const double *B,
                         double *R, int nrhs, int sigma, void *scratch, double *amax, cudaStream_t s);
}  // namespace palial

using namespace palial;

namespace {

struct MpBufs {
    DevBuf w, diag, pa_hi, pa_lo, pb_hi, pb_lo, scales, r, r32, x32, norms, work, krylov, hbuf, gvec;
    DevBuf y32;     // output of the forward triangular solve (n x 16)
    DevBuf xsplit;  // compensated residual: X as FP32 pairs (n x 16 float2) + 16 scale exponents
    DevBuf binv;    // inverses of the current diagonal tile's 64 x 64 diagonal blocks (panel solves)
    DevBuf dinv_u, dinv_l, stile;  // FP32 inverses of the diagonal factor tiles, solve scratch
    DevBuf xdig;    // digit residual scratch (mrd_scratch_bytes): X's digits, exponents, integer sums
};
MpBufs mb;

// PALIAL_IR_TRACE=1 in the environment: one line per refinement step on stderr (diagnostics).
bool ir_trace() {
    static const bool on = [] {
        const char *v = std::getenv("PALIAL_IR_TRACE");
        return v && v[0] == '1';
    }();
    return on;
}

// PALIAL_FACTOR_TRACE=1: the device times at which the mixed factorization's three streams pass
// the marks of each step (ms from the start), one line per step on stderr after the
// factorization (diagnostics; timing events on every mark).
struct FactorTrace {
    enum { DIAG0, DIAG1, BINV, FIRST, PAIR, REST_PANEL, ROW0, ROW1, REST0, REST1, NMARK };
    bool on = false;
    cudaEvent_t t0 = nullptr;
    std::vector<cudaEvent_t> pool;
    std::vector<std::pair<int, int>> tags;  // (step, mark) of pool[i]
    size_t used = 0;
    cudaError_t begin(cudaStream_t s) {
        static const bool env = [] {
            const char *v = std::getenv("PALIAL_FACTOR_TRACE");
            return v && v[0] == '1';
        }();
        on = env;
        used = 0;
        tags.clear();
        if (!on) return cudaSuccess;
        cudaError_t e = t0 ? cudaSuccess : cudaEventCreate(&t0);
        return e == cudaSuccess ? cudaEventRecord(t0, s) : e;
    }
    cudaError_t mark(cudaStream_t q, int k, int m) {
        if (!on) return cudaSuccess;
        if (used == pool.size()) {
            pool.push_back(nullptr);
            const cudaError_t e = cudaEventCreate(&pool.back());
            if (e != cudaSuccess) return e;
        }
        tags.push_back({k, m});
        return cudaEventRecord(pool[used++], q);
    }
    void print(int mt) {
        if (!on) return;
        std::vector<float> t((size_t)mt * NMARK, -1.f);
        for (size_t i = 0; i < used; i++) {
            float ms = -1.f;
            if (cudaEventElapsedTime(&ms, t0, pool[i]) == cudaSuccess) t[(size_t)tags[i].first * NMARK + tags[i].second] = ms;
        }
        std::fprintf(stderr, "[factor] k: diag0 diag1 binv first pair | rest_panel row0 row1 | rest0 rest1 (ms)\n");
        for (int k = 0; k < mt; k++) {
            const float *r = &t[(size_t)k * NMARK];
            std::fprintf(stderr, "[factor] %d: %.3f %.3f %.3f %.3f %.3f | %.3f %.3f %.3f | %.3f %.3f\n", k, r[0], r[1], r[2],
                         r[3], r[4], r[5], r[6], r[7], r[8], r[9]);
        }
    }
} g_ftrace;

// opts.reserved[5] bit 3 of the running solve: the panels of a BF16x3 factorization in FP32 FMAs
// instead of BF16x3 on the tensor cores.
bool g_panel_fp32 = false;

// Update-kernel mode (mp_gemm.cu) of a PALIAL_PREC_* precision: 0 bf16, 1 fp8, 2 bf16x3, 3 tf32x3.
int update_mode(int prec) {
    return prec == PALIAL_PREC_FP8 ? 1 : prec == PALIAL_PREC_BF16X3 ? 2 : prec == PALIAL_PREC_TF32X3 ? 3 : 0;
}

double unit_roundoff(int prec) {
    switch (prec) {
        case PALIAL_PREC_BF16: return 0x1.0p-8;
        case PALIAL_PREC_FP8: return 0x1.0p-4;
        case PALIAL_PREC_BF16X3: return 0x1.0p-16;
        case PALIAL_PREC_TF32X3: return 0x1.0p-21;
        default: return 0x1.0p-24;
    }
}

// Low-precision factorization of W (FP32 tile layout, in place).  Returns PALIAL_OK,
// PALIAL_ERR_NOT_SPD (Cholesky breakdown) or an error.
// Lookahead on three streams.  The diagonal tile of step k+1 needs only tile (k+1, k+1) after
// step k, i.e. the first tile of panel k: so step k's critical chain (high priority) is the
// diagonal tile, its block inverses, the first panel tile and the update of tile (k+1, k+1);
// the rest of the panel and the rest of row (LU: and column) k+1 run beside it on a
// middle-priority stream, and the rest of the trailing update on a low-priority stream,
// overlapping the next steps.  Writers of one tile are ordered by events (the rest update of
// step k-1 before step k's updates of row k+1; row k+1 before step k+1's panel).  Packed panels
// and the diagonal blocks' inverses alternate between two buffers, so step k+1 never
// overwrites what step k's streams still read.
struct Lookahead {
    cudaStream_t hi = nullptr, mid = nullptr, lo = nullptr;
    cudaEvent_t start = nullptr, packed = nullptr, rest = nullptr, join = nullptr;
    cudaEvent_t binv = nullptr, first = nullptr, nextrow = nullptr, join_mid = nullptr;
} g_la;

// Host-buffer solves copy the tiles a Cholesky factorization reads (upper triangle) first
// and the rest on `copy` behind them; `full` marks the whole matrix resident.  g_full_ready
// is that event while such a solve runs (null otherwise): every reader of the full FP64
// matrix waits for it.
struct SplitCopy {
    cudaStream_t copy = nullptr;
    cudaEvent_t upper = nullptr, full = nullptr;
} g_sc;
cudaEvent_t g_full_ready = nullptr;

static cudaError_t wait_full_matrix(cudaStream_t s) {
    return g_full_ready ? cudaStreamWaitEvent(s, g_full_ready, 0) : cudaSuccess;
}

// Row-group arrival (host-buffer mixed Cholesky): the upper triangle arrives in groups of tile
// rows [gs[g], ge[g]) (FP32 working copy converted per group, event ready[g]); group 0 holds
// rows 0 and 1.  The factorization starts on group 0; the rest updates skip groups that have
// not joined.  From the step its data is due, a group catches up on the rest-update stream
// (the skipped steps in order, from packed panels kept for every step) within each step's
// estimated slack (the critical chain's time minus that step's rest update), and joins once
// caught up; at step kg[g] = gs[g] - 2 it must join (the rest update of that step covers its
// first row), so whatever is left is applied then.  Every tile receives the same updates in the
// same order as without deferral (bit-identical factors).  One-shot: mp_factor clears `on`.
struct RowArrival {
    bool on = false;
    int ngroups = 0;
    int gs[64], ge[64], kg[64];
    int due[64];  // step by which the group's data is expected (host link rate)
    cudaEvent_t ready[64] = {};
} g_arrival;

// The row groups of an n x n tile matrix (tile nb) for RowArrival: rows {0, 1}, single rows
// 2..7, then 2, 2, 4, 4, 8, 8, ... rows (the first rows are needed first; a row must be present
// two steps before the front reaches it).  due: the step by which the group's data is expected
// (host link ~200 GB/s, about 1.1 ms per step at NB = 512, scaled by (NB/512)^2); kg: the step by
// which it must join (gs - 2).  At most 64 groups.
static void row_groups(int n, int nb, int &ngroups, int *gs, int *ge, int *due, int *kg) {
    const int mt = n / nb;
    const double te = (double)nb * nb;
    const double step_s = 1.1e-3 * te / (512.0 * 512.0) * std::max(1.0, (double)mt / 64.0);
    double bytes = 0.0;
    ngroups = 0;
    for (int r = 0; r < mt && ngroups < 64;) {
        const int g = ngroups;
        const int size = g == 0 ? 2 : r < 8 ? 1 : 2 << ((g - 7) / 2);
        const int r1 = std::min(mt, g == 63 ? mt : r + size);
        for (int rr = r; rr < r1; rr++) bytes += 8.0 * te * (double)(mt - rr);
        gs[g] = r;
        ge[g] = r1;
        due[g] = (int)std::ceil(bytes / 200e9 / step_s);
        kg[g] = g == 0 ? 0 : std::max(0, r - 2);
        ngroups++;
        r = r1;
    }
}

// The rest-update stream's work per step under RowArrival, decided on the host: before step
// k's rest update the actions pre[k] (group, step sk: apply step sk to the group's rows;
// sk = -1: wait for the group's data), the rows [k + 2, present[k]) that rest update covers,
// then the catch-up actions post[k].  A group joins (is covered by the rest updates) once its
// data is due and it has steps 0..k-1, or at its deadline kg after the rest of them; catch-up
// within a step's slack (the critical chain's time minus the rest update, in tile-pair
// updates: about 0.8 ms per step, a BF16x3 pair update about 0.8 us at NB = 512, BF16 / FP8
// a third; a pair costs NB^3, the chain about NB^2).
struct ArrivalPlan {
    std::vector<std::vector<std::pair<int, int>>> pre, post;
    std::vector<int> present;
};
static ArrivalPlan plan_arrival(int mt, int nb, int mode, int ngroups, const int *gs, const int *ge, const int *due,
                                const int *kg) {
    ArrivalPlan pl;
    pl.pre.resize(mt);
    pl.post.resize(mt);
    pl.present.assign(mt, mt);
    int present = ge[0], next_group = 1;
    int applied[64] = {};
    bool waited[64] = {};
    const long long chain_pairs = (mode == 3 ? 500 : mode == 2 ? 1000 : 3000) * 512 / nb;
    const auto pairs_of = [&](int r0, int r1) {  // tile pairs (r, j >= r) of rows [r0, r1)
        long long c = 0;
        for (int r = r0; r < r1; r++) c += mt - r;
        return c;
    };
    for (int k = 0; k + 1 < mt; k++) {
        auto &pre = pl.pre[k], &post = pl.post[k];
        const auto apply = [&](std::vector<std::pair<int, int>> &to, int gi, int sk) {
            if (!waited[gi]) {
                to.emplace_back(gi, -1);
                waited[gi] = true;
            }
            to.emplace_back(gi, sk);
            applied[gi] = sk + 1;
        };
        while (next_group < ngroups && ((due[next_group] <= k && applied[next_group] >= k) || kg[next_group] <= k)) {
            for (int sk = applied[next_group]; sk < k; sk++) apply(pre, next_group, sk);
            if (!waited[next_group]) {
                pre.emplace_back(next_group, -1);
                waited[next_group] = true;
            }
            present = ge[next_group];
            next_group++;
        }
        pl.present[k] = present;
        long long budget = std::max(chain_pairs / 5, chain_pairs - pairs_of(k + 2, present));
        for (int gi = next_group; gi < ngroups && budget > 0 && due[gi] <= k; gi++) {
            const long long cost = pairs_of(gs[gi], ge[gi]);
            while (budget > 0 && applied[gi] <= k) {
                apply(post, gi, applied[gi]);
                budget -= cost;
            }
        }
    }
    return pl;
}

static cudaError_t lookahead_init() {
    if (g_la.hi) return cudaSuccess;
    int least = 0, greatest = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&g_la.hi, cudaStreamNonBlocking, greatest);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithPriority(&g_la.mid, cudaStreamNonBlocking, greatest < least ? greatest + 1 : greatest);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&g_la.lo, cudaStreamNonBlocking, least);
    for (cudaEvent_t *ev : {&g_la.start, &g_la.packed, &g_la.rest, &g_la.join, &g_la.binv, &g_la.first, &g_la.nextrow,
                            &g_la.join_mid})
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    return e;
}

int mp_factor(int alg, int prec, float *W, int n, int nb, cudaStream_t s, palial_status *st, int *zero_piv) {
    const int mt = n / nb;
    const int mode = update_mode(prec);
    const bool split = mode == 2 || mode == 3;  // hi + lo operand copies
    const size_t elem = (mode == 1) ? 1 : (mode == 3) ? 4 : 2;
    const size_t panel = (size_t)std::max(1, mt - 1) * nb * nb * elem;
    const bool arrive = g_arrival.on && alg == 0 && mt > 2;
    g_arrival.on = false;
    // packed panels: two alternating slots, or one per step when row groups arrive late
    const int slots = arrive ? mt - 1 : 2;
    PALIAL_CK(mb.pa_hi.ensure(slots * panel), "alloc panel");
    PALIAL_CK(mb.pb_hi.ensure(2 * panel), "alloc panel");
    if (split) {
        PALIAL_CK(mb.pa_lo.ensure(slots * panel), "alloc panel");
        PALIAL_CK(mb.pb_lo.ensure(2 * panel), "alloc panel");
    }
    PALIAL_CK(mb.scales.ensure(sizeof(float) * (size_t)std::max(4, slots * 2) * (size_t)std::max(1, mt)), "alloc scales");
    PALIAL_CK(mb.binv.ensure(sizeof(float) * 4 * (size_t)nb * 64), "alloc block inverses");  // two steps' worth
    PALIAL_CK(g.diag.status.ensure(sizeof(int) * ST_NSLOTS + 64), "alloc status");
    PALIAL_CK(lookahead_init(), "lookahead streams");
    PALIAL_CK(cudaMemsetAsync(g.diag.status.ptr, 0, sizeof(int) * ST_NSLOTS, s), "clear status");
    PALIAL_CK(cudaEventRecord(g_la.start, s), "event");
    PALIAL_CK(g_ftrace.begin(s), "trace");
    cudaStream_t hi = g_la.hi, mid = g_la.mid, lo = g_la.lo;
    PALIAL_CK(cudaStreamWaitEvent(hi, g_la.start, 0), "event");
    PALIAL_CK(cudaStreamWaitEvent(mid, g_la.start, 0), "event");
    PALIAL_CK(cudaStreamWaitEvent(lo, g_la.start, 0), "event");
    int *status = g.diag.status.as<int>();
    auto buf = [&](const DevBuf &b, int par) { return static_cast<void *>(static_cast<uint8_t *>(b.ptr) + par * panel); };
    if (arrive) {
        PALIAL_CK(cudaStreamWaitEvent(hi, g_arrival.ready[0], 0), "rows");
        PALIAL_CK(cudaStreamWaitEvent(mid, g_arrival.ready[0], 0), "rows");
        PALIAL_CK(cudaStreamWaitEvent(lo, g_arrival.ready[0], 0), "rows");
    }
    ArrivalPlan plan;
    if (arrive)
        plan = plan_arrival(mt, nb, mode, g_arrival.ngroups, g_arrival.gs, g_arrival.ge, g_arrival.due, g_arrival.kg);
    bool have_rest = false, have_next = false;
    // BF16 / BF16x3: the row-panel solve writes the packed operand with its results; FP8 needs
    // per-tile scales first and TF32x3 FP32 containers, so they pack in a separate pass
    const bool fused = mode == 0 || mode == 2;
    // BF16x3 updates: the panels' block products on the warp tensor cores in BF16x3 too
    // (opts.reserved[5] bit 3 keeps them in FP32)
    const bool panel_tc = mode == 2 && !g_panel_fp32;
    const int upper = alg == 0 ? 1 : 0;
    for (int k = 0; k < mt; k++) {
        float *binv = mb.binv.as<float>() + (size_t)(k & 1) * 2 * nb * 64;
        // the diagonal tile in FP32 (mp_diag.cu)
        PALIAL_CK(g_ftrace.mark(hi, k, FactorTrace::DIAG0), "trace");
        PALIAL_CK(mpd_factor_tile(alg, W, n, nb, k, status, binv, hi), "diag factor");
        PALIAL_CK(g_ftrace.mark(hi, k, FactorTrace::DIAG1), "trace");
        if (k == mt - 1) break;
        const int ntr = mt - k - 1;
        const int par = arrive ? k : (k & 1);
        float *sa = mb.scales.as<float>() + 2 * mt * par, *sb = sa + mt;
        void *ah = buf(mb.pa_hi, par), *al = split ? buf(mb.pa_lo, par) : nullptr;
        void *bh = buf(mb.pb_hi, k & 1), *bl = split ? buf(mb.pb_lo, k & 1) : nullptr;
        if (alg == 0) {
            bh = ah;
            bl = al;
            sb = sa;
        }
        PALIAL_CK(mps_block_inverse(W, n, nb, k, alg == 0 ? 1 : 2, binv, hi), "diagonal block inverses");
        PALIAL_CK(cudaEventRecord(g_la.binv, hi), "event");
        PALIAL_CK(g_ftrace.mark(hi, k, FactorTrace::BINV), "trace");
        // panel tiles [t0, t0 + cnt) on stream q, packed
        const auto panel_part = [&](cudaStream_t q, int t0, int cnt) -> int {
            if (alg == 0) {
                PALIAL_CK(mps_panel_trsm(W, n, nb, k, 0, binv, q, fused ? ah : nullptr, fused ? al : nullptr, t0, cnt,
                                         panel_tc),
                          "panel trsm");
                if (!fused) PALIAL_CK(mp_pack_rows(mode, W, n, nb, k, ah, al, sa, q, t0, cnt), "pack");
            } else {
                PALIAL_CK(mps_panel_trsm(W, n, nb, k, 1, binv, q, fused ? bh : nullptr, fused ? bl : nullptr, t0, cnt,
                                         panel_tc),
                          "row panel trsm");
                PALIAL_CK(mps_panel_trsm(W, n, nb, k, 2, binv, q, nullptr, nullptr, t0, cnt, panel_tc), "column panel trsm");
                PALIAL_CK(mp_pack_cols(mode, W, n, nb, k, ah, al, sa, q, t0, cnt), "pack L");
                if (!fused) PALIAL_CK(mp_pack_rows(mode, W, n, nb, k, bh, bl, sb, q, t0, cnt), "pack U");
            }
            return PALIAL_OK;
        };
        // critical chain: the first panel tile (row k+1's tile (k, k+1) was updated by step k-1's
        // row update), then tile (k+1, k+1) after step k-1's rest update
        if (have_next) PALIAL_CK(cudaStreamWaitEvent(hi, g_la.nextrow, 0), "event");
        int rc2 = panel_part(hi, 0, 1);
        if (rc2) return rc2;
        PALIAL_CK(cudaEventRecord(g_la.first, hi), "event");
        PALIAL_CK(g_ftrace.mark(hi, k, FactorTrace::FIRST), "trace");
        if (have_rest) PALIAL_CK(cudaStreamWaitEvent(hi, g_la.rest, 0), "event");
        PALIAL_CK(mp_update(mode, upper, W, n, nb, k, ah, al, bh, bl, sa, sb, status, hi, 4), "update (diagonal)");
        PALIAL_CK(g_ftrace.mark(hi, k, FactorTrace::PAIR), "trace");
        // beside it: the rest of the panel, then the rest of row (LU: and column) k+1
        PALIAL_CK(cudaStreamWaitEvent(mid, g_la.binv, 0), "event");
        if (ntr > 1) {
            rc2 = panel_part(mid, 1, -1);
            if (rc2) return rc2;
        }
        PALIAL_CK(g_ftrace.mark(mid, k, FactorTrace::REST_PANEL), "trace");
        PALIAL_CK(cudaStreamWaitEvent(mid, g_la.first, 0), "event");
        PALIAL_CK(cudaEventRecord(g_la.packed, mid), "event");  // the whole panel k is packed
        if (have_rest) PALIAL_CK(cudaStreamWaitEvent(mid, g_la.rest, 0), "event");
        PALIAL_CK(g_ftrace.mark(mid, k, FactorTrace::ROW0), "trace");
        if (ntr > 1) PALIAL_CK(mp_update(mode, upper, W, n, nb, k, ah, al, bh, bl, sa, sb, status, mid, 5), "update (next)");
        PALIAL_CK(cudaEventRecord(g_la.nextrow, mid), "event");
        PALIAL_CK(g_ftrace.mark(mid, k, FactorTrace::ROW1), "trace");
        have_next = true;
        // the rest of the trailing update
        PALIAL_CK(cudaStreamWaitEvent(lo, g_la.packed, 0), "event");
        PALIAL_CK(g_ftrace.mark(lo, k, FactorTrace::REST0), "trace");
        if (!arrive) {
            if (ntr > 1)
                PALIAL_CK(mp_update(mode, upper, W, n, nb, k, ah, al, bh, bl, sa, sb, status, lo, 2), "update (rest)");
        } else {
            RowArrival &ar = g_arrival;
            // the planned actions (plan_arrival): group gi's data, or its step sk update, on lo
            const auto run = [&](const std::vector<std::pair<int, int>> &acts) -> int {
                for (const auto &a : acts) {
                    const int gi = a.first, sk = a.second;
                    if (sk < 0) {
                        PALIAL_CK(cudaStreamWaitEvent(lo, ar.ready[gi], 0), "rows");
                        continue;
                    }
                    float *ss = mb.scales.as<float>() + 2 * mt * sk;
                    void *sh = buf(mb.pa_hi, sk), *sl = split ? buf(mb.pa_lo, sk) : nullptr;
                    PALIAL_CK(mp_update(mode, 1, W, n, nb, sk, sh, sl, sh, sl, ss, ss, status, lo, 3,
                                        ar.gs[gi] - sk - 1, ar.ge[gi] - sk - 1),
                              "update (arrived rows)");
                }
                return PALIAL_OK;
            };
            rc2 = run(plan.pre[k]);
            if (rc2) return rc2;
            const int present = plan.present[k];
            if (present - k - 1 > 1)
                PALIAL_CK(mp_update(mode, 1, W, n, nb, k, ah, al, bh, bl, sa, sb, status, lo, 3, 1, present - k - 1),
                          "update (rest)");
            // the next step's chain waits for the rows up to present only: the catch-up below
            // touches rows of groups that have not joined (at or past present)
            PALIAL_CK(cudaEventRecord(g_la.rest, lo), "event");
            rc2 = run(plan.post[k]);
            if (rc2) return rc2;
        }
        if (!arrive) PALIAL_CK(cudaEventRecord(g_la.rest, lo), "event");
        PALIAL_CK(g_ftrace.mark(lo, k, FactorTrace::REST1), "trace");
        have_rest = true;
    }
    PALIAL_CK(cudaEventRecord(g_la.join, lo), "event");
    PALIAL_CK(cudaEventRecord(g_la.join_mid, mid), "event");
    PALIAL_CK(cudaStreamWaitEvent(hi, g_la.join, 0), "event");
    PALIAL_CK(cudaStreamWaitEvent(hi, g_la.join_mid, 0), "event");
    PALIAL_CK(cudaEventRecord(g_la.join, hi), "event");
    PALIAL_CK(cudaStreamWaitEvent(s, g_la.join, 0), "event");
    int hs[ST_NSLOTS];
    PALIAL_CK(cudaMemcpyAsync(hs, g.diag.status.ptr, sizeof hs, cudaMemcpyDeviceToHost, s), "status");
    PALIAL_CK(cudaStreamSynchronize(s), "factorization");
    g_ftrace.print(mt);
    if (zero_piv) *zero_piv = hs[ST_ZEROPIV];
    if (hs[ST_CODE] == PALIAL_ERR_NOT_SPD) {
        if (st) {
            st->tile_m = st->tile_n = hs[6];
            st->column = hs[ST_COL];
        }
        return PALIAL_ERR_NOT_SPD;
    }
    if (hs[ST_CODE] != 0) return set_status(st, hs[ST_CODE], "device error %d in step %d", hs[ST_CODE], hs[6]);
    return PALIAL_OK;
}

// Inverses of the diagonal factor tiles (FP32), used by the refinement solves: one parallel
// launch per factor instead of a chain of single-CTA substitutions.
int mp_prepare_solves(int alg, const float *W, int n, int nb, cudaStream_t s, palial_status *st) {
    const size_t bytes = sizeof(float) * (size_t)n * nb;
    PALIAL_CK(mb.dinv_u.ensure(bytes), "alloc inverses");
    PALIAL_CK(mb.stile.ensure(sizeof(float) * (size_t)nb * 64), "alloc solve tile");
    PALIAL_CK(mps_invert_diag(W, n, nb, mb.dinv_u.as<float>(), 1, s), "invert U tiles");
    if (alg == 1) {
        PALIAL_CK(mb.dinv_l.ensure(bytes), "alloc inverses");
        PALIAL_CK(mps_invert_diag(W, n, nb, mb.dinv_l.as<float>(), 2, s), "invert L tiles");
    }
    return PALIAL_OK;
}

// State of the current solve shared by the refinement helpers: which residual steers, and
// whether the factors are those of the random-butterfly transform.
struct ResidCtx {
    bool df = false;
    bool digits = false;      // the full residuals on the tensor cores (mp_resid_digits.cu)
    int sigma = 0;
    bool rbt = false;         // the factors are those of U^T A V (random butterflies, LU)
    double *f64 = nullptr;    // FP64 factors (n x (n + nb) tile matrix): FP64 triangular solves
} g_rctx;

// d = M^-1 r for the FP32 factors in W; R32 (n x 16, zero padded) in/out.  Block forward and
// backward substitution over tile rows: the diagonal step multiplies by the stored inverse,
// the update step subtracts the solved tile row from the remaining ones.
int mp_apply_inverse(int alg, const float *W, int n, int nb, float *R32, cudaStream_t s, palial_status *st) {
    // forward into Y, backward back into R32: one persistent launch per direction (mp_rhs.cu)
    PALIAL_CK(mb.y32.ensure(sizeof(float) * (size_t)n * 16), "alloc solve output");
    float *Y = mb.y32.as<float>();
    const float *fwd_inv = (alg == 0) ? mb.dinv_u.as<float>() : mb.dinv_l.as<float>();
    int *status = g.diag.status.as<int>();
    PALIAL_CK(mpr_solve(W, fwd_inv, n, nb, alg == 0 ? 0 : 2, R32, Y, status, s), "forward solve");
    PALIAL_CK(mpr_solve(W, mb.dinv_u.as<float>(), n, nb, 1, Y, R32, status, s), "backward solve");
    return PALIAL_OK;
}

// z = M^-1 v for FP64 columns v (n x nrhs), through the FP32 factors (scaled per column).
int precondition(int alg, const float *W, int n, int nb, const double *v, double *z, int nrhs, double *dscale,
                 std::vector<double> &hscale, cudaStream_t s, palial_status *st) {
    if (g_rctx.f64) return fp64_trsolve(alg, g_rctx.f64, n, nb, v, z, nrhs, s, st);
    PALIAL_CK(mps_colmax(v, n, nrhs, dscale, s), "scale");
    PALIAL_CK(cudaMemcpyAsync(hscale.data(), dscale, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s), "scale");
    PALIAL_CK(cudaStreamSynchronize(s), "scale");
    for (int j = 0; j < nrhs; j++) {
        if (!std::isfinite(hscale[j])) return set_status(st, PALIAL_ERR_NOT_CONVERGED, "non-finite residual");
        if (hscale[j] == 0.0) hscale[j] = 1.0;
    }
    PALIAL_CK(cudaMemcpyAsync(dscale, hscale.data(), sizeof(double) * nrhs, cudaMemcpyHostToDevice, s), "scale");
    PALIAL_CK(mps_to_f32_rhs(v, mb.r32.as<float>(), n, nrhs, dscale, s), "to f32");
    if (g_rctx.rbt) PALIAL_CK(rbt_transform_vectors(mb.r32.as<float>(), n, 16, 0, s), "U^T r");
    int rc = mp_apply_inverse(alg, W, n, nb, mb.r32.as<float>(), s, st);
    if (rc) return rc;
    if (g_rctx.rbt) PALIAL_CK(rbt_transform_vectors(mb.r32.as<float>(), n, 16, 1, s), "V y");
    PALIAL_CK(mps_from_f32_rhs(z, mb.r32.as<float>(), n, nrhs, dscale, s), "from f32");
    return PALIAL_OK;
}

// The refinement's FP64-level full residual R = B - A X (B NULL: R = A X) in the solve's form:
// the digit residual on the tensor cores (default), or the compensated-FP32 one
// (opts.reserved[4] = 4).  colmax: per-column max |x|; amax_out (optional): ||A||_inf.
static cudaError_t df_residual(const double *A, int n, int nb, const double *X, const double *colmax, const double *B,
                               double *R, int nrhs, double *amax_out, cudaStream_t s) {
    if (g_rctx.digits) {
        return mrd_residual(A, n, nb, X, colmax, B, R, nrhs, g_rctx.sigma, mb.xdig.ptr, amax_out, s);
    }
    float2 *xs = mb.xsplit.as<float2>();
    return mps_residual_df(A, n, nb, X, colmax, B, R, nrhs, g_rctx.sigma, xs, reinterpret_cast<int *>(xs + (size_t)n * 16),
                           amax_out, s);
}

// A X products of the refinement (B - A X, or A X with B = NULL): the FP64-level residual of the
// current solve's form (df_residual), else FP64.
static cudaError_t apply_A(const double *A, int n, int nb, const double *X, const double *B, double *R, int nrhs,
                           cudaStream_t s) {
    if (!g_rctx.df) return mps_residual(A, n, nb, X, B, R, nrhs, nullptr, s);
    double *cm = mb.norms.as<double>() + 128;
    cudaError_t e = mps_colmax(X, n, nrhs, cm, s);
    if (e != cudaSuccess) return e;
    return df_residual(A, n, nb, X, cm, B, R, nrhs, nullptr, s);
}

// Flexible GMRES on A M^-1 y = r (right preconditioned, FP64 vectors, one Krylov space per
// right-hand side, classical Gram-Schmidt applied twice), restart length m, at most maxit
// iterations; a cycle stops when every column's residual ||r - A d||_2 has dropped by `rtol`.
// Right preconditioning minimises the true residual itself (left preconditioning minimises
// ||M^-1 (r - A d)||, which can grow the true residual when M^-1 is large, as with the
// low-precision factors of an ill-conditioned A).  The preconditioned vectors z_j = M^-1 v_j
// are kept and d = sum_j z_j y_j (flexible GMRES): M^-1 applied in FP32 is not linear in
// floating point, so applying it once more to sum_j v_j y_j would not give the vector whose
// residual the Arnoldi process minimised.  d is overwritten.  Returns PALIAL_OK and the
// iteration count in *iters.
int gmres(int alg, const double *A, const float *W, int n, int nb, const double *r, double *d, int nrhs, int m,
          int maxit, double rtol, cudaStream_t s, palial_status *st, int *iters) {
    const size_t blk = (size_t)n * nrhs;
    PALIAL_CK(mb.krylov.ensure(sizeof(double) * blk * (2 * m + 2)), "alloc krylov");
    PALIAL_CK(mb.hbuf.ensure(sizeof(double) * (size_t)(m + 2) * nrhs * 2), "alloc h");
    double *V = mb.krylov.as<double>();
    double *Z = V + blk * (m + 1);  // z_j = M^-1 v_j
    double *w = Z + blk * m;        // work vector after the bases
    double *dH = mb.hbuf.as<double>(), *dH2 = dH + (size_t)(m + 2) * nrhs;
    double *dscale = mb.norms.as<double>() + 96;
    std::vector<double> hs(nrhs), hh((size_t)(m + 2) * nrhs), hh2((size_t)(m + 2) * nrhs);
    PALIAL_CK(cudaMemsetAsync(d, 0, sizeof(double) * blk, s), "d0");
    int total = 0;
    bool done = false;
    while (!done && total < maxit) {
        // the cycle's residual r - A d (the first cycle: r)
        if (total == 0)
            PALIAL_CK(cudaMemcpyAsync(w, r, sizeof(double) * blk, cudaMemcpyDeviceToDevice, s), "r0");
        else
            PALIAL_CK(apply_A(A, n, nb, d, r, w, nrhs, s), "inner residual");
        // beta = ||r - A d||, V0 = (r - A d) / beta
        PALIAL_CK(mps_multi_dot(w, 1, w, n, nrhs, dH, s), "beta");
        PALIAL_CK(cudaMemcpyAsync(hh.data(), dH, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s), "beta");
        PALIAL_CK(cudaStreamSynchronize(s), "beta");
        std::vector<double> beta(nrhs);
        for (int c = 0; c < nrhs; c++) beta[c] = std::sqrt(hh[c]) > 0 ? std::sqrt(hh[c]) : 1.0;
        PALIAL_CK(cudaMemcpyAsync(dH, beta.data(), sizeof(double) * nrhs, cudaMemcpyHostToDevice, s), "beta");
        PALIAL_CK(mps_scale_cols(w, V, n, nrhs, dH, s), "v0");
        // Hessenberg, Givens rotations and rhs g per column (host)
        std::vector<std::vector<double>> H(nrhs, std::vector<double>((size_t)(m + 1) * m, 0.0));
        std::vector<std::vector<double>> cs(nrhs, std::vector<double>(m)), sn(nrhs, std::vector<double>(m));
        std::vector<std::vector<double>> gv(nrhs, std::vector<double>(m + 1, 0.0));
        for (int c = 0; c < nrhs; c++) gv[c][0] = beta[c];
        int j = 0;
        for (; j < m && total < maxit; j++, total++) {
            // z_j = M^-1 V_j, w = A z_j
            int rc = precondition(alg, W, n, nb, V + blk * j, Z + blk * j, nrhs, dscale, hs, s, st);
            if (rc) return rc;
            PALIAL_CK(apply_A(A, n, nb, Z + blk * j, nullptr, w, nrhs, s), "A z");
            // CGS twice: h = V^T w, w -= V h
            PALIAL_CK(mps_multi_dot(V, j + 1, w, n, nrhs, dH, s), "cgs");
            PALIAL_CK(mps_multi_axpy(V, j + 1, dH, w, n, nrhs, 0, s), "cgs");
            PALIAL_CK(mps_multi_dot(V, j + 1, w, n, nrhs, dH2, s), "cgs2");
            PALIAL_CK(mps_multi_axpy(V, j + 1, dH2, w, n, nrhs, 0, s), "cgs2");
            PALIAL_CK(mps_multi_dot(w, 1, w, n, nrhs, dH2 + (size_t)(j + 1) * nrhs, s), "norm");
            PALIAL_CK(cudaMemcpyAsync(hh.data(), dH, sizeof(double) * (j + 1) * nrhs, cudaMemcpyDeviceToHost, s), "h");
            PALIAL_CK(cudaMemcpyAsync(hh2.data(), dH2, sizeof(double) * (j + 2) * nrhs, cudaMemcpyDeviceToHost, s), "h");
            PALIAL_CK(cudaStreamSynchronize(s), "h");
            std::vector<double> hnext(nrhs);
            bool all_small = true;
            for (int c = 0; c < nrhs; c++) {
                double *Hc = H[c].data();
                for (int l = 0; l <= j; l++) Hc[(size_t)l * m + j] = hh[(size_t)l * nrhs + c] + hh2[(size_t)l * nrhs + c];
                const double hn = std::sqrt(std::max(0.0, hh2[(size_t)(j + 1) * nrhs + c]));
                Hc[(size_t)(j + 1) * m + j] = hn;
                hnext[c] = hn > 0 ? hn : 1.0;
                for (int l = 0; l < j; l++) {  // previous rotations
                    const double a = Hc[(size_t)l * m + j], b = Hc[(size_t)(l + 1) * m + j];
                    Hc[(size_t)l * m + j] = cs[c][l] * a + sn[c][l] * b;
                    Hc[(size_t)(l + 1) * m + j] = -sn[c][l] * a + cs[c][l] * b;
                }
                const double a = Hc[(size_t)j * m + j], b = Hc[(size_t)(j + 1) * m + j];
                const double rr = std::hypot(a, b);
                cs[c][j] = rr > 0 ? a / rr : 1.0;
                sn[c][j] = rr > 0 ? b / rr : 0.0;
                Hc[(size_t)j * m + j] = rr;
                Hc[(size_t)(j + 1) * m + j] = 0.0;
                gv[c][j + 1] = -sn[c][j] * gv[c][j];
                gv[c][j] = cs[c][j] * gv[c][j];
                if (std::fabs(gv[c][j + 1]) > rtol * beta[c]) all_small = false;
            }
            PALIAL_CK(cudaMemcpyAsync(dH2, hnext.data(), sizeof(double) * nrhs, cudaMemcpyHostToDevice, s), "hn");
            PALIAL_CK(mps_scale_cols(w, V + blk * (j + 1), n, nrhs, dH2, s), "v next");
            if (all_small) {
                j++;
                total++;
                done = true;
                break;
            }
        }
        // y = R^-1 g per column, d += Z y
        const int kdim = j;
        std::vector<double> ycoef((size_t)kdim * nrhs, 0.0);
        for (int c = 0; c < nrhs; c++) {
            const double *Hc = H[c].data();
            for (int l = kdim - 1; l >= 0; l--) {
                double v = gv[c][l];
                for (int q = l + 1; q < kdim; q++) v -= Hc[(size_t)l * m + q] * ycoef[(size_t)q * nrhs + c];
                ycoef[(size_t)l * nrhs + c] = Hc[(size_t)l * m + l] != 0 ? v / Hc[(size_t)l * m + l] : 0.0;
            }
        }
        if (kdim > 0) {
            PALIAL_CK(cudaMemcpyAsync(dH, ycoef.data(), sizeof(double) * kdim * nrhs, cudaMemcpyHostToDevice, s), "y");
            PALIAL_CK(mps_multi_axpy(Z, kdim, dH, w, n, nrhs, 1, s), "Z y");  // w = Z y
            std::vector<double> ones(nrhs, -1.0);
            PALIAL_CK(cudaMemcpyAsync(dH2, ones.data(), sizeof(double) * nrhs, cudaMemcpyHostToDevice, s), "one");
            PALIAL_CK(mps_multi_axpy(w, 1, dH2, d, n, nrhs, 0, s), "d += Z y");
        }
        PALIAL_CK(cudaStreamSynchronize(s), "gmres cycle");
    }
    if (iters) *iters = total;
    return PALIAL_OK;
}

}  // namespace

// Frees the mixed-precision path's device buffers (palial_gpu_finalize).
void palial::mp_release() {
    for (DevBuf *b : {&mb.w, &mb.diag, &mb.pa_hi, &mb.pa_lo, &mb.pb_hi, &mb.pb_lo, &mb.scales, &mb.r, &mb.r32,
                      &mb.x32, &mb.norms, &mb.work, &mb.krylov, &mb.hbuf, &mb.gvec, &mb.y32, &mb.xsplit, &mb.binv,
                      &mb.dinv_u, &mb.dinv_l, &mb.stile, &mb.xdig})
        b->release();
    // the streams and events belong to the context current when they were made: forget them
    // (the next solve makes new ones), so a later context on this device is not handed stale ones
    for (cudaStream_t *q : {&g_la.hi, &g_la.mid, &g_la.lo, &g_sc.copy}) {
        if (*q) cudaStreamDestroy(*q);
        *q = nullptr;
    }
    for (cudaEvent_t *ev : {&g_la.start, &g_la.packed, &g_la.rest, &g_la.join, &g_la.binv, &g_la.first, &g_la.nextrow,
                            &g_la.join_mid, &g_sc.upper, &g_sc.full, &g_ftrace.t0}) {
        if (*ev) cudaEventDestroy(*ev);
        *ev = nullptr;
    }
    for (cudaEvent_t &ev : g_arrival.ready) {
        if (ev) cudaEventDestroy(ev);
        ev = nullptr;
    }
    for (cudaEvent_t ev : g_ftrace.pool) cudaEventDestroy(ev);
    g_ftrace.pool.clear();
    g_ftrace.tags.clear();
    g_ftrace.used = 0;
    g_full_ready = nullptr;
}

extern "C" int palial_gpu_gen_kappa(double *dA, int n, int nb, double kappa, int symmetric, uint64_t seed,
                                    void *stream) {
    palial_status *st = nullptr;
    if (!dA || n <= 0 || nb <= 0 || n % nb || n % 64 || kappa < 1.0) return PALIAL_ERR_ARG;
    int rc = ensure_init(nullptr);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nref = 64;
    PALIAL_CK(mb.work.ensure(sizeof(double) * ((size_t)n * 2 * nref + (size_t)n + 1024)), "alloc");
    double *vecs = mb.work.as<double>();               // n x 128 reflector vectors
    double *y = vecs + (size_t)n * 2 * nref;            // n
    double *part = y + n;                               // 512 partial sums
    PALIAL_CK(launch_gen_dense(vecs, n, 2 * nref, seed, 3, s), "vectors");
    std::vector<double> hp(512), norms(2 * nref);
    for (int j = 0; j < 2 * nref; j++) {  // unit vectors: divide each by its 2-norm
        PALIAL_CK(launch_sumsq(vecs + (size_t)j * n, n, part, 512, s), "norm");
        PALIAL_CK(cudaMemcpyAsync(hp.data(), part, sizeof(double) * 512, cudaMemcpyDeviceToHost, s), "norm");
        PALIAL_CK(cudaStreamSynchronize(s), "norm");
        double t = 0;
        for (double x : hp) t += x;
        norms[j] = std::sqrt(t);
    }
    PALIAL_CK(cudaMemcpyAsync(part, norms.data(), sizeof(double) * 2 * nref, cudaMemcpyHostToDevice, s), "norms");
    for (int j = 0; j < 2 * nref; j++)
        PALIAL_CK(mps_scale_cols(vecs + (size_t)j * n, vecs + (size_t)j * n, n, 1, part + j, s), "normalize");
    PALIAL_CK(mps_diag(dA, n, nb, kappa, s), "diag");
    const double *U = vecs, *V = symmetric ? vecs : vecs + (size_t)n * nref;
    // X = D V^T = D G_64 ... G_1 (right), then A = U X = H_1 ... H_64 X (left)
    for (int j = nref - 1; j >= 0; j--) {
        const double *g = V + (size_t)j * n;
        PALIAL_CK(mps_matvec(dA, n, nb, g, y, 0, s), "X g");
        PALIAL_CK(mps_rank1(dA, n, nb, y, g, s), "X -= 2 (Xg) g^T");
    }
    for (int j = nref - 1; j >= 0; j--) {
        const double *h = U + (size_t)j * n;
        PALIAL_CK(mps_matvec(dA, n, nb, h, y, 1, s), "X^T h");
        PALIAL_CK(mps_rank1(dA, n, nb, h, y, s), "X -= 2 h (h^T X)");
    }
    if (symmetric) PALIAL_CK(mps_symmetrize(dA, n, nb, s), "symmetrize");
    PALIAL_CK(cudaStreamSynchronize(s), "gen kappa");
    return PALIAL_OK;
}

extern "C" int palial_gpu_set_update_kernel(int kind) {
    if (kind < 0 || kind > 2) return PALIAL_ERR_ARG;
    return palial::set_update_kernel(kind);
}

extern "C" int palial_gpu_f64_to_f32(const double *dA, float *dW, int n, int nb, int upper_only) {
    if (!dA || !dW || n <= 0 || nb <= 0 || n % nb || (nb * nb) % 2) return PALIAL_ERR_ARG;
    palial_status *st = nullptr;
    int rc = ensure_init(st);
    if (rc) return rc;
    PALIAL_CK(mps_f64_to_f32(dA, dW, n, nb, 0.0, nullptr, nullptr, upper_only != 0), "convert");
    PALIAL_CK(cudaStreamSynchronize(nullptr), "convert");
    return PALIAL_OK;
}

extern "C" int palial_gpu_set_diag_kernel(int kind) {
    if (kind < 0 || kind > 1) return PALIAL_ERR_ARG;
    return palial::set_diag_kernel(kind);
}

extern "C" int palial_gpu_set_update_reserve(int sms, int below_rows) {
    if (sms < 0 || sms > 64 || below_rows < 0) return PALIAL_ERR_ARG;
    return palial::set_update_reserve(sms, below_rows);
}

extern "C" int palial_gpu_mp_update_step(int alg, int precision, float *dW, int n, int nb, int k) {
    palial_status *st = nullptr;
    if ((alg != 0 && alg != 1) || !dW || n % nb || nb % 256 || k < 0 || k >= n / nb) return PALIAL_ERR_ARG;
    int rc = ensure_init(nullptr);
    if (rc) return rc;
    const int mt = n / nb;
    const int mode = update_mode(precision);
    const size_t panel = (size_t)std::max(1, mt - 1) * nb * nb * 4;
    PALIAL_CK(mb.pa_hi.ensure(panel), "alloc");
    PALIAL_CK(mb.pa_lo.ensure(panel), "alloc");
    PALIAL_CK(mb.pb_hi.ensure(panel), "alloc");
    PALIAL_CK(mb.pb_lo.ensure(panel), "alloc");
    PALIAL_CK(mb.scales.ensure(sizeof(float) * 2 * mt), "alloc");
    PALIAL_CK(g.diag.status.ensure(sizeof(int) * ST_NSLOTS + 64), "alloc");
    PALIAL_CK(cudaMemset(g.diag.status.ptr, 0, sizeof(int) * ST_NSLOTS), "clear");
    float *sa = mb.scales.as<float>(), *sb = sa + mt;
    if (alg == 0) {
        PALIAL_CK(mp_pack_rows(mode, dW, n, nb, k, mb.pa_hi.ptr, mb.pa_lo.ptr, sa, nullptr), "pack");
        PALIAL_CK(mp_update(mode, 1, dW, n, nb, k, mb.pa_hi.ptr, mb.pa_lo.ptr, mb.pa_hi.ptr, mb.pa_lo.ptr, sa, sa,
                            g.diag.status.as<int>(), nullptr),
                  "update");
    } else {
        PALIAL_CK(mp_pack_cols(mode, dW, n, nb, k, mb.pa_hi.ptr, mb.pa_lo.ptr, sa, nullptr), "pack");
        PALIAL_CK(mp_pack_rows(mode, dW, n, nb, k, mb.pb_hi.ptr, mb.pb_lo.ptr, sb, nullptr), "pack");
        PALIAL_CK(mp_update(mode, 0, dW, n, nb, k, mb.pa_hi.ptr, mb.pa_lo.ptr, mb.pb_hi.ptr, mb.pb_lo.ptr, sa, sb,
                            g.diag.status.as<int>(), nullptr),
                  "update");
    }
    PALIAL_CK(cudaDeviceSynchronize(), "update");
    int code = 0;
    PALIAL_CK(cudaMemcpy(&code, g.diag.status.ptr, sizeof code, cudaMemcpyDeviceToHost), "status");
    return code;
}

extern "C" int palial_gpu_mp_factor(int alg, const double *dA, float *dW, int n, int nb, const palial_opts *opts,
                                    palial_status *st, void *stream) {
    palial_opts o;
    palial_opts_default(&o);
    if (opts) o = *opts;
    if (st) memset(st, 0, sizeof *st);
    if ((alg != 0 && alg != 1) || !dA || !dW || n <= 0 || nb <= 0 || n % nb || nb % 256)
        return set_status(st, PALIAL_ERR_ARG, "mixed precision needs Cholesky/LU, N %% NB == 0, NB %% 256 == 0");
    int rc = ensure_init(st);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    PALIAL_CK(mps_f64_to_f32(dA, dW, n, nb, 0.0, s), "convert");
    const auto t0 = std::chrono::steady_clock::now();
    int zp = 0;
    g_panel_fp32 = (o.reserved[5] & 8) != 0;
    rc = mp_factor(alg, o.precision, dW, n, nb, s, st, &zp);
    if (st) st->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (rc) return set_status(st, rc, "mixed factorization failed");
    return set_status(st, zp ? PALIAL_WARN_ZERO_PIVOT : PALIAL_OK);
}

static int solve_one(int alg, const double *dA, int n, int nb, const double *dB, double *dX, int nrhs,
                     const palial_opts *opts, palial_status *st, void *stream) {
    palial_opts o;
    palial_opts_default(&o);
    if (opts) o = *opts;
    if (st) memset(st, 0, sizeof *st);
    if ((alg != 0 && alg != 1) || !dA || !dB || !dX || n <= 0 || nb <= 0 || n % nb || nb % 256 || nrhs < 1 ||
        nrhs > 16)
        return set_status(st, PALIAL_ERR_ARG, "solve_ir: Cholesky/LU, N %% NB == 0, NB %% 256 == 0, 1 <= nrhs <= 16");
    int rc = ensure_init(st);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const auto t0 = std::chrono::steady_clock::now();
    const size_t nn = (size_t)n * n;
    PALIAL_CK(mb.w.ensure(sizeof(float) * nn), "alloc W");
    PALIAL_CK(mb.r.ensure(sizeof(double) * (size_t)n * nrhs), "alloc r");
    PALIAL_CK(mb.r32.ensure(sizeof(float) * (size_t)n * 64), "alloc r32");
    PALIAL_CK(mb.norms.ensure(sizeof(double) * 256), "alloc norms");
    float *W = mb.w.as<float>();
    double *nrm = mb.norms.as<double>();  // [0] ||A||, [1..16] scale, [17..32] |r|, [33..48] |x|, [49..64] |b|
    // ||A||_inf and max |a_ii| (for the shift)
    // ||A||_inf comes with the first residual (same pass over A); a shifted retry of a
    // broken-down factorization computes it on its own
    double anorm = -1.0;
    const int prec = o.precision;
    // ---- factorization (FP64 path: plain FP64 scheduler, then the same FP32 solves) -------
    int zp = 0;
    double shift = 0.0;
    const auto f0 = std::chrono::steady_clock::now();
    if (prec == PALIAL_PREC_FP64) {
        g_rctx.rbt = false;
        PALIAL_CK(wait_full_matrix(s), "matrix copy");
        // the factors plus one tile column of right-hand-side workspace (FP64 triangular solves)
        PALIAL_CK(g.mat.ensure(sizeof(double) * (nn + (size_t)n * nb)), "alloc copy");
        PALIAL_CK(cudaMemcpyAsync(g.mat.ptr, dA, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s), "copy");
        palial_opts fo = o;
        palial_status fs;
        rc = palial_gpu_factor_dev(alg, g.mat.as<double>(), nullptr, n, nb, &fo, &fs, stream);
        if (rc < 0) {
            if (st) {
                *st = fs;
            }
            return rc;
        }
        g_rctx.f64 = g.mat.as<double>();
    } else {
        g_rctx.f64 = nullptr;
        // host-buffer Cholesky with row-group arrival: the copy pipeline converts the upper
        // triangle group by group (and accumulates max |a_ij|) while the factorization runs
        const bool arrived_conv = g_arrival.on && alg == 0;
        if (!arrived_conv) PALIAL_CK(cudaMemsetAsync(nrm + 120, 0, sizeof(double), s), "max |a|");
        // opts.reserved[6] = 1: LU of the random-butterfly transform U^T A V (rbt.cu)
        const bool rbt = alg == 1 && o.reserved[6] == 1;
        g_rctx.rbt = rbt;
        if (rbt) PALIAL_CK(rbt_prepare(n, o.reserved[7] ? (uint64_t)o.reserved[7] : 1ull), "butterflies");
        for (int attempt = 0; attempt < 4; attempt++) {
            if (rbt)
                PALIAL_CK(rbt_transform_matrix(dA, W, n, nb, attempt == 0 ? nrm + 120 : nullptr, s), "butterfly transform");
            else if (!(arrived_conv && attempt == 0))
                PALIAL_CK(mps_f64_to_f32(dA, W, n, nb, shift, s, attempt == 0 ? nrm + 120 : nullptr, alg == 0),
                          "convert");
            g_panel_fp32 = (o.reserved[5] & 8) != 0;
            rc = mp_factor(alg, prec, W, n, nb, s, st, &zp);
            // opts.reserved[5] bit 1: no shifted retry (a ladder rung hands a breakdown up)
            if (rc != PALIAL_ERR_NOT_SPD || alg != 0 || (o.reserved[5] & 2)) break;
            if (anorm < 0) {
                PALIAL_CK(wait_full_matrix(s), "matrix copy");
                PALIAL_CK(cudaMemsetAsync(nrm, 0, sizeof(double), s), "norm A");
                PALIAL_CK(mps_norm_inf_matrix(dA, n, nb, nrm, s), "norm A");
                PALIAL_CK(cudaMemcpyAsync(&anorm, nrm, sizeof(double), cudaMemcpyDeviceToHost, s), "norm");
                PALIAL_CK(cudaStreamSynchronize(s), "norm");
            }
            // Higham-Pranesh style shift: a small multiple of u_f * ||A||
            shift = (shift == 0.0) ? 4.0 * unit_roundoff(prec) * anorm / std::sqrt((double)n) : shift * 4.0;
        }
        if (rc) return set_status(st, rc, "mixed factorization failed (shift %.3e)", shift);
    }
    if (!g_rctx.f64) {  // FP32 inverses of the diagonal factor tiles for the FP32 solves
        rc = mp_prepare_solves(alg, W, n, nb, s, st);
        if (rc) return rc;
    }
    // The refinement steers with a compensated-FP32 residual (48-bit operands, error-free
    // products and sums, FP64 chunk accumulation; about 5x faster than the FP64 pipe) and
    // confirms convergence with the FP64 residual, so the reported error is an FP64 one.
    // opts.reserved[4] = 1 keeps every residual in FP64.
    double amax = 0.0;
    if (prec != PALIAL_PREC_FP64) PALIAL_CK(cudaMemcpyAsync(&amax, nrm + 120, sizeof(double), cudaMemcpyDeviceToHost, s), "max |a|");
    PALIAL_CK(cudaStreamSynchronize(s), "factorization");
    const bool use_df = prec != PALIAL_PREC_FP64 && o.reserved[4] != 1 && std::isfinite(amax) && amax > 0.0;
    int sigma = 0;
    if (use_df) {
        std::frexp(amax, &sigma);
        PALIAL_CK(mb.xsplit.ensure(sizeof(float2) * (size_t)n * 16 + 64), "alloc split x");
    }
    bool fp64_phase = false;
    constexpr double kDfConfirmBelow = 1e-11;
    g_rctx.df = use_df;
    g_rctx.digits = use_df && o.reserved[4] != 4 && n <= (1 << 18);
    if (g_rctx.digits) PALIAL_CK(mb.xdig.ensure(mrd_scratch_bytes(n)), "alloc digits");
    g_rctx.sigma = sigma;
    // status words of the refinement's solve launches (a timed-out wait is reported there)
    PALIAL_CK(g.diag.status.ensure(sizeof(int) * ST_NSLOTS + 64), "alloc status");
    PALIAL_CK(cudaMemsetAsync(g.diag.status.ptr, 0, sizeof(int) * ST_NSLOTS, s), "clear status");
    const double fsec = std::chrono::duration<double>(std::chrono::steady_clock::now() - f0).count();
    // ---- refinement -------------------------------------------------------------------------
    const double tol = o.ir_tol > 0 ? o.ir_tol : 1e-14 * n;
    const int maxit = o.ir_max_iter > 0 ? o.ir_max_iter : 50;
    std::vector<double> hb(nrhs), hr(nrhs), hx(nrhs), hd(nrhs), hscale(nrhs), drift(nrhs, 0.0);
    int resid_updates = 0;
    PALIAL_CK(wait_full_matrix(s), "matrix copy");  // the residuals read all of A
    PALIAL_CK(mps_colmax(dB, n, nrhs, nrm + 49, s), "norm b");
    PALIAL_CK(cudaMemcpyAsync(hb.data(), nrm + 49, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s), "norm b");
    PALIAL_CK(cudaMemsetAsync(dX, 0, sizeof(double) * (size_t)n * nrhs, s), "x0");
    PALIAL_CK(cudaMemcpyAsync(mb.r.ptr, dB, sizeof(double) * (size_t)n * nrhs, cudaMemcpyDeviceToDevice, s), "r0");
    PALIAL_CK(cudaStreamSynchronize(s), "init");
    double eta = 1.0, eta_prev = 1e300;
    int it = 0, gmres_total = 0, gmres_stalls = 0, last_inner = 0;
    bool converged = false;
    // GMRES-IR from the first step when the factorization needed a diagonal shift (A beyond the
    // factor precision's reach: plain refinement with the shifted factors stagnates)
    bool use_gmres = (o.gmres == 1) || (shift > 0.0 && o.gmres >= 0);
    PALIAL_CK(mb.x32.ensure(sizeof(double) * (size_t)n * nrhs), "alloc d");
    double *dcorr = mb.x32.as<double>();
    for (it = 1; it <= maxit; it++) {
        if (!use_gmres) {
            // d = M^-1 r in FP32 (scaled per column), x += d
            rc = precondition(alg, W, n, nb, mb.r.as<double>(), dcorr, nrhs, nrm + 1, hscale, s, st);
            if (rc) return rc;
        } else {
            int inner = 0;
            rc = gmres(alg, dA, W, n, nb, mb.r.as<double>(), dcorr, nrhs, 50, o.reserved[1] > 0 ? o.reserved[1] : 200,
                       1e-4, s, st, &inner);
            if (rc) return rc;
            gmres_total += inner;
            last_inner = inner;
            if (o.reserved[3] > 0 && gmres_total >= o.reserved[3]) {
                it++;
                break;  // GMRES budget of this attempt spent (precision ladder moves up)
            }
        }
        {
            std::vector<double> ones(nrhs, -1.0);
            PALIAL_CK(cudaMemcpyAsync(nrm + 80, ones.data(), sizeof(double) * nrhs, cudaMemcpyHostToDevice, s), "one");
            PALIAL_CK(mps_multi_axpy(dcorr, 1, nrm + 80, dX, n, nrhs, 0, s), "x += d");
        }
        PALIAL_CK(mps_colmax(dX, n, nrhs, nrm + 33, s), "norm x");
        const bool need_norm = anorm < 0;
        if (need_norm) PALIAL_CK(cudaMemsetAsync(nrm, 0, sizeof(double), s), "norm A");
        const bool used_df = use_df && !fp64_phase;
        // Update form r <- r - A d for a small correction: FP32 products, error <= 2^-17 |A| |d|
        // per entry, so at most 2^-17 ||d_j|| / ||x_j|| on column j's backward error; one
        // HBM-bound pass over A instead of the issue-bound compensated residual.  drift[j]
        // sums these bounds since the last full residual and convergence needs eta_j +
        // drift_j <= tol.  Used while a step adds at most tol / 4; the first residual (d = x)
        // is always full; opts.reserved[4] = 3 disables the form.
        bool update_form = false;
        if (used_df && !need_norm && o.reserved[4] != 3) {
            PALIAL_CK(mps_colmax(dcorr, n, nrhs, nrm + 176, s), "norm d");
            PALIAL_CK(cudaMemcpyAsync(hd.data(), nrm + 176, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s), "norm d");
            PALIAL_CK(cudaMemcpyAsync(hx.data(), nrm + 33, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s), "norm x");
            PALIAL_CK(cudaStreamSynchronize(s), "norm d");
            update_form = true;
            for (int j = 0; j < nrhs; j++) {
                const double step = std::ldexp(hd[j], -17) / hx[j];
                update_form = update_form && std::isfinite(step) && step <= tol / 4.0;
            }
        }
        const auto full_residual = [&](double *anorm_out) -> int {
            if (used_df) {
                PALIAL_CK(df_residual(dA, n, nb, dX, nrm + 33, dB, mb.r.as<double>(), nrhs, anorm_out, s),
                          "residual (digits / compensated FP32)");
            } else {
                PALIAL_CK(mps_residual(dA, n, nb, dX, dB, mb.r.as<double>(), nrhs, anorm_out, s), "residual");
            }
            std::fill(drift.begin(), drift.end(), 0.0);
            return PALIAL_OK;
        };
        if (update_form) {
            float2 *xs = mb.xsplit.as<float2>();
            PALIAL_CK(mps_residual_update(dA, n, nb, dcorr, nrm + 176, mb.r.as<double>(), nrhs, sigma,
                                          reinterpret_cast<float *>(xs), reinterpret_cast<int *>(xs + (size_t)n * 16), s),
                      "residual (update form)");
            resid_updates++;
            for (int j = 0; j < nrhs; j++) drift[j] += std::ldexp(hd[j], -17) / hx[j];
        } else {
            rc = full_residual(need_norm ? nrm : nullptr);
            if (rc) return rc;
        }
        if (need_norm) PALIAL_CK(cudaMemcpyAsync(&anorm, nrm, sizeof(double), cudaMemcpyDeviceToHost, s), "norm A");
        PALIAL_CK(mps_colmax(mb.r.as<double>(), n, nrhs, nrm + 17, s), "norm r");
        PALIAL_CK(cudaMemcpyAsync(hr.data(), nrm + 17, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s), "norm r");
        PALIAL_CK(cudaMemcpyAsync(hx.data(), nrm + 33, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s), "norm x");
        PALIAL_CK(cudaStreamSynchronize(s), "iteration");
        eta = 0.0;
        double eta_bound = 0.0;
        bool finite = true;
        for (int j = 0; j < nrhs; j++) {
            finite = finite && std::isfinite(hr[j]) && std::isfinite(hx[j]);
            const double ej = hr[j] / (anorm * hx[j] + hb[j]);
            eta = std::max(eta, ej);
            eta_bound = std::max(eta_bound, ej + drift[j]);
        }
        if (!finite || !std::isfinite(eta)) {
            eta = INFINITY;
            break;
        }
        if (eta <= tol && eta_bound > tol) {
            // the update form's drift leaves the decision open: recompute the residual in full
            rc = full_residual(nullptr);
            if (rc) return rc;
            PALIAL_CK(mps_colmax(mb.r.as<double>(), n, nrhs, nrm + 17, s), "norm r");
            PALIAL_CK(cudaMemcpyAsync(hr.data(), nrm + 17, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s), "norm r");
            PALIAL_CK(cudaStreamSynchronize(s), "full residual");
            eta = 0.0;
            for (int j = 0; j < nrhs; j++) {
                finite = finite && std::isfinite(hr[j]);
                eta = std::max(eta, hr[j] / (anorm * hx[j] + hb[j]));
            }
            if (!finite || !std::isfinite(eta)) {
                eta = INFINITY;
                break;
            }
        }
        // The compensated residual's error is below 1e-12 of the backward error's scale
        // (tested); a tolerance 10x above that needs no FP64 confirmation.
        if (eta <= tol && used_df && (tol < kDfConfirmBelow || o.reserved[4] == 2)) {
            // confirm with the FP64 residual; if the compensated residual's floor misled, go on in FP64
            PALIAL_CK(mps_residual(dA, n, nb, dX, dB, mb.r.as<double>(), nrhs, nullptr, s), "residual");
            PALIAL_CK(mps_colmax(mb.r.as<double>(), n, nrhs, nrm + 17, s), "norm r");
            PALIAL_CK(cudaMemcpyAsync(hr.data(), nrm + 17, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s), "norm r");
            PALIAL_CK(cudaStreamSynchronize(s), "confirmation");
            eta = 0.0;
            for (int j = 0; j < nrhs; j++) {
                finite = finite && std::isfinite(hr[j]);
                eta = std::max(eta, hr[j] / (anorm * hx[j] + hb[j]));
            }
            if (!finite || !std::isfinite(eta)) {
                eta = INFINITY;
                break;
            }
            fp64_phase = true;
        }
        if (ir_trace())
            std::fprintf(stderr, "palial ir: alg %d prec %d step %d eta %.3e gmres %d (+%d) %s\n", alg, prec, it, eta,
                         gmres_total, use_gmres ? last_inner : 0, update_form ? "update-form" : "full");
        if (eta <= tol) {
            converged = true;
            break;
        }
        if ((o.reserved[5] & 1) && it >= 2 && eta > 0.1 * eta_prev) {
            break;  // a lower rung of the precision ladder that contracts slowly: move up
        }
        if (!use_gmres && it >= 2 && eta > 0.5 * eta_prev && o.gmres >= 0) {
            use_gmres = true;  // plain refinement contracts too slowly: switch to GMRES-IR
            gmres_stalls = 0;
        } else if (use_gmres && it >= 2) {
            // GMRES-IR gets two outer steps that gain less than 10 % before it is given up:
            // a GMRES cycle that met its inner tolerance may still leave the true residual
            // above it when the preconditioner is poor, and the next cycle starts from there
            gmres_stalls = eta > 0.9 * eta_prev ? gmres_stalls + 1 : 0;
            if (gmres_stalls >= 2) break;
            // a GMRES step that doubles the error: the factors are no preconditioner for this A
            if (eta > 2.0 * eta_prev) break;
            // within a GMRES budget (opts.reserved[3]): give up as soon as the contraction of
            // this step, continued, would need more GMRES iterations than are left
            if (o.reserved[3] > 0 && eta < eta_prev && last_inner > 0) {
                const double steps = std::ceil(std::log(tol / eta) / std::log(eta / eta_prev));
                if (steps * last_inner > (double)(o.reserved[3] - gmres_total)) break;
            }
        } else if (!use_gmres && o.gmres < 0 && it >= 3 && eta > 0.9 * eta_prev) {
            break;
        }
        eta_prev = std::min(eta_prev, eta);
    }
    {
        int code = 0;
        PALIAL_CK(cudaMemcpy(&code, g.diag.status.ptr, sizeof code, cudaMemcpyDeviceToHost), "solve status");
        if (code) return set_status(st, code, "refinement solve: device error %d", code);
    }
    const double total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (st) {
        st->ir_iters = std::min(it, maxit);
        st->backward_error = eta;
        st->seconds = total;
        st->total_seconds = total;
        st->tflops = algorithmic_flops(alg, n) / total * 1e-12;
        st->kappa_est = -1.0;
        st->factor_seconds = fsec;
        st->shift = shift;
        st->gmres_iters = gmres_total;
    }
    if (!converged)
        return set_status(st, PALIAL_ERR_NOT_CONVERGED, "refinement stopped at backward error %.3e after %d iterations",
                          eta, it);
    return set_status(st, zp ? PALIAL_WARN_ZERO_PIVOT : PALIAL_OK,
                      "backward error %.3e in %d iterations (shift %.2e, %d update-form residuals)", eta,
                      st ? st->ir_iters : it, shift, resid_updates);
}

// Precision ladder (PALIAL_PREC_AUTO): BF16x3 updates first (about 2^-16 per product, the
// fastest rung on well-conditioned systems), then TF32x3 (FP32-level factors, about 2^-21),
// then the FP64 factorization.  A rung that misses the target within its budget (refinement
// steps and GMRES iterations) hands over to the next; the status reports the rung that
// produced the result (precision_used) and the total time of all attempts.
extern "C" int palial_gpu_solve_ir(int alg, const double *dA, int n, int nb, const double *dB, double *dX, int nrhs,
                                   const palial_opts *opts, palial_status *st, void *stream) {
    palial_opts o;
    palial_opts_default(&o);
    if (opts) o = *opts;
    if (o.precision != PALIAL_PREC_AUTO) {
        const int rc = solve_one(alg, dA, n, nb, dB, dX, nrhs, &o, st, stream);
        if (st) st->precision_used = o.precision + (alg == 1 && o.reserved[6] == 1 && o.precision != PALIAL_PREC_FP64 ? 100 : 0);
        return rc;
    }
    static const int ladder[] = {PALIAL_PREC_BF16X3, PALIAL_PREC_TF32X3, PALIAL_PREC_FP64};
    const auto t0 = std::chrono::steady_clock::now();
    int rc = PALIAL_ERR_NOT_CONVERGED;
    int used = -1;
    for (int li = 0; li < 3; li++) {
        const int prec = ladder[li];
        palial_opts oo = o;
        oo.precision = prec;
        // lower rungs get a bounded effort.  BF16x3: at most 10 refinement steps and 36 GMRES
        // iterations in all (a GMRES iteration, a full residual and two triangular solves,
        // costs about a twelfth of a factorization: the budget lets a system that a BF16x3
        // preconditioner handles in a few cycles finish, and one that projects past it moves
        // up early), and a Cholesky breakdown (a matrix beyond BF16x3's reach) goes up at once
        // instead of being retried with a shift.  TF32x3: 20 steps, restarts of 200, 600
        // iterations in all.
        if (prec == PALIAL_PREC_BF16X3) {
            if (oo.ir_max_iter <= 0 || oo.ir_max_iter > 10) oo.ir_max_iter = 10;
            oo.reserved[1] = 36;
            oo.reserved[3] = 36;
            oo.reserved[5] |= 2;
        } else if (prec == PALIAL_PREC_TF32X3) {
            if (oo.ir_max_iter <= 0 || oo.ir_max_iter > 20) oo.ir_max_iter = 20;
            oo.reserved[1] = 200;
            oo.reserved[3] = 600;
        }
        rc = solve_one(alg, dA, n, nb, dB, dX, nrhs, &oo, st, stream);
        used = prec + (alg == 1 && oo.reserved[6] == 1 && prec != PALIAL_PREC_FP64 ? 100 : 0);
        if (rc >= 0) break;
        if (rc != PALIAL_ERR_NOT_CONVERGED && rc != PALIAL_ERR_NOT_SPD) break;
    }
    const double total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (st) {
        st->seconds = st->total_seconds = total;
        st->tflops = algorithmic_flops(alg, n) / total * 1e-12;
        st->precision_used = used;
    }
    return rc;
}

// R = B - A X on device buffers (B may be NULL: R = A X), FP64 (mode 0) or compensated FP32
// (mode 1, the refinement's steering residual); nrhs <= 16.
extern "C" int palial_gpu_residual(const double *dA, int n, int nb, const double *dX, const double *dB, double *dR,
                                   int nrhs, int mode, void *stream) {
    if (!dA || !dX || !dR || n <= 0 || nb <= 0 || n % nb || n % 64 || nrhs < 1 || nrhs > 16 || mode < 0 || mode > 3)
        return PALIAL_ERR_ARG;
    if (mode == 2 && dB) return PALIAL_ERR_ARG;  // update form: R <- R - A X in place
    palial_status st0;
    palial_status *st = &st0;
    int rc = ensure_init(st);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (mode == 0) {
        PALIAL_CK(mps_residual(dA, n, nb, dX, dB, dR, nrhs, nullptr, s), "residual");
        return PALIAL_OK;
    }
    PALIAL_CK(mb.norms.ensure(sizeof(double) * 128), "alloc norms");
    PALIAL_CK(mb.xsplit.ensure(sizeof(float2) * (size_t)n * 16 + 64), "alloc split x");
    double *nrm = mb.norms.as<double>();
    PALIAL_CK(cudaMemsetAsync(nrm + 120, 0, sizeof(double), s), "max |a|");
    PALIAL_CK(mb.w.ensure(sizeof(float) * (size_t)n * n), "alloc W");
    PALIAL_CK(mps_f64_to_f32(dA, mb.w.as<float>(), n, nb, 0.0, s, nrm + 120), "max |a|");
    double amax = 0;
    PALIAL_CK(cudaMemcpyAsync(&amax, nrm + 120, sizeof(double), cudaMemcpyDeviceToHost, s), "max |a|");
    PALIAL_CK(cudaStreamSynchronize(s), "max |a|");
    int sigma = 0;
    std::frexp(amax, &sigma);
    PALIAL_CK(mps_colmax(dX, n, nrhs, nrm + 33, s), "norm x");
    float2 *xs = mb.xsplit.as<float2>();
    if (mode == 3) {
        PALIAL_CK(mb.xdig.ensure(mrd_scratch_bytes(n)), "alloc digits");
        PALIAL_CK(mrd_residual(dA, n, nb, dX, nrm + 33, dB, dR, nrhs, sigma, mb.xdig.ptr, nullptr, s), "residual (digits)");
        return PALIAL_OK;
    }
    if (mode == 2) {
        PALIAL_CK(mps_residual_update(dA, n, nb, dX, nrm + 33, dR, nrhs, sigma, reinterpret_cast<float *>(xs),
                                      reinterpret_cast<int *>(xs + (size_t)n * 16), s),
                  "residual (update form)");
        return PALIAL_OK;
    }
    PALIAL_CK(mps_residual_df(dA, n, nb, dX, nrm + 33, dB, dR, nrhs, sigma, xs, reinterpret_cast<int *>(xs + (size_t)n * 16),
                              nullptr, s),
              "residual");
    return PALIAL_OK;
}

// Host-buffer variant (A: reference tile descriptor in host memory; B, X: n x nrhs host,
// column-major): copies in, solves, copies X out.
static int solve_ir_host_impl(int alg, const palial_desc *A, const double *B, double *X, int nrhs,
                              const palial_opts *opts, palial_status *st) {
    if (st) memset(st, 0, sizeof *st);
    if (!A || !A->matrix || !B || !X || nrhs < 1 || nrhs > 16) return set_status(st, PALIAL_ERR_ARG, "bad arguments");
    const int n = A->matrix_size, nb = A->tile_size;
    int rc = ensure_init(st);
    if (rc) return rc;
    const auto t0 = std::chrono::steady_clock::now();
    const size_t bytes = sizeof(double) * (size_t)n * n, vb = sizeof(double) * (size_t)n * nrhs;
    PALIAL_CK(g.smat.ensure(bytes), "alloc A");
    PALIAL_CK(mb.work.ensure(std::max(mb.work.bytes, 2 * vb)), "alloc B/X");
    double *dB = mb.work.as<double>(), *dX = dB + (size_t)n * nrhs;
    PALIAL_CK(cudaMemcpyAsync(dB, B, vb, cudaMemcpyHostToDevice, nullptr), "copy B");
    const int mt = nb > 0 ? n / nb : 0;
    const size_t te = (size_t)nb * nb;
    double *dA = g.smat.as<double>();
    const double *hA = static_cast<const double *>(A->matrix);
    palial_opts oo;
    palial_opts_default(&oo);
    if (opts) oo = *opts;
    const bool mixed = oo.precision != PALIAL_PREC_FP64;
    if (alg == 0 && mt > 2 && n % nb == 0 && nb % 256 == 0 && mixed && oo.reserved[4] != 1) {
        // Cholesky reads only the upper triangle (the reference's dpotrf / dtrsm / dsyrk calls
        // take 'U'), and only the upper triangle crosses the host link: it arrives in groups of
        // tile rows (row r's tiles (r, j >= r): one strided copy), each converted to the FP32
        // working copy on the copy stream, and the factorization starts on the first group
        // (RowArrival).  The residuals read the symmetric matrix the upper triangle defines: its
        // lower triangle is written on the device from the upper one (one HBM pass behind the
        // last group), as a solver given uplo = 'U' treats A.  The host link is the bottleneck,
        // so the copies run back to back on one stream.
        if (!g_sc.copy) {
            PALIAL_CK(cudaStreamCreateWithFlags(&g_sc.copy, cudaStreamNonBlocking), "copy stream");
            PALIAL_CK(cudaEventCreateWithFlags(&g_sc.upper, cudaEventDisableTiming), "copy event");
            PALIAL_CK(cudaEventCreateWithFlags(&g_sc.full, cudaEventDisableTiming), "copy event");
        }
        PALIAL_CK(mb.w.ensure(sizeof(float) * (size_t)n * n), "alloc W");
        PALIAL_CK(mb.norms.ensure(sizeof(double) * 256), "alloc norms");
        double *amax = mb.norms.as<double>() + 120;
        PALIAL_CK(cudaMemsetAsync(amax, 0, sizeof(double), g_sc.copy), "max |a|");
        RowArrival &ar = g_arrival;
        row_groups(n, nb, ar.ngroups, ar.gs, ar.ge, ar.due, ar.kg);
        for (int g = 0; g < ar.ngroups; g++) {
            if (!ar.ready[g]) PALIAL_CK(cudaEventCreateWithFlags(&ar.ready[g], cudaEventDisableTiming), "copy event");
            for (int rr = ar.gs[g]; rr < ar.ge[g]; rr++)
                PALIAL_CK(cudaMemcpy2DAsync(dA + te * ((size_t)rr + (size_t)mt * rr), sizeof(double) * te * mt,
                                            hA + te * ((size_t)rr + (size_t)mt * rr), sizeof(double) * te * mt,
                                            sizeof(double) * te, (size_t)(mt - rr), cudaMemcpyHostToDevice, g_sc.copy),
                          "copy A (row)");
            PALIAL_CK(mps_f64_to_f32(dA, mb.w.as<float>(), n, nb, 0.0, g_sc.copy, amax, true, ar.gs[g], ar.ge[g]),
                      "convert rows");
            PALIAL_CK(cudaEventRecord(ar.ready[g], g_sc.copy), "copy event");
        }
        ar.on = true;
        PALIAL_CK(cudaEventRecord(g_sc.upper, g_sc.copy), "copy A");
        PALIAL_CK(mps_mirror_upper(dA, n, nb, g_sc.copy), "lower triangle");
        PALIAL_CK(cudaEventRecord(g_sc.full, g_sc.copy), "copy A");
        g_full_ready = g_sc.full;
    } else if (alg == 0 && mt > 1 && n % nb == 0) {
        // FP64 Cholesky: the upper triangle (tile column j's tiles 0..j are contiguous), the
        // lower triangle written from it on the device (copied, for tiles not a multiple of 32)
        if (!g_sc.copy) {
            PALIAL_CK(cudaStreamCreateWithFlags(&g_sc.copy, cudaStreamNonBlocking), "copy stream");
            PALIAL_CK(cudaEventCreateWithFlags(&g_sc.upper, cudaEventDisableTiming), "copy event");
            PALIAL_CK(cudaEventCreateWithFlags(&g_sc.full, cudaEventDisableTiming), "copy event");
        }
        for (int j = 0; j < mt; j++)
            PALIAL_CK(cudaMemcpyAsync(dA + te * mt * j, hA + te * mt * j, sizeof(double) * te * (j + 1),
                                      cudaMemcpyHostToDevice, nullptr),
                      "copy A (upper)");
        PALIAL_CK(cudaEventRecord(g_sc.upper, nullptr), "copy A");
        PALIAL_CK(cudaStreamWaitEvent(g_sc.copy, g_sc.upper, 0), "copy A");
        if (nb % 32 == 0)
            PALIAL_CK(mps_mirror_upper(dA, n, nb, g_sc.copy), "lower triangle");
        else
            for (int j = 0; j + 1 < mt; j++)
                PALIAL_CK(cudaMemcpyAsync(dA + te * (mt * j + j + 1), hA + te * (mt * j + j + 1),
                                          sizeof(double) * te * (mt - 1 - j), cudaMemcpyHostToDevice, g_sc.copy),
                          "copy A (lower)");
        PALIAL_CK(cudaEventRecord(g_sc.full, g_sc.copy), "copy A");
        g_full_ready = g_sc.full;
    } else {
        PALIAL_CK(cudaMemcpyAsync(dA, hA, bytes, cudaMemcpyHostToDevice, nullptr), "copy A");
    }
    rc = palial_gpu_solve_ir(alg, dA, n, nb, dB, dX, nrhs, opts, st, nullptr);
    g_arrival.on = false;
    g_full_ready = nullptr;
    if (g_sc.full) PALIAL_CK(cudaStreamWaitEvent(nullptr, g_sc.full, 0), "copy A");  // error paths too
    PALIAL_CK(cudaMemcpy(X, dX, vb, cudaMemcpyDeviceToHost), "copy X");
    if (st) st->total_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

// Whatever path returns, no copy of the caller's host buffers is left in flight (the caller may
// free them as soon as the call returns).
extern "C" int palial_gpu_solve_ir_host(int alg, const palial_desc *A, const double *B, double *X, int nrhs,
                                        const palial_opts *opts, palial_status *st) {
    const int rc = solve_ir_host_impl(alg, A, B, X, nrhs, opts, st);
    g_arrival.on = false;
    g_full_ready = nullptr;
    if (g_sc.copy) cudaStreamSynchronize(g_sc.copy);
    cudaStreamSynchronize(nullptr);
    return rc;
}

// ---- introspection of the host-side schedules (host only, no GPU) -----------------------------
extern "C" int palial_gpu_row_groups(int n, int nb, int *gs, int *ge, int *due, int *kg, int max_groups) {
    if (n <= 0 || nb <= 0 || n % nb || !gs || !ge || !due || !kg || max_groups < 64) return PALIAL_ERR_ARG;
    int ng = 0;
    row_groups(n, nb, ng, gs, ge, due, kg);
    return ng;
}

// Checks the arrival plan for an n x n tile matrix (tile nb) and update mode: each group's data
// is awaited before its first update, it receives steps 0..j-1 in order exactly once before it
// joins at step j <= gs - 2, no update uses a panel not yet produced, and every rest update
// covers the row the next step's first update needs.  0, or a positive code naming the
// failed property.  Host only.
extern "C" int palial_gpu_check_arrival_plan(int n, int nb, int mode) {
    if (n <= 0 || nb <= 0 || n % nb || mode < 0 || mode > 3) return -1;
    const int mt = n / nb;
    if (mt <= 2) return 0;
    int ng = 0, gs[64], ge[64], due[64], kg[64];
    row_groups(n, nb, ng, gs, ge, due, kg);
    const ArrivalPlan pl = plan_arrival(mt, nb, mode, ng, gs, ge, due, kg);
    std::vector<int> applied(ng, 0), joined(ng, -1);
    std::vector<char> waited(ng, 0);
    joined[0] = 0;
    waited[0] = 1;
    int present = ge[0];
    for (int k = 0; k + 1 < mt; k++) {
        for (int half = 0; half < 2; half++) {
            for (const auto &a : half ? pl.post[k] : pl.pre[k]) {
                const int gi = a.first, sk = a.second;
                if (gi <= 0 || gi >= ng || joined[gi] >= 0) return 1;  // only groups not joined
                if (sk < 0) {
                    if (waited[gi]) return 2;  // one wait per group
                    waited[gi] = 1;
                    continue;
                }
                if (!waited[gi]) return 3;               // data before the first update
                if (sk != applied[gi] || sk > k) return 4;  // steps in order, panels exist
                applied[gi]++;
            }
            if (half == 0) {  // groups that are caught up join this step's rest update
                while (present < pl.present[k]) {
                    int gi = 0;
                    while (gi < ng && ge[gi] <= present) gi++;
                    if (gi >= ng || !waited[gi] || applied[gi] != k || gs[gi] < k + 2) return 5;
                    joined[gi] = k;
                    present = ge[gi];
                }
                if (present != pl.present[k]) return 6;
                if (present < std::min(mt, k + 3)) return 7;  // row k + 2 for the next step
            }
        }
    }
    for (int gi = 0; gi < ng; gi++)
        if (joined[gi] < 0 || (gi > 0 && joined[gi] > gs[gi] - 2)) return 8;
    return 0;
}
