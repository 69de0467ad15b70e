// dag.cpp -- host-side DAG builder, critical-path ordering and validation for the
// persistent device scheduler.
#include "dag.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <functional>
#include <queue>
#include <random>
#include <stdexcept>

namespace palial {

namespace {
constexpr double kWorkerFlops = 8.0e9;  // FP64 flop/s of one SM (about 1.25 TFLOP/s / 152)

double nominal_flops(int type, int bs, int nb, int part) {
    const double b = bs, q = nb, w = 64.0;
    switch (type) {
        case T_POTRF: return b * b * b / 3.0;
        case T_TRSM_LUT: return b * b * w;
        case T_SYRK: return 2.0 * b * w * (part * 64.0 + 32.0);
        case T_GEMM_TN: return 2.0 * b * b * w;
        case T_GETRF: return 2.0 * b * b * b / 3.0;
        case T_TRSM_RUN: return b * b * w;
        case T_TRSM_LLU: return b * b * w;
        case T_GEMM_NN: return 2.0 * b * b * w;
        case T_GEQRT: return 5.0 * q * q * q / 3.0;
        case T_UNMQR: return 3.0 * q * q * w;
        case T_TSQRT: return 3.0 * q * q * q;
        case T_TSMQR: return 5.0 * q * q * w;
        case T_TRSM_LUN: return b * b * w;
        default: return 0.0;
    }
}

struct Builder {
    Dag &d;
    std::vector<uint32_t> cnt;
    explicit Builder(Dag &dd, int nobj) : d(dd), cnt(nobj, 0) { d.nobj = nobj; }

    void emit(int type, int k, int m, int n, int nparts, std::initializer_list<uint32_t> reads,
              std::initializer_list<uint32_t> writes, const double *costs) {
        LogicalTask t{};
        t.type = (uint8_t)type;
        t.nparts = (uint8_t)nparts;
        t.k = (uint16_t)k;
        t.m = (uint16_t)m;
        t.n = (uint16_t)n;
        auto add_wait = [&](uint32_t o) {
            for (int i = 0; i < t.nwait; i++)
                if (t.wait_obj[i] == o) return;
            if (cnt[o] == 0) return;  // nothing produced yet: trivially satisfied
            if (t.nwait >= 3) throw std::runtime_error("dag: more than 3 waits");
            t.wait_obj[t.nwait] = o;
            t.wait_cnt[t.nwait] = cnt[o];
            t.nwait++;
        };
        for (uint32_t o : reads) add_wait(o);
        for (uint32_t o : writes) add_wait(o);
        for (uint32_t o : writes) {
            if (t.nsig >= 2) throw std::runtime_error("dag: more than 2 outputs");
            t.sig_obj[t.nsig++] = o;
        }
        for (uint32_t o : writes) cnt[o] += (uint32_t)nparts;
        t.cost = task_cost(type, d.bs, d.nb, 0, costs);
        d.logical.push_back(t);
    }
};
}  // namespace

double task_cost(int type, int bs, int nb, int part, const double *costs) {
    const double f = nominal_flops(type, bs, nb, part);
    if (costs && type < T_TRSM_LUN && costs[type] > 0.0) return costs[type] * f;
    return f / kWorkerFlops;
}

double algorithmic_flops(int alg, double n) {
    if (alg == 0) return n * n * n / 3.0;
    if (alg == 1) return 2.0 * n * n * n / 3.0;
    return 4.0 * n * n * n / 3.0;
}

Dag build_dag(int alg, int n, int nb, int bs, const double *costs) {
    Dag d;
    d.alg = alg;
    d.n = n;
    d.nb = nb;
    if (alg == 2) bs = nb;
    d.bs = bs;
    if (nb <= 0 || bs <= 0 || n % nb || nb % bs || bs % 64) throw std::runtime_error("dag: bad sizes");
    const int mb = n / bs;
    const int parts = bs / 64;
    if (parts > 255) throw std::runtime_error("dag: block too large");
    auto obj = [mb](int i, int j) { return (uint32_t)(i + j * mb); };
    Builder b(d, mb * mb);
    if (alg == 0) {
        for (int k = 0; k < mb; k++) {
            b.emit(T_POTRF, k, k, k, 1, {}, {obj(k, k)}, costs);
            for (int m = k + 1; m < mb; m++) b.emit(T_TRSM_LUT, k, m, 0, parts, {obj(k, k)}, {obj(k, m)}, costs);
            for (int m = k + 1; m < mb; m++) {
                b.emit(T_SYRK, k, m, 0, parts, {obj(k, m)}, {obj(m, m)}, costs);
                for (int j = k + 1; j < m; j++)
                    b.emit(T_GEMM_TN, k, m, j, parts, {obj(k, j), obj(k, m)}, {obj(j, m)}, costs);
            }
        }
    } else if (alg == 1) {
        for (int k = 0; k < mb; k++) {
            b.emit(T_GETRF, k, k, k, 1, {}, {obj(k, k)}, costs);
            for (int m = k + 1; m < mb; m++) b.emit(T_TRSM_RUN, k, m, 0, parts, {obj(k, k)}, {obj(m, k)}, costs);
            for (int j = k + 1; j < mb; j++) {
                b.emit(T_TRSM_LLU, k, 0, j, parts, {obj(k, k)}, {obj(k, j)}, costs);
                for (int m = k + 1; m < mb; m++)
                    b.emit(T_GEMM_NN, k, m, j, parts, {obj(m, k), obj(k, j)}, {obj(m, j)}, costs);
            }
        }
    } else {
        for (int k = 0; k < mb; k++) {
            b.emit(T_GEQRT, k, k, k, 1, {}, {obj(k, k)}, costs);
            for (int j = k + 1; j < mb; j++) b.emit(T_UNMQR, k, 0, j, parts, {obj(k, k)}, {obj(k, j)}, costs);
            for (int m = k + 1; m < mb; m++) {
                // TSQRT updates R in the upper triangle of A(k,k); UNMQR(k,j) reads only the
                // strictly lower part (V), so TSQRT does not wait for the UNMQRs.
                b.emit(T_TSQRT, k, m, 0, 1, {}, {obj(k, k), obj(m, k)}, costs);
                for (int j = k + 1; j < mb; j++)
                    b.emit(T_TSMQR, k, m, j, parts, {obj(m, k)}, {obj(k, j), obj(m, j)}, costs);
            }
        }
    }
    recompute_bottom_levels(d);
    return d;
}

Dag build_qr_solve_dag(int rows, int cols, int nb, int nrhs, bool apply_only) {
    Dag d;
    d.alg = 3;
    d.n = rows;
    d.cols = cols;
    d.nrhs = nrhs;
    d.nb = nb;
    d.bs = nb;
    if (nb <= 0 || nb % 64 || rows % nb || cols % nb || cols <= 0 || rows < cols || nrhs < 1 || nrhs > nb)
        throw std::runtime_error("dag: bad QR solve sizes");
    const int mt = rows / nb, nt = cols / nb;
    const int parts = nb / 64, rparts = (nrhs + 63) / 64;
    if (mt > 65535 || parts > 255) throw std::runtime_error("dag: QR solve too large");
    auto obj = [mt](int i, int j) { return (uint32_t)(i + j * mt); };
    Builder b(d, mt * (nt + 1));
    for (int k = 0; k < nt; k++) {
        if (!apply_only) {
            b.emit(T_GEQRT, k, k, k, 1, {}, {obj(k, k)}, nullptr);
            for (int j = k + 1; j < nt; j++) b.emit(T_UNMQR, k, 0, j, parts, {obj(k, k)}, {obj(k, j)}, nullptr);
        }
        b.emit(T_UNMQR, k, 0, nt, rparts, {obj(k, k)}, {obj(k, nt)}, nullptr);
        for (int m = k + 1; m < mt; m++) {
            if (!apply_only) {
                b.emit(T_TSQRT, k, m, 0, 1, {}, {obj(k, k), obj(m, k)}, nullptr);
                for (int j = k + 1; j < nt; j++)
                    b.emit(T_TSMQR, k, m, j, parts, {obj(m, k)}, {obj(k, j), obj(m, j)}, nullptr);
            }
            b.emit(T_TSMQR, k, m, nt, rparts, {obj(m, k)}, {obj(k, nt), obj(m, nt)}, nullptr);
        }
    }
    // R X = Y: the last tile row first; every solved block updates the rows above it
    for (int k = nt - 1; k >= 0; k--) {
        b.emit(T_TRSM_LUN, k, k, nt, rparts, {obj(k, k)}, {obj(k, nt)}, nullptr);
        for (int i = 0; i < k; i++) b.emit(T_GEMM_NN, k, i, nt, rparts, {obj(i, k), obj(k, nt)}, {obj(i, nt)}, nullptr);
    }
    recompute_bottom_levels(d);
    return d;
}

Dag build_trsolve_dag(int n, int nb, int nrhs, int alg) {
    Dag d;
    d.alg = 4;
    d.n = n;
    d.cols = n;
    d.nrhs = nrhs;
    d.nb = nb;
    d.bs = nb;
    if (nb <= 0 || nb % 64 || n % nb || nrhs < 1 || nrhs > nb || (alg != 0 && alg != 1))
        throw std::runtime_error("dag: bad triangular solve sizes");
    const int mt = n / nb, rparts = (nrhs + 63) / 64;
    if (mt > 65535) throw std::runtime_error("dag: triangular solve too large");
    auto obj = [mt](int i, int j) { return (uint32_t)(i + j * mt); };
    Builder b(d, mt * (mt + 1));
    // forward: Cholesky U^T Y = B, LU L Y = B (unit); each solved block updates the rows below
    for (int k = 0; k < mt; k++) {
        if (alg == 0) {
            b.emit(T_TRSM_LUT, k, mt, 0, rparts, {obj(k, k)}, {obj(k, mt)}, nullptr);
            for (int i = k + 1; i < mt; i++)
                b.emit(T_GEMM_TN, k, mt, i, rparts, {obj(k, i), obj(k, mt)}, {obj(i, mt)}, nullptr);
        } else {
            b.emit(T_TRSM_LLU, k, 0, mt, rparts, {obj(k, k)}, {obj(k, mt)}, nullptr);
            for (int i = k + 1; i < mt; i++)
                b.emit(T_GEMM_NN, k, i, mt, rparts, {obj(i, k), obj(k, mt)}, {obj(i, mt)}, nullptr);
        }
    }
    // backward: U X = Y, the last tile row first; each solved block updates the rows above
    for (int k = mt - 1; k >= 0; k--) {
        b.emit(T_TRSM_LUN, k, k, mt, rparts, {obj(k, k)}, {obj(k, mt)}, nullptr);
        for (int i = 0; i < k; i++) b.emit(T_GEMM_NN, k, i, mt, rparts, {obj(i, k), obj(k, mt)}, {obj(i, mt)}, nullptr);
    }
    recompute_bottom_levels(d);
    return d;
}

void recompute_bottom_levels(Dag &d) {
    // reverse program order; M[x] = max bl of later tasks waiting on / updating x
    std::vector<double> M(d.nobj, 0.0);
    d.critical_path = 0.0;
    for (size_t i = d.logical.size(); i-- > 0;) {
        LogicalTask &t = d.logical[i];
        double succ = 0.0;
        for (int s = 0; s < t.nsig; s++) succ = std::max(succ, M[t.sig_obj[s]]);
        t.bl = t.cost + succ;
        for (int w = 0; w < t.nwait; w++) M[t.wait_obj[w]] = std::max(M[t.wait_obj[w]], t.bl);
        for (int s = 0; s < t.nsig; s++) M[t.sig_obj[s]] = std::max(M[t.sig_obj[s]], t.bl);
    }
    for (const auto &t : d.logical) d.critical_path = std::max(d.critical_path, t.bl);
}

double nominal_task_flops(int type, int bs, int nb, int part) { return nominal_flops(type, bs, nb, part); }

std::vector<int> step_widths(const Dag &d) {
    std::vector<int> w;
    for (const auto &t : d.logical) {
        if (t.k >= w.size()) w.resize(t.k + 1, 0);
        w[t.k] += t.nparts;
    }
    return w;
}

void task_features(const Dag &d, const LogicalTask &t, int part, int nworkers, int precision,
                   const std::vector<int> &step_width, float *f) {
    for (int i = 0; i < kFeatures; i++) f[i] = 0.f;
    f[t.type == T_TRSM_LUN ? (int)T_TRSM_LUT : (t.type < 12 ? t.type : 11)] = 1.f;
    const int bs = d.bs > 0 ? d.bs : 64, nb = d.nb > 0 ? d.nb : bs;
    const double mb = std::max(1, d.n / bs);
    f[12] = (float)(std::log2((double)bs) / 10.0);
    f[13] = (float)(std::log2((double)nb) / 10.0);
    f[14] = (float)(t.k / mb);
    f[15] = (float)((mb - t.k) / mb);
    f[16] = (float)((double)part / std::max(1, (int)t.nparts));
    const int w = t.k < step_width.size() ? step_width[t.k] : 1;
    f[17] = (float)(std::log2((double)std::max(1, w)) / 20.0);
    f[18] = (float)(std::log2(std::max(1.0, nominal_flops(t.type, bs, nb, part))) / 40.0);
    f[19] = (float)(std::log2((double)std::max(1, nworkers)) / 10.0);
    f[20] = (float)(precision / 3.0);
}

Dag build_batch_dag(const std::vector<BatchSpec> &specs, const double *costs) {
    Dag all;
    all.alg = -1;
    all.nobj = 0;
    for (size_t i = 0; i < specs.size(); i++) {
        const BatchSpec &b = specs[i];
        Dag d = build_dag(b.alg, b.n, b.nb, b.bs, costs);
        const uint32_t base = (uint32_t)all.nobj;
        for (LogicalTask t : d.logical) {
            t.mat = (uint32_t)i;
            for (int w = 0; w < t.nwait; w++) t.wait_obj[w] += base;
            for (int s2 = 0; s2 < t.nsig; s2++) t.sig_obj[s2] += base;
            all.logical.push_back(t);
        }
        all.nobj += d.nobj;
        all.critical_path = std::max(all.critical_path, d.critical_path);
    }
    return all;
}

namespace {
Task make_record(const LogicalTask &t, int part) {
    Task r{};
    r.type = t.type;
    r.part = (uint8_t)part;
    r.nparts = t.nparts;
    r.nwait = t.nwait;
    r.k = t.k;
    r.m = t.m;
    r.n = t.n;
    r.nsig = t.nsig;
    for (int i = 0; i < 3; i++) {
        r.wait_obj[i] = t.wait_obj[i];
        r.wait_cnt[i] = t.wait_cnt[i];
    }
    r.sig_obj[0] = t.sig_obj[0];
    r.sig_obj[1] = t.sig_obj[1];
    r.mat = t.mat;
    return r;
}

// Event-driven list scheduling of the parts.  Returns the start order (indices into the
// flat part list) and the simulated makespan.  dur(part) gives its duration; prio(part)
// its priority (higher first); ties broken by program order.
struct Sim {
    std::vector<uint32_t> order;
    double makespan = 0.0;
    bool complete = false;
};

Sim simulate(const Dag &d, const std::vector<uint32_t> &part_logical, int nworkers,
             const std::function<double(uint32_t)> &dur, const std::function<double(uint32_t)> &prio) {
    const size_t np = part_logical.size();
    Sim sim;
    sim.order.reserve(np);
    std::vector<uint32_t> done(d.nobj, 0);
    std::vector<uint8_t> next_wait(np, 0);
    // per-object min-heap of (target, part)
    using Wt = std::pair<uint32_t, uint32_t>;
    std::vector<std::priority_queue<Wt, std::vector<Wt>, std::greater<Wt>>> waiters(d.nobj);
    using Rd = std::pair<double, uint32_t>;  // (priority, -index) max-heap
    auto rcmp = [](const Rd &a, const Rd &b) {
        if (a.first != b.first) return a.first < b.first;
        return a.second > b.second;
    };
    std::priority_queue<Rd, std::vector<Rd>, decltype(rcmp)> ready(rcmp);
    std::function<void(uint32_t)> advance = [&](uint32_t p) {
        const LogicalTask &t = d.logical[part_logical[p]];
        while (next_wait[p] < t.nwait) {
            const int w = next_wait[p];
            if (done[t.wait_obj[w]] >= t.wait_cnt[w]) {
                next_wait[p]++;
                continue;
            }
            waiters[t.wait_obj[w]].push({t.wait_cnt[w], p});
            return;
        }
        ready.push({prio(p), p});
    };
    for (uint32_t p = 0; p < np; p++) advance(p);
    using Ev = std::pair<double, uint32_t>;  // (finish time, part)
    std::priority_queue<Ev, std::vector<Ev>, std::greater<Ev>> running;
    double now = 0.0;
    int idle = nworkers;
    size_t finished = 0;
    while (finished < np) {
        while (idle > 0 && !ready.empty()) {
            const uint32_t p = ready.top().second;
            ready.pop();
            sim.order.push_back(p);
            running.push({now + dur(p), p});
            idle--;
        }
        if (running.empty()) break;  // stuck: waits that nothing satisfies
        const Ev e = running.top();
        running.pop();
        now = e.first;
        idle++;
        finished++;
        const LogicalTask &t = d.logical[part_logical[e.second]];
        for (int s = 0; s < t.nsig; s++) {
            const uint32_t o = t.sig_obj[s];
            done[o]++;
            auto &h = waiters[o];
            while (!h.empty() && h.top().first <= done[o]) {
                const uint32_t q = h.top().second;
                h.pop();
                next_wait[q]++;
                advance(q);
            }
        }
    }
    sim.makespan = now;
    sim.complete = (finished == np);
    return sim;
}
// Ticket dispatch exactly as on the device: idle workers take records strictly in dispatch
// order and block until the record's waits are met.  Returns the makespan, or -1 if some
// record waits for signals that no earlier record produces (a deadlock on the device).
double simulate_ticket(const Dag &d, int nworkers, const std::function<double(size_t)> &dur) {
    std::vector<std::vector<double>> sig_times(d.nobj);  // sorted finish times of signals
    std::priority_queue<double, std::vector<double>, std::greater<double>> free_at;
    for (int w = 0; w < std::max(1, nworkers); w++) free_at.push(0.0);
    double makespan = 0.0;
    for (size_t r = 0; r < d.records.size(); r++) {
        const Task &t = d.records[r];
        double start = free_at.top();
        free_at.pop();
        for (int w = 0; w < t.nwait; w++) {
            const auto &v = sig_times[t.wait_obj[w]];
            if (v.size() < t.wait_cnt[w]) return -1.0;
            start = std::max(start, v[t.wait_cnt[w] - 1]);
        }
        const double fin = start + dur(r);
        makespan = std::max(makespan, fin);
        free_at.push(fin);
        for (int s = 0; s < t.nsig; s++) {
            auto &v = sig_times[t.sig_obj[s]];
            v.insert(std::upper_bound(v.begin(), v.end(), fin), fin);
        }
    }
    return makespan;
}
}  // namespace

void order_dag(Dag &d, int priority, int nworkers, unsigned shuffle_seed) {
    std::vector<uint32_t> part_logical;
    std::vector<uint8_t> part_index;
    for (uint32_t i = 0; i < d.logical.size(); i++)
        for (int p = 0; p < d.logical[i].nparts; p++) {
            part_logical.push_back(i);
            part_index.push_back((uint8_t)p);
        }
    d.records.clear();
    d.rec_logical.clear();
    if (priority == 1 && shuffle_seed == 0) {
        for (size_t p = 0; p < part_logical.size(); p++) {
            d.records.push_back(make_record(d.logical[part_logical[p]], part_index[p]));
            d.rec_logical.push_back(part_logical[p]);
        }
        d.sim_makespan = simulate_ticket(d, nworkers, [&](size_t r) { return d.logical[d.rec_logical[r]].cost; });
        return;
    }
    std::mt19937_64 rng(shuffle_seed);
    std::uniform_real_distribution<double> jitter(0.5, 1.5);
    std::vector<double> pr(part_logical.size()), du(part_logical.size());
    // Batches: shortest matrix first (total work of its tasks), critical path within a matrix.
    // The makespan is set by the total work and the largest matrices' critical paths, so the
    // small matrices can finish early at almost no cost.
    std::vector<double> mat_work;
    const bool batch = (d.alg < 0);
    if (batch) {
        for (const auto &t : d.logical) {
            if (t.mat >= mat_work.size()) mat_work.resize(t.mat + 1, 0.0);
            mat_work[t.mat] += t.cost * t.nparts;
        }
    }
    for (size_t p = 0; p < part_logical.size(); p++) {
        const LogicalTask &t = d.logical[part_logical[p]];
        const double j = shuffle_seed ? jitter(rng) : 1.0;
        du[p] = t.cost * j;
        pr[p] = (priority == 1) ? -(double)p : t.bl * (shuffle_seed ? jitter(rng) : 1.0);
        if (batch && priority != 1) pr[p] -= 1e6 * mat_work[t.mat];
    }
    Sim s = simulate(d, part_logical, std::max(1, nworkers), [&](uint32_t p) { return du[p]; },
                     [&](uint32_t p) { return pr[p]; });
    if (!s.complete) throw std::runtime_error("dag: simulation did not complete (invalid waits)");
    for (uint32_t p : s.order) {
        d.records.push_back(make_record(d.logical[part_logical[p]], part_index[p]));
        d.rec_logical.push_back(part_logical[p]);
    }
    d.sim_makespan = simulate_ticket(d, nworkers, [&](size_t r) { return d.logical[d.rec_logical[r]].cost; });
}

std::string validate_dag(const Dag &d, int nworkers, unsigned seed) {
    char buf[256];
    // 1. every wait target is reachable from records earlier in dispatch order
    std::vector<uint32_t> produced(d.nobj, 0);
    std::vector<uint32_t> final_count(d.nobj, 0);
    for (const auto &t : d.logical)
        for (int s = 0; s < t.nsig; s++) final_count[t.sig_obj[s]] += t.nparts;
    for (size_t i = 0; i < d.records.size(); i++) {
        const Task &r = d.records[i];
        for (int w = 0; w < r.nwait; w++) {
            if (produced[r.wait_obj[w]] < r.wait_cnt[w]) {
                snprintf(buf, sizeof buf, "record %zu waits for object %u >= %u but only %u signals precede it", i,
                         r.wait_obj[w], r.wait_cnt[w], produced[r.wait_obj[w]]);
                return buf;
            }
        }
        for (int s = 0; s < r.nsig; s++) produced[r.sig_obj[s]]++;
    }
    // 2. each writer of an object waits for all earlier writers of that object (total order
    //    of updates = k order), and every reader waits for the writer it reads.
    std::vector<uint32_t> cnt(d.nobj, 0);
    for (size_t i = 0; i < d.logical.size(); i++) {
        const LogicalTask &t = d.logical[i];
        for (int s = 0; s < t.nsig; s++) {
            const uint32_t o = t.sig_obj[s];
            if (cnt[o] > 0) {
                bool ok = false;
                for (int w = 0; w < t.nwait; w++) ok |= (t.wait_obj[w] == o && t.wait_cnt[w] == cnt[o]);
                if (!ok) {
                    snprintf(buf, sizeof buf, "logical task %zu updates object %u without waiting for its %u earlier updates",
                             i, o, cnt[o]);
                    return buf;
                }
            }
        }
        for (int s = 0; s < t.nsig; s++) cnt[t.sig_obj[s]] += t.nparts;
    }
    // 3. emulate the device's ticket dispatch with random durations
    std::mt19937_64 rng(seed ? seed : 1);
    std::uniform_real_distribution<double> u(0.01, 1.0);
    std::vector<double> du(d.records.size());
    for (auto &x : du) x = u(rng);
    if (simulate_ticket(d, nworkers, [&](size_t r) { return du[r]; }) < 0.0)
        return "emulation stalled: some record waits for a signal that never comes";
    return "";
}

std::vector<std::string> reference_names(const Dag &d) {
    std::vector<std::string> names;
    names.reserve(d.logical.size());
    const int mt = d.n / d.bs;
    auto nm = [](const char *ty, int k, int m, int n) {
        char b[64];
        snprintf(b, sizeof b, "%s%d%d%d", ty, k, m, n);
        return std::string(b);
    };
    int k = 0, m = 0, n = 0;  // zero-initialised, as the reference's loop variables read as
    if (d.alg < 0 || d.alg > 2) {
        // no reference counterpart (batched, QR solve): type + the task's own coordinates
        static const char *tn[] = {"potrf", "trsm", "syrk", "gemm", "getrf", "trsm", "trsm",
                                   "gemm",  "geqrt", "ormqr", "tsqrt", "tsmqr", "trsm"};
        for (const LogicalTask &t : d.logical)
            names.push_back(nm(t.type < T_NUM_TYPES ? tn[t.type] : "task", t.k, t.m, t.n));
        return names;
    }
    if (d.alg == 0) {
        for (k = 0; k < mt; k++) {
            names.push_back(nm("potrf", k, m, n));
            for (m = k + 1; m < mt; m++) names.push_back(nm("trsm", k, m, n));
            for (m = k + 1; m < mt; m++) {
                names.push_back(nm("syrk", k, m, n));
                for (n = k + 1; n < m; n++) names.push_back(nm("gemm", k, m, n));
            }
        }
    } else if (d.alg == 1) {
        for (k = 0; k < mt; k++) {
            names.push_back(nm("getrf", k, m, n));
            for (m = k + 1; m < mt; m++) names.push_back(nm("trsm", k, m, n));
            for (n = k + 1; n < mt; n++) {
                names.push_back(nm("trsm", k, m, n));
                for (m = k + 1; m < mt; m++) names.push_back(nm("gemm", k, m, n));
            }
        }
    } else {
        for (k = 0; k < mt; k++) {
            names.push_back(nm("geqrt", k, m, n));
            for (n = k + 1; n < mt; n++) names.push_back(nm("ormqr", k, m, n));
            for (m = k + 1; m < mt; m++) {
                names.push_back(nm("tsqrt", k, m, n));
                for (n = k + 1; n < mt; n++) names.push_back(nm("tsmqr", k, m, n));
            }
        }
    }
    return names;
}

}  // namespace palial
