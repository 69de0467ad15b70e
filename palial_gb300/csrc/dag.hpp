// dag.hpp -- host-side DAG builder for the persistent scheduler.
//
// The tile algorithms are the reference's right-looking loops (src/cholesky.h:15-176,
// src/lu.h:14-174, src/qr.h:18-191) with the dependences they really have (the
// reference's LU declares the wrong output dependence on its two TRSM tasks, src/lu.h:62
// and :104; here every task waits on the objects it reads and updates).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "common.cuh"

namespace palial {

struct LogicalTask {
    uint32_t mat;      // matrix index (batched DAGs)
    uint8_t type;
    uint8_t nparts;
    uint16_t k, m, n;
    uint8_t nwait, nsig;
    uint32_t wait_obj[3], wait_cnt[3];
    uint32_t sig_obj[2];
    double cost;       // seconds per part (model)
    double bl;         // bottom level (critical path to the end, seconds)
};

struct Dag {
    int alg = 0, n = 0, nb = 0, bs = 0;  // alg 3 = QR solve: n = rows
    int cols = 0, nrhs = 0;              // QR solve only
    int nobj = 0;
    unsigned long long uid = 0;         // unique per built DAG (device upload cache key)
    std::vector<LogicalTask> logical;   // program order
    std::vector<Task> records;          // dispatch order (one per part)
    std::vector<uint32_t> rec_logical;  // logical index of each record
    double critical_path = 0.0;         // model seconds
    double sim_makespan = 0.0;          // model seconds of the simulated dispatch
};

// Per-part cost in seconds on one worker, FP64 path.  `costs` (optional, T_NUM_TYPES
// entries, seconds per unit of the type's nominal work) overrides the flop model.
double task_cost(int type, int bs, int nb, int part, const double *costs);

// Build the program-order DAG.  bs = block size (divides nb) for Cholesky/LU; QR uses nb.
Dag build_dag(int alg, int n, int nb, int bs, const double *costs = nullptr);

// QR solve / least squares (alg 3): the flat-tree tile QR of a rows x cols tile matrix
// (rows >= cols, both multiples of nb) extended by one tile column holding nrhs <= nb
// right-hand sides (tile column cols/nb of the rows x (cols + nb) tile layout), so the
// UNMQR/TSMQR tasks apply Q^T to them inside the same launch; then the blocked
// back-substitution R X = (Q^T B)(0:cols) with left-upper TRSM and GEMM tasks.  apply_only:
// the factors are already in place; only Q^T B and the back-substitution are emitted (the
// refinement steps of the mixed-precision QR solve).
Dag build_qr_solve_dag(int rows, int cols, int nb, int nrhs, bool apply_only = false);
// A X = B with the FP64 factors of a Cholesky (alg 0, U^T U) or no-pivot LU (alg 1) in the first
// n / nb tile columns of an n x (n + nb) tile matrix whose last tile column holds B (nrhs <= nb
// columns): forward substitution tasks (TRSM + GEMM on the extra column), then backward.
Dag build_trsolve_dag(int n, int nb, int nrhs, int alg);

// One matrix of a batch: algorithm (0 Cholesky, 1 LU), padded size, tile size, block size.
struct BatchSpec {
    int alg, n, nb, bs;
};
// Merge the DAGs of independent matrices (object ranges offset per matrix) into one.
Dag build_batch_dag(const std::vector<BatchSpec> &specs, const double *costs = nullptr);

// Dispatch order.  priority 0: critical-path list scheduling simulated with `nworkers`
// workers; 1: program order; 2: same as 0 with the caller's costs.  shuffle_seed != 0
// perturbs costs and ties (tests of schedule independence).
void order_dag(Dag &d, int priority, int nworkers, unsigned shuffle_seed);

// Host validation: every wait target is produced by earlier records; per-object updates
// are totally ordered; an emulation with random durations finishes.  Returns "" if valid.
std::string validate_dag(const Dag &d, int nworkers, unsigned seed);

// Reference task name (type + k + m + n with the reference's stale loop variables,
// src/cholesky.h:19-28, src/lu.h:18-26, src/qr.h:23-31), one per logical task.
std::vector<std::string> reference_names(const Dag &d);

double algorithmic_flops(int alg, double n);

// Bottom levels (critical path to the end) from the current per-task costs.
void recompute_bottom_levels(Dag &d);

// Features of the cost model for one task part (kFeatures floats): task type one-hot, block
// and tile size, k-step progress, part position, parallel width of the step, nominal flops,
// workers, precision.  The same function serves training (trace records) and planning.
constexpr int kFeatures = 21;
void task_features(const Dag &d, const LogicalTask &t, int part, int nworkers, int precision,
                   const std::vector<int> &step_width, float *f);
std::vector<int> step_widths(const Dag &d);
double nominal_task_flops(int type, int bs, int nb, int part);

}  // namespace palial
