"""Learned task-cost model: training data from the scheduler's device traces, an MLP trained on
the GPU by the library's own kernels, and its two uses -- per-task costs for the critical-path
dispatch order (opts.priority = 2) and the choice of the tile size NB (and block) by the
makespan the host's ticket-dispatch simulation predicts under the learned costs.

The network predicts log(duration / nominal flops) of a task record (its inverse throughput;
the nominal flop count comes from the record's own features), from standardised features.
The duration itself is exp(prediction) * flops.

The fallback it is compared with: an exhaustive autotuner (every candidate timed at the target
size) with the static flop-model critical-path priorities.
"""
from __future__ import annotations

import ctypes
import math
import time

import numpy as np

from . import PalialError, factor_dev, lib

HIDDEN = 64
FLOP_FEATURE = 18   # log2(nominal flops of the record) / 40 (dag.cpp task_features)


def log_flops(x: np.ndarray) -> np.ndarray:
    """Natural log of each record's nominal flop count, from its features."""
    return x[:, FLOP_FEATURE].astype(np.float64) * 40.0 * math.log(2.0)


def nfeatures() -> int:
    return int(lib().palial_dag_features_count())


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _bind():
    h = lib()
    f, i, ll, vp = ctypes.POINTER(ctypes.c_float), ctypes.c_int, ctypes.c_longlong, ctypes.c_void_p
    h.palial_mlp_init.argtypes = [i, i, ctypes.c_uint64]
    h.palial_mlp_param_count.restype = ll
    h.palial_mlp_get_params.argtypes = [f]
    h.palial_mlp_set_params.argtypes = [f]
    h.palial_mlp_grad.argtypes = [f, f, i, f, f]
    h.palial_mlp_train.argtypes = [f, f, i, i, i, ctypes.c_float, ctypes.c_uint64, f]
    h.palial_mlp_predict.argtypes = [f, i, f]
    h.palial_gpu_trace_features.restype = ll
    h.palial_gpu_trace_features.argtypes = [f, f, ll]
    h.palial_dag_logical_features.restype = ll
    h.palial_dag_logical_features.argtypes = [i, i, i, i, i, f, ll]
    h.palial_gpu_set_task_costs.argtypes = [i, i, i, i, ctypes.POINTER(ctypes.c_double), ll]
    return h


class CostModel:
    def __init__(self, seed: int = 0, hidden: int = HIDDEN):
        self.h = _bind()
        self.nin = nfeatures()
        self.hidden = hidden
        self.mu = np.zeros(self.nin, dtype=np.float32)
        self.sd = np.ones(self.nin, dtype=np.float32)
        rc = self.h.palial_mlp_init(self.nin, hidden, seed)
        if rc:
            raise PalialError(rc, "mlp init")

    # ---- the task-time model (inputs: raw features; outputs: log microseconds) ---------------
    def fit(self, x, y_log_us, epochs: int = 30, batch: int = 1024, lr: float = 2e-3, seed: int = 1) -> float:
        """Train on raw features and log(us) targets: standardise the features (statistics of
        this training set) and learn log(us / flops)."""
        x = np.asarray(x, dtype=np.float32)
        self.mu = x.mean(axis=0).astype(np.float32)
        sd = x.std(axis=0)
        self.sd = np.where(sd > 1e-6, sd, 1.0).astype(np.float32)
        t = (np.asarray(y_log_us, dtype=np.float64) - log_flops(x)).astype(np.float32)
        return self.train((x - self.mu) / self.sd, t, epochs=epochs, batch=batch, lr=lr, seed=seed)

    def predict_log_us(self, x) -> np.ndarray:
        x = np.asarray(x, dtype=np.float32)
        return self.predict((x - self.mu) / self.sd).astype(np.float64) + log_flops(x)

    def params(self) -> np.ndarray:
        p = np.zeros(int(self.h.palial_mlp_param_count()), dtype=np.float32)
        self.h.palial_mlp_get_params(_fp(p))
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        self.h.palial_mlp_set_params(_fp(p))

    def grad(self, x: np.ndarray, y: np.ndarray) -> tuple[float, np.ndarray]:
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        g = np.zeros(int(self.h.palial_mlp_param_count()), dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        rc = self.h.palial_mlp_grad(_fp(x), _fp(y), len(y), _fp(g), _fp(loss))
        if rc:
            raise PalialError(rc, "mlp grad")
        return float(loss[0]), g

    def train(self, x, y, epochs: int = 30, batch: int = 1024, lr: float = 2e-3, seed: int = 1) -> float:
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        rc = self.h.palial_mlp_train(_fp(x), _fp(y), len(y), epochs, min(batch, len(y)), lr, seed, _fp(loss))
        if rc:
            raise PalialError(rc, "mlp train")
        return float(loss[0])

    def predict(self, x) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        out = np.zeros(len(x), dtype=np.float32)
        rc = self.h.palial_mlp_predict(_fp(x), len(x), _fp(out))
        if rc:
            raise PalialError(rc, "mlp predict")
        return out

    # ---- planning ---------------------------------------------------------------------------
    def task_costs(self, alg: int, n: int, nb: int, bs: int, nworkers: int) -> np.ndarray:
        cnt = int(self.h.palial_dag_logical_features(alg, n, nb, bs, nworkers, None, 0))
        if cnt < 0:
            raise PalialError(-1, "bad DAG shape")
        x = np.zeros((cnt, self.nin), dtype=np.float32)
        self.h.palial_dag_logical_features(alg, n, nb, bs, nworkers, _fp(x), cnt)
        return np.exp(self.predict_log_us(x)) * 1e-6   # seconds per part

    def register(self, alg: int, n: int, nb: int, bs: int, nworkers: int) -> np.ndarray:
        c = np.ascontiguousarray(self.task_costs(alg, n, nb, bs, nworkers), dtype=np.float64)
        self.h.palial_gpu_set_task_costs(alg, n, nb, bs, c.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(c))
        return c

    def predicted_makespan(self, alg: int, n: int, nb: int, bs: int, nworkers: int) -> float:
        """Makespan of the ticket-dispatch simulation with the learned task costs and the
        learned critical-path priorities (block 0 = the library's default for nb)."""
        from . import dag_info
        self.register(alg, n, nb, bs, nworkers)
        return dag_info(["cholesky", "lu", "qr"][alg], n, nb, block=bs, priority=2, nworkers=nworkers)["makespan_s"]

    def choose_nb(self, alg: int, n: int, candidates, nworkers: int) -> tuple[int, dict]:
        """Tile size NB (default block) with the smallest predicted makespan."""
        pred = {nb: self.predicted_makespan(alg, n, nb, 0, nworkers) for nb in candidates if n % nb == 0}
        return min(pred, key=pred.get), pred

    def choose_block(self, alg: int, n: int, nb: int, candidates, nworkers: int) -> tuple[int, dict]:
        """Block size with the smallest makespan predicted by the ticket-dispatch simulation
        under the learned costs."""
        from . import dag_info
        pred = {}
        for bs in candidates:
            self.register(alg, n, nb, bs, nworkers)
            pred[bs] = dag_info(["cholesky", "lu", "qr"][alg], n, nb, block=bs, priority=2,
                                nworkers=nworkers)["makespan_s"]
        return min(pred, key=pred.get), pred


COST_NBS = (256, 384, 512, 768, 1024)


def sweep_plan(alg: str, sizes=(8192, 16384, 24576, 32768), nbs=COST_NBS) -> list:
    """(N, NB, block) of a trace sweep: every N x NB with N % NB == 0 (the reference's rule,
    palial_src/main.c:101-105), each with the library's default block (0) and, where it differs,
    the largest block in {192, 256, 384, 512} dividing NB (the model must generalise over blocks
    too).  QR (block = tile) at N <= 16384 only: its FP64 runs at 24576 / 32768 take 25-55 s."""
    out = []
    for n in sizes:
        if alg == "qr" and n > 16384:
            continue
        for nb in nbs:
            if n % nb:
                continue
            if alg == "qr":
                out.append((n, nb, nb))
                continue
            out.append((n, nb, 0))
            big = max(b for b in (192, 256, 384, 512) if nb % b == 0)
            if big != min(nb, 256):
                out.append((n, nb, big))
    return out


def plan_space(n: int, nbs=COST_NBS) -> list:
    """(NB, block) plans the learned model chooses among at size n."""
    return [(nb, bs) for nb in nbs if n % nb == 0 for bs in (192, 256, 384, 512) if nb % bs == 0]


def trace_records(torch, alg: str, n: int, nb: int, bs: int, seed: int = 1, with_time: bool = False):
    """Run one traced FP64 factorization; return (features, log-us) of its task records (and
    the measured makespan in seconds with with_time=True)."""
    from . import gen_spd, gen_uniform
    h = _bind()
    d = torch.empty(n * n, dtype=torch.float64, device="cuda")
    if alg == "cholesky":
        gen_spd(d.data_ptr(), n, nb, seed)
    else:
        gen_uniform(d.data_ptr(), n, nb, seed)
    s = torch.zeros_like(d) if alg == "qr" else None
    st = factor_dev(alg, d.data_ptr(), s.data_ptr() if s is not None else None, n, nb, block=bs, trace=True)
    cnt = int(h.palial_gpu_trace_features(None, None, 0))
    x = np.zeros((cnt, nfeatures()), dtype=np.float32)
    y = np.zeros(cnt, dtype=np.float32)
    h.palial_gpu_trace_features(_fp(x), _fp(y), cnt)
    del d, s
    torch.cuda.empty_cache()
    return (x, y, st.seconds) if with_time else (x, y)


def checksum(torch, d) -> int:
    """Order-independent fingerprint of a float64 device buffer's bits (equal bits -> equal)."""
    v = d.view(torch.int64)
    return int(v.sum().item()) ^ int((v * 0x9E3779B1).sum().item())


def exhaustive_nb(torch, alg: str, n: int, candidates, seed: int = 0, reps: int = 1):
    """Fallback autotuner: factor the target problem with every candidate NB (the library's
    default block, static priorities) and keep the fastest.  Returns (best NB, {NB: seconds},
    {NB: checksum of the factors}, seconds spent searching)."""
    from . import gen_spd, gen_uniform
    t0 = time.perf_counter()
    times, sums = {}, {}
    for nb in candidates:
        if n % nb:
            continue
        d0 = torch.empty(n * n, dtype=torch.float64, device="cuda")
        (gen_spd if alg == "cholesky" else gen_uniform)(d0.data_ptr(), n, nb, seed)
        d = torch.empty_like(d0)
        best = None
        for _ in range(reps):
            d.copy_(d0)
            st = factor_dev(alg, d.data_ptr(), None, n, nb, priority=0)
            best = st.seconds if best is None else min(best, st.seconds)
        times[nb] = best
        sums[nb] = checksum(torch, d)
        del d, d0
        torch.cuda.empty_cache()
    return min(times, key=times.get), times, sums, time.perf_counter() - t0


def learned_run(torch, model, alg: str, n: int, nb: int, nworkers: int, block: int = 0, seed: int = 0):
    """Factor the target problem with plan (nb, block): with the learned critical-path
    priorities of `model`, or (model None) the static flop-model priorities; returns (seconds,
    checksum of the factors)."""
    from . import gen_spd, gen_uniform
    if model is not None:
        model.register(["cholesky", "lu", "qr"].index(alg), n, nb, block, nworkers)
    d = torch.empty(n * n, dtype=torch.float64, device="cuda")
    (gen_spd if alg == "cholesky" else gen_uniform)(d.data_ptr(), n, nb, seed)
    st = factor_dev(alg, d.data_ptr(), None, n, nb, block=block, priority=2 if model is not None else 0)
    c = checksum(torch, d)
    del d
    torch.cuda.empty_cache()
    return st.seconds, c


def exhaustive_block(torch, alg: str, n_proxy: int, nb: int, candidates) -> tuple[int, dict]:
    """Fallback autotuner: time every candidate block size on a proxy size (static priorities)."""
    from . import gen_spd, gen_uniform
    d0 = torch.empty(n_proxy * n_proxy, dtype=torch.float64, device="cuda")
    if alg == "cholesky":
        gen_spd(d0.data_ptr(), n_proxy, nb, 0)
    else:
        gen_uniform(d0.data_ptr(), n_proxy, nb, 1)
    d = torch.empty_like(d0)
    times = {}
    for bs in candidates:
        best = None
        for _ in range(2):
            d.copy_(d0)
            st = factor_dev(alg, d.data_ptr(), None, n_proxy, nb, block=bs)
            best = st.seconds if best is None else min(best, st.seconds)
        times[bs] = best
    del d, d0
    torch.cuda.empty_cache()
    return min(times, key=times.get), times
