"""Learned task-cost model: training data from the scheduler's device traces, an MLP trained on
the GPU by the library's own kernels, and its two uses -- per-task costs for the critical-path
dispatch order (opts.priority = 2) and the choice of the block size by predicted makespan.

The fallback it is compared with: an exhaustive autotuner (every candidate block size timed
on a proxy size) with the static flop-model critical-path priorities.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import PalialError, factor_dev, lib

HIDDEN = 64


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
        rc = self.h.palial_mlp_init(self.nin, hidden, seed)
        if rc:
            raise PalialError(rc, "mlp init")

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
        return np.exp(self.predict(x).astype(np.float64)) * 1e-6   # seconds per part

    def register(self, alg: int, n: int, nb: int, bs: int, nworkers: int) -> np.ndarray:
        c = np.ascontiguousarray(self.task_costs(alg, n, nb, bs, nworkers), dtype=np.float64)
        self.h.palial_gpu_set_task_costs(alg, n, nb, bs, c.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(c))
        return c

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


def trace_records(torch, alg: str, n: int, nb: int, bs: int, seed: int = 1):
    """Run one traced FP64 factorization; return (features, log-us) of its task records."""
    from . import gen_spd, gen_uniform
    h = _bind()
    d = torch.empty(n * n, dtype=torch.float64, device="cuda")
    if alg == "cholesky":
        gen_spd(d.data_ptr(), n, nb, seed)
    else:
        gen_uniform(d.data_ptr(), n, nb, seed)
    s = torch.zeros_like(d) if alg == "qr" else None
    factor_dev(alg, d.data_ptr(), s.data_ptr() if s is not None else None, n, nb, block=bs, trace=True)
    cnt = int(h.palial_gpu_trace_features(None, None, 0))
    x = np.zeros((cnt, nfeatures()), dtype=np.float32)
    y = np.zeros(cnt, dtype=np.float32)
    h.palial_gpu_trace_features(_fp(x), _fp(y), cnt)
    del d, s
    torch.cuda.empty_cache()
    return x, y


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
