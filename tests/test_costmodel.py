"""Cost model host logic and its CPU oracle (no GPU): the numpy MLP oracle against finite
differences, and the planning plumbing (features, learned costs, predicted makespan)."""
import ctypes

import numpy as np

import palial_gb300 as P
from oracle import mlp_ref


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    nin, h = 5, 7
    npar = nin * h + h + h * h + h + h + 1
    p = rng.normal(size=npar) * 0.5
    x = rng.normal(size=(11, nin))
    y = rng.normal(size=11)
    loss, g = mlp_ref.loss_and_grad(p, x, y, nin, h)
    eps = 1e-6
    for i in rng.choice(npar, 25, replace=False):
        q = p.copy()
        q[i] += eps
        lp, _ = mlp_ref.loss_and_grad(q, x, y, nin, h)
        q[i] -= 2 * eps
        lm, _ = mlp_ref.loss_and_grad(q, x, y, nin, h)
        assert abs((lp - lm) / (2 * eps) - g[i]) <= 1e-6 * max(1.0, abs(g[i]))


def test_features_and_learned_priorities_plumbing():
    lib = P.lib()
    lib.palial_dag_logical_features.restype = ctypes.c_longlong
    lib.palial_dag_logical_features.argtypes = [ctypes.c_int] * 5 + [ctypes.POINTER(ctypes.c_float), ctypes.c_longlong]
    nf = lib.palial_dag_features_count()
    cnt = lib.palial_dag_logical_features(0, 4096, 512, 256, 152, None, 0)
    x = np.zeros((cnt, nf), dtype=np.float32)
    assert lib.palial_dag_logical_features(0, 4096, 512, 256, 152, x.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                           cnt) == cnt
    assert np.allclose(x[:, :12].sum(1), 1.0)           # one-hot task type
    base = P.dag_info("cholesky", 4096, 512, block=256, priority=0)
    # learned costs = 2x the flop model everywhere: same order, twice the makespan
    flop = P.dag_info("cholesky", 4096, 512, block=256, priority=2)   # none registered: flop model
    assert abs(flop["makespan_s"] - base["makespan_s"]) < 1e-9
    lib.palial_gpu_set_task_costs.argtypes = [ctypes.c_int] * 4 + [ctypes.POINTER(ctypes.c_double), ctypes.c_longlong]
    costs = np.full(cnt, 1e-3)
    lib.palial_gpu_set_task_costs(0, 4096, 512, 256, costs.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), cnt)
    learned = P.dag_info("cholesky", 4096, 512, block=256, priority=2)
    assert learned["makespan_s"] > 0 and abs(learned["critical_path_s"] - base["critical_path_s"]) > 0
    lib.palial_gpu_set_task_costs(0, 4096, 512, 256, None, 0)
    assert P.dag_validate("cholesky", 4096, 512, block=256, priority=0) == ""
