"""The task-cost MLP on the GPU: gradients and forward pass against the numpy oracle, training
convergence, and training data from a real device trace."""
import numpy as np
import pytest

from oracle import mlp_ref

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _model():
    from palial_gb300.costmodel import CostModel
    return CostModel(seed=3)


def test_gradients_match_cpu_oracle():
    m = _model()
    rng = np.random.default_rng(1)
    x = rng.normal(size=(257, m.nin)).astype(np.float32)
    y = rng.normal(size=257).astype(np.float32)
    p = m.params()
    loss, g = m.grad(x, y)
    lref, gref = mlp_ref.loss_and_grad(p.astype(np.float64), x.astype(np.float64), y.astype(np.float64), m.nin, m.hidden)
    assert abs(loss - lref) <= 1e-4 * abs(lref)
    assert np.linalg.norm(g - gref) <= 1e-4 * np.linalg.norm(gref)
    out, _ = mlp_ref.forward(p.astype(np.float64), x.astype(np.float64), m.nin, m.hidden)
    assert np.allclose(m.predict(x), out, rtol=1e-4, atol=1e-4)


def test_training_fits_a_smooth_target():
    m = _model()
    rng = np.random.default_rng(2)
    x = rng.uniform(-1, 1, size=(8192, m.nin)).astype(np.float32)
    y = (np.sin(2 * x[:, 0]) + 0.5 * x[:, 1] * x[:, 2]).astype(np.float32)
    l0, _ = m.grad(x[:1024], y[:1024])
    m.train(x, y, epochs=40, batch=512, lr=3e-3)
    l1, _ = m.grad(x[:1024], y[:1024])
    assert l1 < 0.05 * l0, (l0, l1)


def test_trace_training_data():
    from palial_gb300.costmodel import trace_records
    x, y = trace_records(torch, "cholesky", 2048, 512, 128)
    assert len(y) > 100 and np.isfinite(x).all() and np.isfinite(y).all()
    assert np.allclose(x[:, :12].sum(1), 1.0)


def test_learned_plan_against_exhaustive_autotuner():
    """What the trained network gains: trained on traces of FP64 Cholesky at N = 4096 and 6144
    (every NB in {256, 512, 1024}, default and large blocks), it chooses an (NB, block) plan for
    N = 8192 and runs it with its learned critical-path priorities.  The fallback, the
    exhaustive autotuner, factors N = 8192 once per NB (default block, static priorities) and
    keeps the fastest.  The learned plan must come within 10 % of the fallback's makespan (or
    beat it) without the search, and its factors must equal, bit for bit, the same plan's
    factors under the static priorities (numerics are schedule-independent)."""
    import palial_gb300 as P
    from palial_gb300.costmodel import CostModel, exhaustive_nb, learned_run, plan_space, sweep_plan, trace_records
    nbs = (256, 512, 1024)
    xs, ys = [], []
    for n, nb, bs in sweep_plan("cholesky", sizes=(4096, 6144), nbs=nbs):
        x, y = trace_records(torch, "cholesky", n, nb, bs)
        xs.append(x)
        ys.append(y)
    m = CostModel(seed=5)
    m.fit(np.concatenate(xs), np.concatenate(ys), epochs=40, batch=512, lr=2e-3)
    workers = P.lib().palial_gpu_sm_count()
    n = 8192
    preds = {plan: m.predicted_makespan(0, n, plan[0], plan[1], workers) for plan in plan_space(n, nbs)}
    plan = min(preds, key=preds.get)
    fb_nb, fb_times, _, search_s = exhaustive_nb(torch, "cholesky", n, nbs, reps=2)
    learned = min(learned_run(torch, m, "cholesky", n, plan[0], workers, block=plan[1])[0] for _ in range(2))
    _, c_learned = learned_run(torch, m, "cholesky", n, plan[0], workers, block=plan[1])
    static_s, c_static = learned_run(torch, None, "cholesky", n, plan[0], workers, block=plan[1])
    print(f"learned plan nb={plan[0]} bs={plan[1]}: {learned:.4f} s (predicted {preds[plan]:.4f}); "
          f"static priorities {static_s:.4f} s; exhaustive best nb={fb_nb}: {fb_times[fb_nb]:.4f} s "
          f"after {search_s:.2f} s of search; all {fb_times}")
    assert c_learned == c_static
    assert learned <= 1.10 * fb_times[fb_nb], (learned, fb_times)
