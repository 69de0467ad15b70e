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
