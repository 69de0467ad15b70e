"""Batched uneven factorizations (one persistent launch): every factor against numpy, padding
exactness, graph replay bit-identical to a direct launch, completion times."""
import numpy as np
import pytest

import palial_gb300 as P
from palial_gb300 import batched as B
from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_batched_factors_match_numpy():
    ns, algs = B.batch_sizes(48, 9)
    ns = np.minimum(ns, 700)
    bsc = {c: (64 if c < 2 else 128) for c in range(6)}
    b = B.Batch(torch, ns, algs, bsc, seed=9)
    st, comp = b.run(graph=False, completion=True)
    assert st.code in (0, 1)
    assert (comp > 0).all() and np.isfinite(comp).all()
    for i in range(b.count):
        a = b.original(i)
        f = b.factor(i)
        n = a.shape[0]
        if algs[i] == 0:
            u = np.triu(f)
            assert np.linalg.norm(u - np.linalg.cholesky(a).T) <= 1e-12 * np.linalg.norm(u), i
        else:
            l = np.tril(f, -1) + np.eye(n)
            assert np.linalg.norm(a - l @ np.triu(f)) <= 1e-8 * np.linalg.norm(a), i


def test_graph_replay_bitwise_equal():
    ns, algs = B.batch_sizes(24, 4)
    b = B.Batch(torch, ns, algs, {c: 64 for c in range(6)}, seed=4)
    b.run(graph=False)
    direct = b.buf.clone()
    for _ in range(2):
        b.reset()
        st, _ = b.run(graph=True)
        assert torch.equal(b.buf, direct)
    assert st.seconds > 0


def test_library_synthetic_batch_split_over_two_ranks():
    """The library's synthetic batch driver: the two ranks' shares cover the batch, and every
    share runs and reports per-class completion times."""
    reps = [B.synthetic(64, seed=5, rank=r, world=2, autotune=False, reps=1) for r in range(2)]
    assert sum(r["count"] for r in reps) == 64
    for r in reps:
        assert r["seconds"] > 0 and r["matrices_per_s"] > 0
        assert sum(r["count_of_class"]) == r["count"]
        for c in range(6):
            if r["count_of_class"][c]:
                assert 0 < r["p50_ms"][c] <= r["p99_ms"][c] <= r["seconds"] * 1e3 * 1.01


def test_library_autotune_picks_a_candidate():
    ns, algs = B.batch_sizes(40, 6)
    choice, timings = B.autotune(torch, ns, algs, reps=1, seed=6)
    for c, bs in choice.items():
        assert bs in B.CANDIDATE_BS and bs <= max(64, B.CLASS_EDGES[c + 1])
        assert timings[(c, bs)] == min(t for (cc, _), t in timings.items() if cc == c)
