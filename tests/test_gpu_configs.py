"""GPU parity at the benchmark configurations' own sizes, through the host-buffer C ABI (the
drop-in entry points palial_gpu_cholesky / lu / qr).

* Cholesky N = 4096, NB = 512 on A = B B^T + N I (seed 0): the factor against the oracle's
  (the reference's algorithm over OpenBLAS, program order), normwise <= 1e-12, and the
  elementwise maximum difference relative to max |U| reported and bounded.
* LU N = 4096, NB = 512: on a diagonally dominant input normwise <= 1e-12 against the oracle;
  on the uniform [-1, 1) input of the FP64 configuration (seed 1) the backward error against
  the oracle's own (no pivoting: no ordering-independent factor exists).  Pivots bit-exact
  (identity, as the reference never pivots, src/srclu/dgetrf.h:17-23).
* QR N = 4096, NB = 512 (uniform, seed 1): R/V and T normwise <= 1e-12 against the oracle,
  ||Q^T A - R|| / ||A|| and ||Q^T Q - I|| / sqrt(N).
* N = 16384, NB = 512, FP64, every algorithm, against the oracle run as OpenMP tasks: Cholesky
  and QR factors normwise <= 1e-12; random-probe residuals computed here with numpy from the
  returned factors (||A X - F(X)|| / ||A X||); LU identity pivots and a probe within 10x of
  the oracle's; QR probes ||Q^T A X - R X|| / ||A X|| and | ||Q^T X|| / ||X|| - 1 |.
"""
import os

import numpy as np
import pytest

import palial_gb300 as P
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def dominant(seed, n):
    a = np.full((n, n), 0.5)
    u = (O.gen_uniform(seed, n, 1)[:, 0] + 1.0) * 0.5
    a[np.diag_indices(n)] = 173.0 * u + 173.0
    return a


def test_config1_cholesky_4096_matches_oracle(record_property):
    n, nb = 4096, 512
    a = O.gen_spd(0, n)
    ref = O.to_tiles(a, nb)
    O.run("cholesky", ref, n, nb)
    got = O.to_tiles(a, nb)
    P.cholesky(got, n, nb)
    nrm = rel(got, ref)
    u_ref = np.triu(O.from_tiles(ref, n, nb))
    u_got = np.triu(O.from_tiles(got, n, nb))
    elem = float(np.max(np.abs(u_got - u_ref)) / np.max(np.abs(u_ref)))
    record_property("normwise", nrm)
    record_property("elementwise_max_rel", elem)
    print(f"config 1 Cholesky 4096/512: normwise {nrm:.3e}, elementwise max |dU| / max |U| {elem:.3e}")
    assert nrm <= 1e-12
    assert elem <= 1e-12
    assert O.cholesky_residual(a, u_got) <= 1e-15


def test_lu_4096_dominant_matches_oracle():
    n, nb = 4096, 512
    a = dominant(3, n)
    ref = O.to_tiles(a, nb)
    O.run("lu", ref, n, nb)
    got = O.to_tiles(a, nb)
    _, ipiv = P.lu(got, n, nb)
    assert np.array_equal(ipiv, np.arange(1, n + 1, dtype=np.int32))
    assert rel(got, ref) <= 1e-12
    assert O.lu_residual(a, O.from_tiles(got, n, nb)) <= 1e-15


def test_lu_4096_uniform_backward_error():
    n, nb = 4096, 512
    a = O.gen_uniform(1, n)
    ref = O.to_tiles(a, nb)
    O.run("lu", ref, n, nb)
    got = O.to_tiles(a, nb)
    _, ipiv = P.lu(got, n, nb)
    assert np.array_equal(ipiv, np.arange(1, n + 1, dtype=np.int32))
    be_gpu = O.lu_residual(a, O.from_tiles(got, n, nb))
    be_ref = O.lu_residual(a, O.from_tiles(ref, n, nb))
    print(f"LU 4096 uniform: backward error GPU {be_gpu:.3e}, oracle {be_ref:.3e}, distance {rel(got, ref):.3e}")
    assert be_gpu <= max(10 * be_ref, 1e-13), (be_gpu, be_ref)


def test_qr_4096_matches_oracle():
    n, nb = 4096, 512
    a = O.gen_uniform(1, n)
    ref, sref = O.to_tiles(a, nb), np.zeros(n * n)
    O.run("qr", ref, n, nb, sref)
    got, s = O.to_tiles(a, nb), np.zeros(n * n)
    P.qr(got, s, n, nb)
    assert rel(got, ref) <= 1e-12
    f_got, s_got, s_ref = O.from_tiles(got, n, nb), O.from_tiles(s, n, nb), O.from_tiles(sref, n, nb)
    # T factors: only the upper triangle of each tile of S is defined
    mt = n // nb
    blk = lambda i: slice(i * nb, (i + 1) * nb)  # noqa: E731
    num = den = 0.0
    for m in range(mt):
        for k in range(mt):
            tr = np.triu(s_ref[blk(m), blk(k)])
            tg = np.triu(s_got[blk(m), blk(k)])
            num += np.sum((tg - tr) ** 2)
            den += np.sum(tr ** 2)
    assert np.sqrt(num / den) <= 1e-12
    res, orth = O.qr_checks(a, f_got, s_got, nb)
    print(f"QR 4096: ||Q^T A - R||/||A|| {res:.3e}, ||Q^T Q - I||/sqrt(N) {orth:.3e}")
    assert res <= 1e-14 and orth <= 1e-14


def _probe(n, k=4, seed=11):
    return np.random.default_rng(seed).uniform(-1, 1, (n, k))


@pytest.mark.parametrize("alg", ["cholesky", "lu", "qr"])
def test_config2_fp64_16384(alg):
    """Full-size FP64 factorizations against the oracle run as OpenMP tasks on every host core
    (the reference's dependences, so each tile's updates keep program order: the same result as
    the serial oracle)."""
    n, nb = 16384, 512
    threads = os.cpu_count() or 1
    a = O.gen_spd(0, n) if alg == "cholesky" else O.gen_uniform(1, n)
    t, ref = O.to_tiles(a, nb), O.to_tiles(a, nb)
    s = np.zeros(n * n) if alg == "qr" else None
    sref = np.zeros(n * n) if alg == "qr" else None
    O.run(alg, ref, n, nb, sref, nthreads=threads)
    x = _probe(n)
    ax = a @ x
    if alg == "cholesky":
        st = P.cholesky(t, n, nb)
        u = np.triu(O.from_tiles(t, n, nb))
        r = np.linalg.norm(ax - u.T @ (u @ x)) / np.linalg.norm(ax)
        d = rel(t, ref)
        print(f"Cholesky 16384 FP64: {st.tflops:.3f} TFLOP/s, probe {r:.3e}, distance to oracle {d:.3e}")
        assert d <= 1e-12 and r <= 1e-14
        return
    if alg == "lu":
        st, ipiv = P.lu(t, n, nb)
        assert np.array_equal(ipiv, np.arange(1, n + 1, dtype=np.int32))

        def probe(buf):
            f = O.from_tiles(buf, n, nb)
            ux = np.triu(f) @ x
            return np.linalg.norm(ax - (np.tril(f, -1) @ ux + ux)) / np.linalg.norm(ax)

        r, r_ref = probe(t), probe(ref)
        print(f"LU 16384 FP64 (uniform, no pivoting): {st.tflops:.3f} TFLOP/s, probe {r:.3e}, oracle's {r_ref:.3e}")
        # no pivoting on a uniform random matrix: element growth sets both backward errors
        assert r <= max(10 * r_ref, 1e-13), (r, r_ref)
        return
    st = P.qr(t, s, n, nb)
    d = rel(t, ref)
    f, sf = O.from_tiles(t, n, nb), O.from_tiles(s, n, nb)
    qtax = O.qr_apply_qt(f, sf, nb, ax)
    r = np.linalg.norm(qtax - O.r_factor(f, nb) @ x) / np.linalg.norm(ax)
    qtx = O.qr_apply_qt(f, sf, nb, x)
    orth = float(np.max(np.abs(np.linalg.norm(qtx, axis=0) / np.linalg.norm(x, axis=0) - 1.0)))
    print(f"QR 16384 FP64: {st.tflops:.3f} TFLOP/s, distance to oracle {d:.3e}, "
          f"||Q^T A X - R X|| / ||A X|| {r:.3e}, norm drift {orth:.3e}")
    assert d <= 1e-12 and r <= 1e-14 and orth <= 1e-13
