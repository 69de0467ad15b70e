"""GPU parity: whole factorizations through the C ABI against the CPU oracle (the
reference's algorithm over OpenBLAS) and the reference-made golden fixtures.

Tolerances (normwise, ||X_gpu - X_ref||_F / ||X_ref||_F): Cholesky and QR 1e-12; LU on
dominant inputs 1e-12; LU on uniform random inputs has no ordering-independent answer
(no pivoting), so it is gated by backward error and identity pivots."""
import json
import os

import numpy as np
import pytest

import palial_gb300 as P
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def dominant(seed, n):
    a = np.full((n, n), 0.5)
    u = (O.gen_uniform(seed, n, 1)[:, 0] + 1.0) * 0.5
    a[np.diag_indices(n)] = 173.0 * u + 173.0
    return a


def oracle_factor(alg, a, nb):
    n = a.shape[0]
    t = O.to_tiles(a, nb)
    s = np.zeros_like(t) if alg == "qr" else None
    O.run(alg, t, n, nb, s)
    return t, s


def gpu_factor(alg, a, nb, **kw):
    n = a.shape[0]
    t = O.to_tiles(a, nb)
    if alg == "cholesky":
        st = P.cholesky(t, n, nb, **kw)
        return t, None, st
    if alg == "lu":
        st, ipiv = P.lu(t, n, nb, **kw)
        assert np.array_equal(ipiv, np.arange(1, n + 1, dtype=np.int32))
        return t, None, st
    s = np.zeros_like(t)
    st = P.qr(t, s, n, nb, **kw)
    return t, s, st


def upper_s(s, n, nb):
    """T factors: only the upper triangles of the S tiles are defined."""
    mt = n // nb
    x = s.reshape(mt, mt, nb, nb).copy()  # [tile n][tile m][col][row]
    for i in range(mt):
        for j in range(mt):
            x[i, j] = np.tril(x[i, j])       # row <= col
    return x.ravel()


@pytest.mark.parametrize("n,nb,bs", [(192, 64, 64), (1024, 256, 128), (1024, 256, 256), (2048, 512, 256),
                                     (2048, 512, 512), (512, 512, 512), (1024, 512, 256)])
def test_cholesky_matches_oracle(n, nb, bs):
    a = O.gen_spd(0, n)
    ref, _ = oracle_factor("cholesky", a, nb)
    got, _, st = gpu_factor("cholesky", a, nb, block=bs)
    assert rel(got, ref) <= 1e-12
    assert O.cholesky_residual(a, O.from_tiles(got, n, nb)) <= 1e-15
    # lower tiles untouched, as the reference leaves them
    F, A0 = O.from_tiles(got, n, nb), a
    for k in range(n // nb):
        for m in range(k + 1, n // nb):
            assert np.array_equal(F[m * nb:(m + 1) * nb, k * nb:(k + 1) * nb], A0[m * nb:(m + 1) * nb, k * nb:(k + 1) * nb])


@pytest.mark.parametrize("n,nb,bs", [(128, 64, 64), (1024, 256, 256), (2048, 512, 256), (1024, 512, 512)])
def test_lu_dominant_matches_oracle(n, nb, bs):
    a = dominant(3, n)
    ref, _ = oracle_factor("lu", a, nb)
    got, _, _ = gpu_factor("lu", a, nb, block=bs)
    assert rel(got, ref) <= 1e-12
    assert O.lu_residual(a, O.from_tiles(got, n, nb)) <= 1e-15


@pytest.mark.parametrize("n,nb,bs", [(256, 64, 64), (1024, 256, 256), (2048, 512, 256)])
def test_lu_uniform_backward_error(n, nb, bs):
    a = O.gen_uniform(1, n)
    ref, _ = oracle_factor("lu", a, nb)
    got, _, _ = gpu_factor("lu", a, nb, block=bs)
    be_gpu = O.lu_residual(a, O.from_tiles(got, n, nb))
    be_ref = O.lu_residual(a, O.from_tiles(ref, n, nb))
    # same order of magnitude as the reference's own backward error (no pivoting: growth)
    assert be_gpu <= max(10 * be_ref, 1e-13), (be_gpu, be_ref)
    assert rel(got, ref) < 1e-3  # reported distance; no ordering-independent bound exists


@pytest.mark.parametrize("n,nb", [(128, 64), (512, 128), (1024, 256), (1024, 512)])
def test_qr_matches_oracle(n, nb):
    a = O.gen_uniform(1, n)
    ref, sref = oracle_factor("qr", a, nb)
    got, s, _ = gpu_factor("qr", a, nb)
    assert rel(got, ref) <= 1e-12
    assert rel(upper_s(s, n, nb), upper_s(sref, n, nb)) <= 1e-12
    res, orth = O.qr_checks(a, O.from_tiles(got, n, nb), O.from_tiles(s, n, nb), nb)
    assert res <= 1e-14 and orth <= 1e-14


@pytest.mark.parametrize("name", ["chol_192_64", "lu_dom_128_32", "qr_192_64", "lu_192_64"])
def test_against_reference_golden(name):
    """Factors of the reference itself (golden fixtures made from the reference's sources)."""
    meta = json.load(open(os.path.join(GOLD, "sha256.json")))[name]
    n, nb, alg = meta["n"], meta["nb"], meta["alg"]
    if nb % 64:
        pytest.skip("the GPU path needs NB to be a multiple of 64")
    g = np.load(os.path.join(GOLD, name + ".npz"))
    a = O.gen_spd(0, n) if alg == "cholesky" else O.gen_uniform(1, n)
    got, s, _ = gpu_factor(alg, a, nb)
    if name == "lu_192_64":
        assert O.lu_residual(a, O.from_tiles(got, n, nb)) <= 1e-12
        return
    assert rel(got, g["out_tiles"]) <= 1e-12
    if s is not None:
        assert rel(upper_s(s, n, nb), upper_s(g["s_tiles"], n, nb)) <= 1e-12


@pytest.mark.parametrize("alg", ["cholesky", "lu", "qr"])
def test_schedule_independence_bitwise(alg):
    """Every object's updates are applied in k order: any dispatch order / worker count gives
    the same bits."""
    n, nb = 2048, 256
    a = O.gen_spd(0, n) if alg == "cholesky" else dominant(4, n)
    base, bs_, _ = gpu_factor(alg, a, nb, block=128 if alg != "qr" else 0)
    for kw in ({"priority": 1}, {"shuffle_seed": 11}, {"shuffle_seed": 12, "max_sms": 7}, {"max_sms": 1}):
        got, s, _ = gpu_factor(alg, a, nb, block=128 if alg != "qr" else 0, **kw)
        assert np.array_equal(got, base), kw
        if s is not None:
            assert np.array_equal(s, bs_), kw


def test_identity_and_single_tile():
    for n, nb in ((64, 64), (128, 64), (512, 512)):
        a = np.eye(n)
        for alg in ("cholesky", "lu"):
            got, _, _ = gpu_factor(alg, a, nb)
            assert np.array_equal(O.from_tiles(got, n, nb), a)


def test_not_spd_reports_error():
    n, nb = 512, 128
    a = O.gen_spd(0, n)
    a[300, 300] = -1.0
    with pytest.raises(P.PalialError) as e:
        gpu_factor("cholesky", a, nb)
    assert e.value.code == -3


def test_zero_pivot_warns_like_reference():
    n, nb = 256, 64
    a = dominant(1, n)
    a[0, 0] = 0.0
    got, _, st = gpu_factor("lu", a, nb)
    assert st.code == 1  # PALIAL_WARN_ZERO_PIVOT, computation continued as in the reference


def test_bad_arguments():
    with pytest.raises(P.PalialError):
        P.cholesky(np.zeros(1000 * 1000), 1000, 512)


def test_dependency_timeout_is_reported_not_hung():
    """Record 5 also waits on a counter that nothing signals; the wait must end by deadline
    with PALIAL_ERR_TIMEOUT and the context stays usable."""
    n, nb = 1024, 256
    a = O.gen_spd(0, n)
    t = O.to_tiles(a, nb)
    o = P.make_opts(timeout_s=0.5)
    o.reserved[0] = 6
    st = P.Status()
    rc = P.lib().palial_gpu_cholesky(P.ctypes.byref(P.desc(t, n, nb)), P.ctypes.byref(o), P.ctypes.byref(st))
    assert rc == -4, (rc, st.message)
    got, _, _ = gpu_factor("cholesky", a, nb)  # still works afterwards
    ref, _ = oracle_factor("cholesky", a, nb)
    assert rel(got, ref) <= 1e-12


def test_trace_names_equal_reference_published_trace(tmp_path):
    """Device trace of Cholesky N=8192 NB=512 (block = tile): one `name, ms` line per task in
    the reference's creation order, the same names as its own published trace
    (exp/data/tasks_times_8192_512_31_ondemand), every duration positive and finite."""
    import torch
    n, nb = 8192, 512
    a = torch.empty(n * n, dtype=torch.float64, device="cuda")
    P.gen_spd(a.data_ptr(), n, nb, 0)
    P.factor_dev("cholesky", a.data_ptr(), None, n, nb, block=nb, trace=True)
    out = tmp_path / "trace.txt"
    P.trace_dump(str(out))
    lines = out.read_text().splitlines()
    gold = open(os.path.join(GOLD, "trace_names_cholesky_8192_512.txt")).read().split()
    assert [ln.split(",")[0] for ln in lines] == gold
    ms = np.array([float(ln.split(",")[1]) for ln in lines])
    assert np.all(np.isfinite(ms)) and np.all(ms > 0)
