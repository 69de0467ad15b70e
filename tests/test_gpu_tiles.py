"""GPU parity of the single-tile kernels (the reference's tile-kernel ABI) against the
oracle's restated tile kernels and LAPACK-equivalent numpy references (normwise 1e-12)."""
import ctypes

import numpy as np
import pytest

import palial_gb300 as P
from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def dev(x):
    return torch.from_numpy(np.asfortranarray(x).ravel(order="F").copy()).cuda()


def host(t, nb):
    return t.cpu().numpy().reshape(nb, nb, order="F")


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


NB = [64, 256, 512]


@pytest.mark.parametrize("nb", NB)
def test_tile_potrf(nb):
    a = O.gen_spd(2, nb)
    d = dev(a)
    assert P.lib().palial_gpu_tile_dpotrf(nb, d.data_ptr(), nb) == 0
    torch.cuda.synchronize()
    u = np.triu(host(d, nb))
    assert rel(u, np.linalg.cholesky(a).T) <= 1e-12
    assert np.array_equal(np.tril(host(d, nb), -1), np.tril(a, -1))


@pytest.mark.parametrize("nb", NB)
def test_tile_getrf(nb):
    a = O.gen_uniform(3, nb) + nb * np.eye(nb)
    ref = np.asfortranarray(a.copy())
    O.lib().orc_dgetrf_nopiv(nb, ref.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), nb)
    d = dev(a)
    assert P.lib().palial_gpu_tile_dgetrf(nb, d.data_ptr(), nb) == 0
    assert rel(host(d, nb), ref) <= 1e-12


@pytest.mark.parametrize("nb", NB)
@pytest.mark.parametrize("kind", [0, 1, 2])
def test_tile_trsm(nb, kind):
    import scipy.linalg as sl
    t = O.gen_uniform(4, nb) + nb * np.eye(nb)
    b = O.gen_uniform(5, nb)
    db = dev(b)
    assert P.lib().palial_gpu_tile_dtrsm(kind, nb, dev(t).data_ptr(), db.data_ptr(), nb) == 0
    if kind == 0:
        ref = sl.solve_triangular(np.triu(t), b, trans="T", lower=False)
    elif kind == 1:
        ref = sl.solve_triangular(np.triu(t), b.T, trans="T", lower=False).T
    else:
        ref = sl.solve_triangular(np.tril(t, -1) + np.eye(nb), b, lower=True, unit_diagonal=True)
    assert rel(host(db, nb), ref) <= 1e-12


@pytest.mark.parametrize("nb", NB)
def test_tile_syrk_gemm(nb):
    a, b, c = O.gen_uniform(6, nb), O.gen_uniform(7, nb), O.gen_uniform(8, nb)
    dc = dev(c)
    assert P.lib().palial_gpu_tile_dsyrk(nb, dev(a).data_ptr(), dc.data_ptr(), nb) == 0
    got = host(dc, nb)
    ref = c - a.T @ a
    assert rel(np.triu(got), np.triu(ref)) <= 1e-12
    assert np.array_equal(np.tril(got, -1), np.tril(c, -1))
    for kind, ref in ((0, c - a.T @ b), (1, c - a @ b)):
        dc = dev(c)
        assert P.lib().palial_gpu_tile_dgemm(kind, nb, dev(a).data_ptr(), dev(b).data_ptr(), dc.data_ptr(), nb) == 0
        assert rel(host(dc, nb), ref) <= 1e-12


@pytest.mark.parametrize("nb", [64, 256])
def test_tile_qr_kernels(nb):
    dp = ctypes.POINTER(ctypes.c_double)
    L = O.lib()
    a = O.gen_uniform(9, nb)
    # GEQRT
    ra, rt, tau, work = np.asfortranarray(a.copy()), np.zeros((nb, nb), order="F"), np.zeros(nb), np.zeros(nb * nb)
    L.orc_dgeqrt(nb, ra.ctypes.data_as(dp), nb, rt.ctypes.data_as(dp), nb, tau.ctypes.data_as(dp), work.ctypes.data_as(dp))
    da, dt = dev(a), dev(np.zeros((nb, nb)))
    assert P.lib().palial_gpu_tile_dgeqrt(nb, da.data_ptr(), dt.data_ptr(), nb) == 0
    assert rel(host(da, nb), ra) <= 1e-12 and rel(np.triu(host(dt, nb)), np.triu(rt)) <= 1e-12
    # ORMQR on another tile with (V, T) from GEQRT
    c = O.gen_uniform(10, nb)
    rc = np.asfortranarray(c.copy())
    L.orc_dormqr(nb, ra.ctypes.data_as(dp), nb, rt.ctypes.data_as(dp), nb, rc.ctypes.data_as(dp), nb, work.ctypes.data_as(dp))
    dc = dev(c)
    assert P.lib().palial_gpu_tile_dormqr(nb, dev(ra).data_ptr(), dev(rt).data_ptr(), dc.data_ptr(), nb) == 0
    assert rel(host(dc, nb), rc) <= 1e-12
    # TSQRT on [R; A2]
    a2 = O.gen_uniform(11, nb)
    r1, r2, t2 = np.asfortranarray(ra.copy()), np.asfortranarray(a2.copy()), np.zeros((nb, nb), order="F")
    L.orc_dtsqrt(nb, r1.ctypes.data_as(dp), nb, r2.ctypes.data_as(dp), nb, t2.ctypes.data_as(dp), nb,
                 tau.ctypes.data_as(dp), work.ctypes.data_as(dp))
    d1, d2, dt2 = dev(ra), dev(a2), dev(np.zeros((nb, nb)))
    assert P.lib().palial_gpu_tile_dtsqrt(nb, d1.data_ptr(), d2.data_ptr(), dt2.data_ptr(), nb) == 0
    assert rel(host(d1, nb), r1) <= 1e-12 and rel(host(d2, nb), r2) <= 1e-12
    assert rel(np.triu(host(dt2, nb)), np.triu(t2)) <= 1e-12
    # TSMQR with (V, T) from TSQRT
    b1, b2 = O.gen_uniform(12, nb), O.gen_uniform(13, nb)
    s1, s2 = np.asfortranarray(b1.copy()), np.asfortranarray(b2.copy())
    L.orc_dtsmqr(nb, s1.ctypes.data_as(dp), nb, s2.ctypes.data_as(dp), nb, r2.ctypes.data_as(dp), nb,
                 t2.ctypes.data_as(dp), nb, work.ctypes.data_as(dp))
    e1, e2 = dev(b1), dev(b2)
    assert P.lib().palial_gpu_tile_dtsmqr(nb, e1.data_ptr(), e2.data_ptr(), dev(r2).data_ptr(), dev(t2).data_ptr(), nb) == 0
    assert rel(host(e1, nb), s1) <= 1e-12 and rel(host(e2, nb), s2) <= 1e-12


def test_generators_bitwise_equal_to_oracle():
    for n, nb in ((192, 64), (512, 128), (1024, 512)):
        d = torch.empty(n * n, dtype=torch.float64, device="cuda")
        P.gen_uniform(d.data_ptr(), n, nb, 1)
        torch.cuda.synchronize()
        assert np.array_equal(d.cpu().numpy(), O.to_tiles(O.gen_uniform(1, n), nb))
        P.gen_spd(d.data_ptr(), n, nb, 0)
        torch.cuda.synchronize()
        assert np.array_equal(d.cpu().numpy(), O.to_tiles(O.gen_spd(0, n), nb))
    # the benchmarks' right-hand sides: column-major n x 16
    r = torch.empty(1024 * 16, dtype=torch.float64, device="cuda")
    P.gen_dense(r.data_ptr(), 1024, 16, 5, P.STREAM_RHS)
    torch.cuda.synchronize()
    assert np.array_equal(r.cpu().numpy(), O.gen_uniform(5, 1024, 16, stream=O.STREAM_RHS).ravel(order="F"))
