"""Mixed-precision QR solve: the reference's flat-tree TS QR computed in FP32 by the FP32 task
scheduler, FP64 refinement, FP64 QR solve when the refinement stalls."""
import numpy as np
import pytest

import palial_gb300 as P
from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _solve(a, b, nb, **kw):
    n, nrhs = a.shape[0], b.shape[1]
    da = torch.from_numpy(O.to_tiles(a, nb)).cuda()
    db = torch.from_numpy(np.ascontiguousarray(b.T).ravel()).cuda()
    dx = torch.full((n * nrhs,), float("nan"), dtype=torch.float64, device="cuda")
    kw.setdefault("timeout_s", 10.0)
    st = P.qr_solve_ir(da.data_ptr(), n, nb, db.data_ptr(), dx.data_ptr(), nrhs, **kw)
    return st, dx.cpu().numpy().reshape(nrhs, n).T


def _berr(a, x, b):
    r = b - a @ x
    return (np.abs(r).max(axis=0) / (np.abs(a).sum(axis=1).max() * np.abs(x).max(axis=0) + np.abs(b).max(axis=0))).max()


@pytest.mark.parametrize("n,nb,nrhs", [(512, 128, 1), (1024, 256, 4), (2048, 512, 16), (768, 64, 3)])
def test_fp32_qr_refined_to_fp64_backward_error(n, nb, nrhs):
    rng = np.random.default_rng(n)
    a = rng.uniform(-1, 1, (n, n))
    b = rng.uniform(-1, 1, (n, nrhs))
    st, x = _solve(a, b, nb)
    assert st.code == 0 and st.precision_used == 5, st.message  # FP32 QR sufficed
    assert 1 <= st.ir_iters <= 30
    assert st.backward_error <= 1e-14 * n
    assert _berr(a, x, b) <= 1e-14 * n
    xr = np.linalg.solve(a, b)
    assert np.linalg.norm(x - xr) <= 1e-8 * np.linalg.norm(xr)


@pytest.mark.parametrize("n,nb,nrhs", [(1024, 256, 4), (2048, 512, 16)])
def test_tensor_core_tsmqr_refined_to_fp64_backward_error(n, nb, nrhs):
    """TSMQR's products with V on the warp tensor cores (BF16x3, precision="bf16x3"): the FP32
    factors are a little less accurate, the refinement still reaches the FP64-level target from
    them without the FP64 fallback, and the solution matches numpy's."""
    rng = np.random.default_rng(n + 1)
    a = rng.uniform(-1, 1, (n, n))
    b = rng.uniform(-1, 1, (n, nrhs))
    st, x = _solve(a, b, nb, precision="bf16x3")
    assert st.code == 0 and st.precision_used == 3, st.message  # the tensor-core form sufficed
    assert st.backward_error <= 1e-14 * n and _berr(a, x, b) <= 1e-14 * n
    xr = np.linalg.solve(a, b)
    assert np.linalg.norm(x - xr) <= 1e-8 * np.linalg.norm(xr)
    st32, _ = _solve(a, b, nb)
    print(f"n={n}: tensor-core TSMQR {st.ir_iters} refinement steps, factor {st.factor_seconds:.4f} s; "
          f"FP32 {st32.ir_iters} steps, factor {st32.factor_seconds:.4f} s")


def test_ill_conditioned_system_falls_back_to_fp64_qr():
    n, nb = 512, 128
    rng = np.random.default_rng(9)
    q1 = np.linalg.qr(rng.standard_normal((n, n)))[0]
    q2 = np.linalg.qr(rng.standard_normal((n, n)))[0]
    a = (q1 * 1e10 ** (-np.arange(n) / (n - 1))) @ q2.T
    b = rng.uniform(-1, 1, (n, 2))
    st, x = _solve(a, b, nb)
    assert st.code == 0 and st.precision_used == 0, st.message  # the FP64 QR solve produced X
    assert _berr(a, x, b) <= 1e-14 * n


def test_bad_arguments():
    with pytest.raises(P.PalialError):
        P.qr_solve_ir(1 << 20, 512, 96, 1 << 20, 1 << 20, 1)
    with pytest.raises(P.PalialError):
        P.qr_solve_ir(1 << 20, 512, 128, 1 << 20, 1 << 20, 17)


def _dev32(x):
    return torch.from_numpy(np.asfortranarray(x).ravel(order="F").astype(np.float32)).cuda()


def _host(t, nb):
    return t.cpu().numpy().astype(np.float64).reshape(nb, nb, order="F")


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("nb", [64, 256, 512])
def test_fp32_qr_tile_kernels_match_the_oracle(nb):
    """The FP32 tile routines against the oracle's FP64 restatement of the reference's tile
    kernels (same inputs rounded to FP32; FP32 tolerance)."""
    import ctypes
    dp = ctypes.POINTER(ctypes.c_double)
    L = O.lib()
    lib = P.lib()
    a = O.gen_uniform(9, nb).astype(np.float32).astype(np.float64)
    ra, rt, tau, work = np.asfortranarray(a.copy()), np.zeros((nb, nb), order="F"), np.zeros(nb), np.zeros(nb * nb)
    L.orc_dgeqrt(nb, ra.ctypes.data_as(dp), nb, rt.ctypes.data_as(dp), nb, tau.ctypes.data_as(dp), work.ctypes.data_as(dp))
    da, dt = _dev32(a), _dev32(np.zeros((nb, nb)))
    assert lib.palial_gpu_tile_sgeqrt(nb, da.data_ptr(), dt.data_ptr(), nb) == 0
    # the backward error of the GPU's own factors: Q R = A and Q^T Q = I to a small multiple of
    # u_32 (measured at most 1.4e-6 at nb = 512), and the factors against the oracle's
    g, gt = _host(da, nb), np.triu(_host(dt, nb))
    v = np.tril(g, -1) + np.eye(nb)
    q = np.eye(nb) - v @ gt @ v.T
    back = _rel(q @ np.triu(g), a)
    orth = np.linalg.norm(q.T @ q - np.eye(nb)) / np.sqrt(nb)
    fwd_r, fwd_t = _rel(g, ra), _rel(gt, np.triu(rt))
    print(f"nb={nb}: GEQRT backward {back:.2e}, orthogonality {orth:.2e}, forward R/V {fwd_r:.2e}, T {fwd_t:.2e}")
    assert back <= 1e-5 and orth <= 1e-5, (back, orth)
    assert fwd_r <= 2e-5 and fwd_t <= 2e-5  # measured at most 2.7e-6 (nb = 512)
    c = O.gen_uniform(10, nb).astype(np.float32).astype(np.float64)
    rc = np.asfortranarray(c.copy())
    L.orc_dormqr(nb, ra.ctypes.data_as(dp), nb, rt.ctypes.data_as(dp), nb, rc.ctypes.data_as(dp), nb, work.ctypes.data_as(dp))
    dc = _dev32(c)
    assert lib.palial_gpu_tile_sormqr(nb, _dev32(ra).data_ptr(), _dev32(rt).data_ptr(), dc.data_ptr(), nb) == 0
    e_orm = _rel(_host(dc, nb), rc)  # applying a given Q is forward stable: ~ u_32
    print(f"nb={nb}: ORMQR {e_orm:.2e}")
    assert e_orm <= 1e-5, e_orm
    a2 = O.gen_uniform(11, nb).astype(np.float32).astype(np.float64)
    r1, r2, t2 = np.asfortranarray(ra.copy()), np.asfortranarray(a2.copy()), np.zeros((nb, nb), order="F")
    L.orc_dtsqrt(nb, r1.ctypes.data_as(dp), nb, r2.ctypes.data_as(dp), nb, t2.ctypes.data_as(dp), nb,
                 tau.ctypes.data_as(dp), work.ctypes.data_as(dp))
    d1, d2, dt2 = _dev32(ra), _dev32(a2), _dev32(np.zeros((nb, nb)))
    assert lib.palial_gpu_tile_stsqrt(nb, d1.data_ptr(), d2.data_ptr(), dt2.data_ptr(), nb) == 0
    # backward error of the TS factorization: Q [R1; 0] = [R_in; A2] with Q = I - [I; V] T [I; V]^T
    g1, g2, gt2 = np.triu(_host(d1, nb)), _host(d2, nb), np.triu(_host(dt2, nb))
    w = np.vstack([np.eye(nb), g2])
    q2 = np.eye(2 * nb) - w @ gt2 @ w.T
    back2 = np.linalg.norm(q2 @ np.vstack([g1, np.zeros((nb, nb))]) - np.vstack([np.triu(ra), a2])) / \
        np.linalg.norm(np.vstack([np.triu(ra), a2]))
    print(f"nb={nb}: TSQRT backward {back2:.2e}, forward R {_rel(g1, np.triu(r1)):.2e}")
    assert back2 <= 1e-5, back2
    assert _rel(_host(d1, nb), r1) <= 2e-5 and _rel(g2, r2) <= 1e-4 and _rel(gt2, np.triu(t2)) <= 1e-4
    b1 = O.gen_uniform(12, nb).astype(np.float32).astype(np.float64)
    b2 = O.gen_uniform(13, nb).astype(np.float32).astype(np.float64)
    s1, s2 = np.asfortranarray(b1.copy()), np.asfortranarray(b2.copy())
    L.orc_dtsmqr(nb, s1.ctypes.data_as(dp), nb, s2.ctypes.data_as(dp), nb, r2.ctypes.data_as(dp), nb,
                 t2.ctypes.data_as(dp), nb, work.ctypes.data_as(dp))
    e1, e2 = _dev32(b1), _dev32(b2)
    assert lib.palial_gpu_tile_stsmqr(nb, e1.data_ptr(), e2.data_ptr(), _dev32(r2).data_ptr(), _dev32(t2).data_ptr(),
                                      nb) == 0
    e_ts = max(_rel(_host(e1, nb), s1), _rel(_host(e2, nb), s2))
    print(f"nb={nb}: TSMQR {e_ts:.2e}")
    assert e_ts <= 1e-5, e_ts
