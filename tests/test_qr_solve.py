"""Linear solve and least squares through the tile QR: DAG structure (host), the oracle's
solve path against LAPACK-based numpy, and on the GPU the one-launch QR solve against the
oracle (square: the reference's QR algorithm over OpenBLAS, then Q^T b and back-substitution)
and against numpy's least squares (tall: no reference counterpart).

Tolerances: normwise ||X - X_ref|| / ||X_ref|| <= 1e-10 (uniform random A, kappa ~ 1e3-1e4
at these sizes, so 1e-10 leaves two orders of magnitude over kappa * u); residual norms of
least squares <= 1e-10 relative; backward error ||A X - B|| / (||A|| ||X|| + ||B||) <= 1e-13 (N = 8192)."""
import numpy as np
import pytest

import palial_gb300 as P
from oracle import oracle as O


def expected_counts(mt, nt):
    return {
        8: nt,                                                     # GEQRT
        9: nt * (nt - 1) // 2 + nt,                                # UNMQR (trailing + RHS)
        10: sum(mt - 1 - k for k in range(nt)),                    # TSQRT
        11: sum((mt - 1 - k) * (nt - 1 - k) + (mt - 1 - k) for k in range(nt)),  # TSMQR
        12: nt,                                                    # TRSM (R X = Y)
        7: nt * (nt - 1) // 2,                                     # GEMM (Y_i -= R_ik X_k)
    }


@pytest.mark.parametrize("rows,cols,nb,nrhs", [(512, 512, 128, 1), (1024, 512, 128, 16), (2048, 256, 256, 70),
                                               (768, 768, 256, 256), (4096, 4096, 512, 16)])
def test_qr_solve_dag_valid_and_counts(rows, cols, nb, nrhs):
    for seed in (0, 3):
        d = P.qr_solve_dag(rows, cols, nb, nrhs, nworkers=37, seed=seed)
        assert d["records"] > 0, d["message"]
    c = d["type_counts"]
    mt, nt = rows // nb, cols // nb
    for ty, want in expected_counts(mt, nt).items():
        assert c[ty] == want, (ty, c[ty], want)
    parts, rparts = nb // 64, (nrhs + 63) // 64
    recs = (nt + c[10] + (nt * (nt - 1) // 2) * parts + nt * rparts
            + sum((mt - 1 - k) * (nt - 1 - k) for k in range(nt)) * parts + sum(mt - 1 - k for k in range(nt)) * rparts
            + nt * rparts + c[7] * rparts)
    assert d["records"] == recs


@pytest.mark.parametrize("rows,cols,nb,nrhs", [(256, 512, 128, 1), (512, 512, 96, 1), (512, 512, 128, 0),
                                               (512, 512, 128, 129)])
def test_qr_solve_dag_rejects_bad_sizes(rows, cols, nb, nrhs):
    assert P.qr_solve_dag(rows, cols, nb, nrhs)["records"] == -1


@pytest.mark.parametrize("n,nb,nrhs", [(512, 128, 1), (1024, 256, 16), (4096, 512, 16), (768, 128, 70)])
def test_qr_apply_dag_valid_and_counts(n, nb, nrhs):
    """The refinement steps' DAG: Q^T on the extra tile column and the back-substitution only
    (no GEQRT/TSQRT, no update of the factor tiles), deadlock-free under ticket dispatch."""
    for seed in (0, 5):
        d = P.qr_apply_dag(n, nb, nrhs, nworkers=41, seed=seed)
        assert d["records"] > 0, d["message"]
    c = d["type_counts"]
    mt, rparts = n // nb, (nrhs + 63) // 64
    # GEQRT 8, UNMQR 9, TSQRT 10, TSMQR 11, TRSM_LUN 12, GEMM_NN 7
    assert c[8] == 0 and c[10] == 0
    assert c[9] == mt and c[11] == mt * (mt - 1) // 2
    assert c[12] == mt and c[7] == mt * (mt - 1) // 2
    assert sum(c) == c[7] + c[9] + c[11] + c[12]
    assert d["records"] == rparts * sum(c)
    assert P.qr_apply_dag(n, nb, 0)["records"] == -1


def test_oracle_qr_solve_matches_lapack():
    """The oracle's solve path (reference QR algorithm, then Q^T b and R back-substitution)
    against numpy's LAPACK solve."""
    n, nb = 384, 64
    a = O.gen_uniform(1, n)
    b = O.gen_uniform(2, n, 4)
    t = O.to_tiles(a, nb)
    s = np.zeros_like(t)
    O.run("qr", t, n, nb, s)
    f, sf = O.from_tiles(t, n, nb), O.from_tiles(s, n, nb)
    x, r = O.qr_solve(f, sf, nb, b)
    xr = np.linalg.solve(a, b)
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-11
    assert np.all(r == 0)


def test_rect_tiles_roundtrip():
    a = O.gen_uniform(5, 384, 192)
    t = O.to_tiles(a, 64)
    assert np.array_equal(O.from_tiles(t, 384, 64, 192), a)
    # tile (m, n) at element nb*nb*(m + mt*n), column-major inside
    assert t[64 * 64 * (2 + 6 * 1) + 3 + 64 * 5] == a[2 * 64 + 3, 64 + 5]


def _gpu_solve(a, nb, b):
    import torch
    rows, cols = a.shape
    nrhs = b.shape[1]
    da = torch.from_numpy(O.to_tiles(a, nb)).cuda()
    db = torch.from_numpy(np.asfortranarray(b).ravel(order="F")).cuda()
    dx = torch.zeros(cols * nrhs, dtype=torch.float64, device="cuda")
    dr = torch.zeros(nrhs, dtype=torch.float64, device="cuda")
    st = P.qr_solve(da.data_ptr(), rows, cols, nb, db.data_ptr(), dx.data_ptr(), nrhs, dr.data_ptr())
    x = dx.cpu().numpy().reshape(nrhs, cols).T
    return x, dr.cpu().numpy(), st


@pytest.mark.gpu
@pytest.mark.parametrize("n,nb,nrhs", [(512, 128, 1), (1024, 256, 16), (768, 256, 256), (1024, 512, 70)])
def test_gpu_qr_solve_square_matches_oracle(n, nb, nrhs):
    a = O.gen_uniform(1, n)
    b = O.gen_uniform(2, n, nrhs)
    t = O.to_tiles(a, nb)
    s = np.zeros_like(t)
    O.run("qr", t, n, nb, s)
    xo, _ = O.qr_solve(O.from_tiles(t, n, nb), O.from_tiles(s, n, nb), nb, b)
    x, r, st = _gpu_solve(a, nb, b)
    assert st.code == 0
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-10
    assert np.all(r == 0.0)


@pytest.mark.gpu
@pytest.mark.parametrize("rows,cols,nb,nrhs", [(1536, 512, 256, 5), (2048, 1024, 128, 64), (1024, 256, 256, 1)])
def test_gpu_least_squares_matches_numpy(rows, cols, nb, nrhs):
    a = O.gen_uniform(3, rows, cols)
    b = O.gen_uniform(4, rows, nrhs)
    x, r, st = _gpu_solve(a, nb, b)
    assert st.code == 0
    xr, *_ = np.linalg.lstsq(a, b, rcond=None)
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-10
    rr = np.linalg.norm(a @ xr - b, axis=0)
    assert np.allclose(r, rr, rtol=1e-10)
    # normal equations: A^T (A x - b) = 0 up to rounding
    g = a.T @ (a @ x - b)
    assert np.linalg.norm(g) / (np.linalg.norm(a) * np.linalg.norm(a @ x - b)) < 1e-12


@pytest.mark.gpu
def test_gpu_least_squares_consistent_system_has_zero_residual():
    rows, cols, nb = 1024, 512, 128
    a = O.gen_uniform(5, rows, cols)
    xt = O.gen_uniform(6, cols, 3)
    x, r, _ = _gpu_solve(a, nb, a @ xt)
    assert np.linalg.norm(x - xt) / np.linalg.norm(xt) < 1e-11
    assert np.all(r < 1e-11 * np.linalg.norm(a @ xt, axis=0))


@pytest.mark.gpu
def test_gpu_qr_solve_host_and_large_backward_error():
    import torch
    n, nb, nrhs = 8192, 512, 16
    da = torch.empty(n * n, dtype=torch.float64, device="cuda")
    P.gen_uniform(da.data_ptr(), n, nb, 1)
    b = torch.rand(n, nrhs, dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(2))
    db = b.t().contiguous()  # column-major n x nrhs
    dx = torch.zeros(nrhs * n, dtype=torch.float64, device="cuda")
    st = P.qr_solve(da.data_ptr(), n, n, nb, db.data_ptr(), dx.data_ptr(), nrhs)
    assert st.code == 0 and st.tflops > 0
    # A in dense form from the tile layout (tile (m, k) column-major)
    mt = n // nb
    A = da.view(mt, mt, nb, nb).permute(1, 3, 0, 2).reshape(n, n)
    X = dx.view(nrhs, n).t()
    res = torch.linalg.norm(A @ X - b) / (torch.linalg.norm(A) * torch.linalg.norm(X) + torch.linalg.norm(b))
    assert float(res) < 1e-13
    # host-buffer entry point gives the same X bit for bit (same DAG, same kernels)
    xh, _, _ = P.qr_solve_host(da.cpu().numpy(), n, n, nb, b.cpu().numpy())
    assert np.array_equal(xh, X.cpu().numpy())
