"""Batched mixed-precision solves: the FP32 factorizations of one persistent launch against
numpy, per-matrix breakdown flags that leave the other matrices intact, FP64-level solutions
from FP32 and FP64 factors, the FP64 fallback of matrices that FP32 cannot handle, and the
synthetic batch's solve driver and autotuner."""
import numpy as np
import pytest

from oracle import oracle as O
from palial_gb300 import batched as B

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _spd(n, rng):
    b = rng.uniform(-1, 1, (n, n))
    return b @ b.T + n * np.eye(n)


def _dominant(n, rng):
    return rng.uniform(-1, 1, (n, n)) + n * np.eye(n)


def _kappa(n, kappa, rng, symmetric):
    q1 = np.linalg.qr(rng.standard_normal((n, n)))[0]
    q2 = q1 if symmetric else np.linalg.qr(rng.standard_normal((n, n)))[0]
    s = kappa ** (-np.arange(n) / (n - 1))
    a = (q1 * s) @ q2.T
    return (a + a.T) / 2 if symmetric else a


class Dev:
    """Matrices in the tile layout (one device buffer), right-hand sides and solutions."""

    def __init__(self, mats, nbs, dtype=torch.float64, rhs_seed=11):
        self.mats, self.nbs = mats, list(nbs)
        self.ns = [a.shape[0] for a in mats]
        offs = np.concatenate([[0], np.cumsum([n * n for n in self.ns])])
        self.offs = offs
        host = np.concatenate([O.to_tiles(a, nb) for a, nb in zip(mats, self.nbs)])
        self.buf = torch.from_numpy(host).to(dtype).cuda()
        es = self.buf.element_size()
        self.ptrs = [self.buf.data_ptr() + es * int(o) for o in offs[:-1]]
        rng = np.random.default_rng(rhs_seed)
        self.b = [rng.uniform(-1, 1, n) for n in self.ns]
        voffs = np.concatenate([[0], np.cumsum(self.ns)])
        self.bdev = torch.from_numpy(np.concatenate(self.b)).cuda()
        self.xdev = torch.full((int(voffs[-1]),), float("nan"), dtype=torch.float64, device="cuda")
        self.bptrs = [self.bdev.data_ptr() + 8 * int(o) for o in voffs[:-1]]
        self.xptrs = [self.xdev.data_ptr() + 8 * int(o) for o in voffs[:-1]]
        self.voffs = voffs

    def factor(self, i):
        t = self.buf[int(self.offs[i]):int(self.offs[i + 1])].double().cpu().numpy()
        return O.from_tiles(t, self.ns[i], self.nbs[i])

    def x(self, i):
        return self.xdev[int(self.voffs[i]):int(self.voffs[i + 1])].cpu().numpy()


def _berr(a, x, b):
    r = b - a @ x
    return np.abs(r).max() / (np.abs(a).sum(axis=1).max() * np.abs(x).max() + np.abs(b).max())


def test_fp32_batched_factors_match_numpy():
    rng = np.random.default_rng(1)
    spec = [(0, 64, 64), (0, 320, 64), (0, 512, 128), (1, 192, 64), (1, 256, 256), (0, 1024, 256), (1, 640, 128)]
    mats = [(_spd if a == 0 else _dominant)(n, rng) for a, n, _ in spec]
    d = Dev(mats, [nb for _, _, nb in spec], dtype=torch.float32)
    st, flags = B.factor_f32([a for a, _, _ in spec], d.ns, d.nbs, d.ptrs)
    assert st.code == 0 and not flags.any()
    for i, (alg, n, _) in enumerate(spec):
        a = mats[i].astype(np.float32).astype(np.float64)
        f = d.factor(i)
        if alg == 0:
            u = np.triu(f)
            assert np.linalg.norm(a - u.T @ u) <= 3e-5 * np.linalg.norm(a), i
            assert np.linalg.norm(u - np.linalg.cholesky(a).T) <= 1e-4 * np.linalg.norm(u), i
        else:
            l = np.tril(f, -1) + np.eye(n)
            assert np.linalg.norm(a - l @ np.triu(f)) <= 3e-5 * np.linalg.norm(a), i


def test_fp32_breakdown_is_flagged_per_matrix():
    """A Cholesky with a negative pivot and an LU with an exact zero pivot are flagged; the
    other matrices of the same launch are factored as if alone."""
    rng = np.random.default_rng(2)
    indef = _spd(128, rng)
    indef[0, 0] = -1.0
    zero = _dominant(128, rng)
    zero[0, 0] = 0.0
    mats = [_spd(128, rng), indef, zero, _spd(256, rng)]
    algs = [0, 0, 1, 0]
    d = Dev(mats, [64, 64, 64, 128], dtype=torch.float32)
    st, flags = B.factor_f32(algs, d.ns, d.nbs, d.ptrs)
    assert st.code == 0
    assert flags[0] == 0 and flags[1] == 1 and flags[2] != 0 and flags[3] == 0
    for i in (0, 3):
        a = mats[i].astype(np.float32).astype(np.float64)
        u = np.triu(d.factor(i))
        assert np.linalg.norm(a - u.T @ u) <= 3e-5 * np.linalg.norm(a), i


def test_batched_solve_reaches_fp64_backward_error():
    rng = np.random.default_rng(3)
    spec = [(0, 64, 64, "fp32"), (0, 384, 128, "fp32"), (0, 1024, 256, "fp32"), (1, 128, 64, "fp32"),
            (1, 512, 128, "fp32"), (0, 256, 64, "fp64"), (1, 320, 64, "fp64"), (1, 2048, 256, "fp32")]
    mats = [(_spd if a == 0 else _dominant)(n, rng) for a, n, _, _ in spec]
    d = Dev(mats, [nb for _, _, nb, _ in spec])
    st, iters, berr = B.solve([a for a, *_ in spec], d.ns, d.nbs, d.ptrs, d.bptrs, d.xptrs,
                              precs=[p for *_, p in spec])
    assert st.code == 0 and st.fallbacks == 0
    assert (iters >= 1).all() and st.ir_iters == iters.max()
    for i, (alg, n, _, prec) in enumerate(spec):
        x = d.x(i)
        tol = 1e-14 * n
        assert berr[i] <= tol, (i, berr[i])
        assert _berr(mats[i], x, d.b[i]) <= tol, i
        xr = np.linalg.solve(mats[i], d.b[i])
        assert np.linalg.norm(x - xr) <= 1e-11 * np.linalg.norm(xr), i
        if prec == "fp64":
            assert iters[i] <= 2, (i, iters[i])
    assert st.backward_error == berr.max()


def test_batched_solve_falls_back_to_fp64():
    """kappa = 1e10 is beyond FP32 (kappa * u_fp32 > 1): those matrices are refactored in FP64
    (iters < 0) and still reach the tolerance; the well-conditioned one stays on FP32."""
    rng = np.random.default_rng(4)
    mats = [_kappa(256, 1e10, rng, True), _kappa(192, 1e10, rng, False), _spd(256, rng)]
    algs = [0, 1, 0]
    d = Dev(mats, [64, 64, 128])
    st, iters, berr = B.solve(algs, d.ns, d.nbs, d.ptrs, d.bptrs, d.xptrs)
    assert st.code == 0
    assert iters[0] < 0 and iters[1] < 0 and iters[2] > 0
    assert st.fallbacks == 2
    for i in range(3):
        tol = 1e-14 * d.ns[i]
        assert berr[i] <= tol, (i, berr[i])
        assert _berr(mats[i], d.x(i), d.b[i]) <= tol, i


def test_batched_solve_rejects_bad_arguments():
    rng = np.random.default_rng(5)
    d = Dev([_spd(128, rng)], [64])
    with pytest.raises(B.PalialError):
        B.solve([0], [128], [48], d.ptrs, d.bptrs, d.xptrs)
    with pytest.raises(B.PalialError):
        B.solve([0], [128], [64], d.ptrs, d.bptrs, d.xptrs, precs=["bf16"])


def test_synthetic_batched_solve_split_over_two_ranks():
    reps = [B.solve_synthetic(48, seed=3, rank=r, world=2, autotune=False, reps=1) for r in range(2)]
    assert sum(r["count"] for r in reps) == 48
    for r in reps:
        assert r["rc"] == 0 and r["not_converged"] == 0
        assert r["seconds"] > 0 and r["matrices_per_s"] > 0 and r["tflops"] > 0
        assert 0 <= r["max_backward_error"] <= 1e-14 * 2048
        assert r["max_iters"] >= 1 and all(p == 1 for p in r["prec_of_class"])


def test_bf16x3_update_form_reaches_fp64_target():
    """The batched "BF16-update" form: FP32 storage, the SYRK / GEMM update tasks' products on the
    warp tensor cores as BF16x3, FP64 refinement (FP64 fallback kept).  Every matrix reaches the
    FP64-level target, and matches the FP32 form's solution within the refinement's reach."""
    rng = np.random.default_rng(11)
    sizes, nbs, algs = [512, 384, 256, 192], [128, 128, 64, 64], [0, 1, 0, 1]
    mats = []
    for a, m in zip(algs, sizes):
        q = rng.uniform(-1, 1, (m, m))
        mats.append(q @ q.T + m * np.eye(m) if a == 0 else q + m * np.eye(m))
    d = Dev(mats, nbs)
    st, iters, berr = B.solve(algs, sizes, nbs, d.ptrs, d.bptrs, d.xptrs, precs=["bf16x3"] * 4)
    assert st.code == 0, st.message
    for i, m in enumerate(mats):
        ref = np.linalg.solve(m, d.b[i])
        assert berr[i] <= 1e-14 * sizes[i], (i, berr[i])
        assert np.linalg.norm(d.x(i) - ref) <= 1e-10 * np.linalg.norm(ref), i
    print("bf16x3 update form: refinement steps", iters.tolist(), "backward errors", berr.tolist())


def test_solve_autotune_keeps_the_fastest_converging_choice():
    r = B.solve_synthetic(24, seed=4, autotune=True, reps=1)
    assert r["rc"] == 0 and r["not_converged"] == 0
    ns, algs = B.batch_sizes(24, 4)
    present = {(int(a), B.size_class(int(n))) for n, a in zip(ns, algs)}
    for a, c in present:
        k = a * 6 + c
        times = r["autotune_s"][k * 9:(k + 1) * 9]  # [precision 0, 1, 2][block 64, 128, 256]
        ok = [t for t in times if t >= 0]
        assert ok, (a, c)
        chosen = r["prec_of_class"][k] * 3 + B.CANDIDATE_BS.index(r["bs_of_class"][k])
        assert times[chosen] == min(ok), (a, c, times)


def test_batched_lu_failing_in_fp32_is_solved_on_its_butterfly_transform():
    """A no-pivot LU matrix whose FP32 factorization meets a tiny pivot (pivot growth beyond
    FP32) gets a second FP32 attempt on U^T A V (random butterflies): it reaches the FP64-level
    tolerance without the FP64 fallback, and the solution matches numpy's."""
    rng = np.random.default_rng(11)
    n = 256
    a = rng.uniform(-1, 1, (n, n))
    a[0, 0] = 1e-9  # a leading pivot FP32 cannot factor without growth
    mats = [a, _spd(128, rng)]
    d = Dev(mats, [64, 64])
    st, iters, berr = B.solve([1, 0], d.ns, d.nbs, d.ptrs, d.bptrs, d.xptrs)
    assert st.code == 0, st.message
    assert st.butterflies == 1 and st.fallbacks == 0, (st.butterflies, st.fallbacks)
    assert iters[0] > 0
    for i in range(2):
        assert berr[i] <= 1e-14 * d.ns[i], (i, berr[i])
        xr = np.linalg.solve(mats[i], d.b[i])
        assert np.linalg.norm(d.x(i) - xr) <= 1e-9 * np.linalg.norm(xr), i
