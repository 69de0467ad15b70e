"""Mixed precision: the tcgen05 trailing update against a torch FP32 reference computed from
the same quantized operands, and mixed-precision factorization + iterative refinement
against numpy's FP64 solution (backward error gate 1e-14 * N, the target of the path)."""
import ctypes

import numpy as np
import pytest

import palial_gb300 as P
from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

PREC = {1: "bf16", 2: "fp8", 3: "bf16x3", 6: "tf32x3"}


def tf32(x):
    """The kernel's TF32 rounding: half away from zero to 10 explicit mantissa bits."""
    return ((x.view(torch.int32) + 0x1000) & ~0x1FFF).view(torch.float32)


def quant(x, prec, nb):
    """Operand quantization of the kernel: x is (rows, nb*t) float32 panel, tiles along dim 1."""
    if prec == 1:
        return x.bfloat16().float()
    if prec == 3:
        hi = x.bfloat16().float()
        return hi, (x - hi).bfloat16().float()
    out = torch.empty_like(x)
    for t in range(x.shape[1] // nb):
        blk = x[:, t * nb:(t + 1) * nb]
        s = blk.abs().max() / torch.tensor(448.0, dtype=torch.float32, device=x.device)
        inv = torch.tensor(1.0, dtype=torch.float32, device=x.device) / s
        out[:, t * nb:(t + 1) * nb] = (blk * inv).to(torch.float8_e4m3fn).float() * s
    return out


def prod(a, b, prec, nb):
    """a: (nb x r1) operand whose columns are output rows, b: (nb x r2): returns a^T b."""
    if prec == 6:
        ah, bh = tf32(a), tf32(b)
        al, bl = tf32(a - ah), tf32(b - bh)
        return ah.T @ bh + ah.T @ bl + al.T @ bh
    if prec == 3:
        ah, al = quant(a, 3, nb)
        bh, bl = quant(b, 3, nb)
        return ah.T @ bh + ah.T @ bl + al.T @ bh
    return quant(a, prec, nb).T @ quant(b, prec, nb)


@pytest.mark.parametrize("prec", [1, 2, 3, 6])
@pytest.mark.parametrize("alg", [0, 1])
def test_tcgen05_trailing_update(alg, prec):
    """BF16 / FP8 / BF16x3: against torch's FP32 products of the same quantized operands
    (relative 1e-4).  TF32x3 (kind::tf32, hi + lo split): against the FP64 product of the FP32
    operands themselves, relative 4e-6 (FP32-level), and the split is checked exact up to the
    two lowest bits."""
    n, nb, k = 1536, 512, 0
    a = torch.from_numpy(O.gen_uniform(21 + alg, n).astype(np.float32)).cuda()
    w = torch.from_numpy(O.to_tiles(a.cpu().numpy().astype(np.float64), nb).astype(np.float32)).cuda()
    rc = P.lib().palial_gpu_mp_update_step(alg, prec, w.data_ptr(), n, nb, k)
    torch.cuda.synchronize()
    assert rc == 0
    got = torch.from_numpy(O.from_tiles(w.cpu().numpy().astype(np.float64), n, nb)).cuda().float()
    r0 = (k + 1) * nb
    kk = slice(k * nb, (k + 1) * nb)
    if alg == 0:
        upd = prod(a[kk, r0:], a[kk, r0:], prec, nb)          # U(k,n)^T U(k,m)
    else:
        # L(m,k) U(k,n): the L panel enters as its transpose (columns = output rows)
        upd = prod(a[r0:, kk].T.contiguous(), a[kk, r0:], prec, nb)
    ref = a.clone()
    ref[r0:, r0:] -= upd
    if alg == 0:  # only tile pairs (n <= m) are updated
        mt = n // nb
        for ti in range(k + 1, mt):
            for tj in range(k + 1, ti):
                ref[ti * nb:(ti + 1) * nb, tj * nb:(tj + 1) * nb] = a[ti * nb:(ti + 1) * nb, tj * nb:(tj + 1) * nb]
    if prec == 6:
        ad = a.double()
        if alg == 0:
            upd64 = ad[kk, r0:].T @ ad[kk, r0:]
        else:
            upd64 = ad[r0:, kk] @ ad[kk, r0:]
        ref64 = ad.clone()
        ref64[r0:, r0:] -= upd64
        if alg == 0:
            for ti in range(k + 1, n // nb):
                for tj in range(k + 1, ti):
                    ref64[ti * nb:(ti + 1) * nb, tj * nb:(tj + 1) * nb] = ad[ti * nb:(ti + 1) * nb, tj * nb:(tj + 1) * nb]
        err = float(torch.linalg.norm(got.double() - ref64) / torch.linalg.norm(upd64))
        hi = tf32(a)
        lo = tf32(a - hi)
        split = float(((a.double() - hi.double() - lo.double()).abs() / a.double().abs().clamp_min(1e-30)).max())
        print(f"tf32x3 update: relative error {err:.3e} against FP64, split error {split:.3e}")
        assert split <= 2.0 ** -21
        assert err <= 4e-6, err
    else:
        err = float(torch.linalg.norm(got - ref) / torch.linalg.norm(upd))
        assert err <= 1e-4, err
    # the panel itself and the leading tiles are untouched
    assert torch.equal(got[kk, :], a[kk, :]) and torch.equal(got[:, kk], a[:, kk])


@pytest.mark.parametrize("prec", [1, 2, 3, 6])
@pytest.mark.parametrize("alg", [0, 1])
def test_update_kernels_bitwise_equal(alg, prec):
    """The tile-run update kernel (double-buffered TMEM, one CTA per SM) issues the same MMAs
    and epilogue arithmetic per output block as the one-block-per-CTA kernel: equal bits, at a
    size where runs of 2 (n = 4096) and 8 (n = 16384) blocks per CTA occur."""
    lib = P.lib()
    for n in (4096, 16384):
        nb = 512
        g = torch.Generator("cuda").manual_seed(31 + alg)
        a = torch.rand(n * n, dtype=torch.float32, device="cuda", generator=g) * 2 - 1
        w0 = a.clone()
        w1 = a.clone()
        w2 = a.clone()
        old = lib.palial_gpu_set_update_kernel(0)
        try:
            assert lib.palial_gpu_mp_update_step(alg, prec, w0.data_ptr(), n, nb, 0) == 0
            lib.palial_gpu_set_update_kernel(2)
            assert lib.palial_gpu_mp_update_step(alg, prec, w2.data_ptr(), n, nb, 0) == 0
            lib.palial_gpu_set_update_kernel(1)
            assert lib.palial_gpu_mp_update_step(alg, prec, w1.data_ptr(), n, nb, 0) == 0
        finally:
            lib.palial_gpu_set_update_kernel(old)
        torch.cuda.synchronize()
        assert not torch.equal(w0, a)
        assert torch.equal(w0, w2), (n, alg, prec)
        assert torch.equal(w0, w1), (n, alg, prec)


def dominant(seed, n):
    a = np.full((n, n), 0.5)
    u = (O.gen_uniform(seed, n, 1)[:, 0] + 1.0) * 0.5
    a[np.diag_indices(n)] = 173.0 * u + 173.0
    return a


@pytest.mark.parametrize("prec", ["bf16", "bf16x3", "tf32x3", "fp8", "fp64"])
@pytest.mark.parametrize("alg", ["cholesky", "lu"])
def test_solve_ir_reaches_fp64_backward_error(alg, prec):
    n, nb, nrhs = 2048, 512, 16
    a = O.gen_spd(0, n) if alg == "cholesky" else dominant(3, n)
    b = O.gen_uniform(5, n, nrhs, stream=O.STREAM_RHS)
    da = torch.from_numpy(O.to_tiles(a, nb)).cuda()
    db = torch.from_numpy(np.asfortranarray(b).ravel(order="F")).cuda()
    dx = torch.zeros_like(db)
    st = P.solve_ir(alg, da.data_ptr(), n, nb, db.data_ptr(), dx.data_ptr(), nrhs, precision=prec,
                    ir_max_iter=100, raise_on_error=False)
    x = dx.cpu().numpy().reshape(nrhs, n).T
    r = b - a @ x
    eta = np.max(np.abs(r).max(0) / (np.abs(a).sum(1).max() * np.abs(x).max(0) + np.abs(b).max(0)))
    xref = np.linalg.solve(a, b)
    fwd = np.max(np.abs(x - xref).max(0) / np.abs(xref).max(0))
    print(alg, prec, "iters", st.ir_iters, "eta(dev)", st.backward_error, "eta(host)", eta, "fwd", fwd,
          "factor s", st.factor_seconds, "total s", st.seconds)
    assert st.code in (0, 1), st.message
    assert eta <= 1e-14 * n and st.backward_error <= 1e-14 * n
    assert fwd <= 1e-10


@pytest.mark.parametrize("kappa", [1e2, 1e6, 1e10])
@pytest.mark.parametrize("alg", ["cholesky", "lu"])
def test_kappa_sweep_small(alg, kappa):
    """A = U diag(s) V^T with kappa(A) = kappa (64 Householder reflectors each side), the AUTO
    precision ladder: every kappa must reach the FP64-level target (at kappa = 1e10 through the
    FP64 rung, whose refinement solves with the FP64 factors)."""
    n, nb, nrhs = 2048, 512, 16
    da = torch.empty(n * n, dtype=torch.float64, device="cuda")
    P.gen_kappa(da.data_ptr(), n, nb, kappa, alg == "cholesky", seed=7)
    torch.cuda.synchronize()
    a = O.from_tiles(da.cpu().numpy(), n, nb)
    s = np.linalg.svd(a, compute_uv=False)
    assert abs(s[0] / s[-1] / kappa - 1) < 1e-3 * max(1.0, kappa / 1e6)
    if alg == "cholesky":
        assert np.array_equal(a, a.T)
    b = O.gen_uniform(5, n, nrhs, stream=O.STREAM_RHS)
    db = torch.from_numpy(np.asfortranarray(b).ravel(order="F")).cuda()
    dx = torch.zeros_like(db)
    st = P.solve_ir(alg, da.data_ptr(), n, nb, db.data_ptr(), dx.data_ptr(), nrhs, precision="auto",
                    ir_max_iter=30, raise_on_error=False)
    x = dx.cpu().numpy().reshape(nrhs, n).T
    xref = np.linalg.solve(a, b)
    fwd = np.max(np.abs(x - xref).max(0) / np.abs(xref).max(0))
    print(f"{alg} kappa={kappa:.0e} code={st.code} prec={P.PREC_NAME.get(st.precision_used)} iters={st.ir_iters} "
          f"gmres={st.gmres_iters} eta={st.backward_error:.3e} fwd={fwd:.3e} shift={st.shift:.2e} t={st.seconds:.3f}s")
    assert st.code in (0, 1), st.message
    assert st.backward_error <= 1e-14 * n


@pytest.mark.parametrize("alg", ["cholesky", "lu"])
def test_tf32x3_rung_reaches_target_at_kappa_1e6(alg):
    """kappa = 1e6 at N = 8192: the FP32-level TF32x3 factors reach the FP64-level target
    (GMRES-IR where plain refinement stalls; no-pivot LU there is beyond BF16x3 within the
    ladder's budget, printed for reference).  The forward error against numpy's FP64 solution
    is what the reached backward error allows: <= 10 * kappa * 1e-14 * N."""
    n, nb, nrhs = 8192, 512, 16
    kappa = 1e6
    da = torch.empty(n * n, dtype=torch.float64, device="cuda")
    P.gen_kappa(da.data_ptr(), n, nb, kappa, alg == "cholesky", seed=7)
    torch.cuda.synchronize()
    b = O.gen_uniform(5, n, nrhs, stream=O.STREAM_RHS)
    db = torch.from_numpy(np.asfortranarray(b).ravel(order="F")).cuda()
    a = O.from_tiles(da.cpu().numpy(), n, nb)
    xref = np.linalg.solve(a, b)
    for prec in ("bf16x3", "tf32x3"):
        dx = torch.zeros_like(db)
        o = P.make_opts(precision=prec, ir_max_iter=10)
        o.reserved[1] = 100  # GMRES iterations per call, as the ladder's TF32x3 rung
        o.reserved[3] = 400  # GMRES iterations in all
        st = P.Status()
        st.code = P.lib().palial_gpu_solve_ir(P.ALG[alg], da.data_ptr(), n, nb, db.data_ptr(), dx.data_ptr(), nrhs,
                                              P.ctypes.byref(o), P.ctypes.byref(st), None)
        x = dx.cpu().numpy().reshape(nrhs, n).T
        fwd = float(np.max(np.abs(x - xref).max(0) / np.abs(xref).max(0)))
        print(f"{alg} kappa={kappa:.0e} {prec}: code={st.code} iters={st.ir_iters} gmres={st.gmres_iters} "
              f"eta={st.backward_error:.3e} fwd={fwd:.3e} shift={st.shift:.2e} t={st.seconds:.3f}s")
    assert st.code in (0, 1), st.message
    assert st.backward_error <= 1e-14 * n
    assert fwd <= 10 * kappa * 1e-14 * n


def test_non_finite_factor_is_not_reported_as_converged():
    """An exact zero leading pivot: the no-pivot LU skips it (as the reference does) and the
    factor is singular; refinement must end with an error, never with a false success."""
    n, nb, nrhs = 1024, 256, 4
    a = dominant(3, n)
    a[0, :] = 0.0
    a[:, 0] = 0.0
    b = O.gen_uniform(5, n, nrhs, stream=O.STREAM_RHS)
    da = torch.from_numpy(O.to_tiles(a, nb)).cuda()
    db = torch.from_numpy(np.asfortranarray(b).ravel(order="F")).cuda()
    dx = torch.zeros_like(db)
    for prec in ("bf16", "fp8", "fp64"):
        st = P.solve_ir("lu", da.data_ptr(), n, nb, db.data_ptr(), dx.data_ptr(), nrhs, precision=prec,
                        ir_max_iter=5, raise_on_error=False)
        assert st.code < 0, (prec, st.code, st.backward_error)


@pytest.mark.parametrize("nb", [256, 512, 768, 1024])
@pytest.mark.parametrize("alg", ["cholesky", "lu"])
def test_fp32_diagonal_tile_factor(alg, nb):
    """A one-tile matrix: the mixed factorization is exactly the FP32 diagonal-tile kernel.
    Factors against numpy's FP64 ones (FP32 accuracy: normwise 2e-6 on these well-conditioned
    inputs); for Cholesky the strictly lower triangle must stay untouched."""
    n = nb
    a = O.gen_spd(0, n) if alg == "cholesky" else dominant(3, n)
    da = torch.from_numpy(O.to_tiles(a, nb)).cuda()
    dw = torch.zeros(n * n, dtype=torch.float32, device="cuda")
    st = P.mp_factor(alg, da.data_ptr(), dw.data_ptr(), n, nb, precision="bf16")
    assert st.code == 0
    w = O.from_tiles(dw.double().cpu().numpy(), n, nb)
    if alg == "cholesky":
        u = np.linalg.cholesky(a).T
        assert np.linalg.norm(np.triu(w) - u) / np.linalg.norm(u) < 2e-6
        assert np.array_equal(np.tril(w, -1), np.tril(a.astype(np.float32).astype(np.float64), -1))
    else:
        import scipy.linalg as sl
        p, l, u = sl.lu(a)
        assert np.array_equal(p, np.eye(n))  # diagonally dominant: partial pivoting keeps the order
        assert np.linalg.norm(np.triu(w) - u) / np.linalg.norm(u) < 2e-6
        assert np.linalg.norm(np.tril(w, -1) - np.tril(l, -1)) / np.linalg.norm(np.tril(l, -1)) < 2e-6


def test_fp32_diagonal_tile_reports_breakdown():
    """An indefinite diagonal tile: the kernel reports the failing column, not NaN factors."""
    n, nb = 512, 512
    a = O.gen_spd(0, n)
    a[300, 300] = -1.0
    da = torch.from_numpy(O.to_tiles(a, nb)).cuda()
    dw = torch.zeros(n * n, dtype=torch.float32, device="cuda")
    with pytest.raises(P.PalialError):
        P.mp_factor("cholesky", da.data_ptr(), dw.data_ptr(), n, nb, precision="bf16")


@pytest.mark.parametrize("kind", ["spd", "kappa"])
def test_compensated_residual_matches_fp64(kind):
    """The refinement's steering residual (compensated FP32, 48-bit operands) against a torch
    FP64 product: normwise error <= 1e-12 of |A||x| scale; the FP64 mode against torch <= 1e-14."""
    import ctypes
    n, nb, nrhs = 4096, 512, 16
    da = torch.empty(n * n, dtype=torch.float64, device="cuda")
    if kind == "spd":
        P.gen_spd(da.data_ptr(), n, nb, 0)
    else:
        P.gen_kappa(da.data_ptr(), n, nb, 1e8, False, seed=3)
    x = torch.rand(nrhs, n, dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(1)) - 0.5
    x[3] *= 1e-9  # a column of very different scale
    b = torch.rand(nrhs, n, dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(2))
    mt = n // nb
    A = da.view(mt, mt, nb, nb).permute(1, 3, 0, 2).reshape(n, n)
    ref = b.t() - A @ x.t()
    scale = (A.abs() @ x.t().abs()).max(dim=0).values + b.t().abs().max(dim=0).values
    lib = P.lib()
    lib.palial_gpu_residual.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    for mode, bound in ((0, 1e-14), (1, 1e-12), (3, 1e-13)):
        r = torch.zeros(nrhs, n, dtype=torch.float64, device="cuda")
        assert lib.palial_gpu_residual(da.data_ptr(), n, nb, x.data_ptr(), b.data_ptr(), r.data_ptr(), nrhs, mode,
                                       None) == 0
        torch.cuda.synchronize()
        err = ((r.t() - ref).abs().max(dim=0).values / scale).max().item()
        assert err <= bound, (mode, err)


@pytest.mark.parametrize("nrhs", [16, 5, 1])
def test_digit_residual_against_exact_products(nrhs):
    """The digit residual (mode 3: A and X as 48-bit integers in BF16 digits on the tensor cores),
    R = A X with B = NULL, against torch's FP64 product: entrywise |error| <= 2^-40 (|A| |X|)_i
    (its own rounding) + 4 n 2^-53 (|A| |X|)_i (the FP64 reference's); a zero column stays
    exactly zero and a column of scale 1e-30 is handled by its own exponent."""
    import ctypes
    n, nb = 2048, 512
    da = torch.empty(n * n, dtype=torch.float64, device="cuda")
    P.gen_kappa(da.data_ptr(), n, nb, 1e6, False, seed=5)
    g = torch.Generator("cuda").manual_seed(9)
    x = torch.rand(nrhs, n, dtype=torch.float64, device="cuda", generator=g) - 0.5
    if nrhs > 3:
        x[1] = 0.0
        x[2] *= 1e-30
    mt = n // nb
    A = da.view(mt, mt, nb, nb).permute(1, 3, 0, 2).reshape(n, n)
    lib = P.lib()
    lib.palial_gpu_residual.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    r = torch.zeros(nrhs, n, dtype=torch.float64, device="cuda")
    assert lib.palial_gpu_residual(da.data_ptr(), n, nb, x.data_ptr(), None, r.data_ptr(), nrhs, 3, None) == 0
    torch.cuda.synchronize()
    ref = A @ x.t()
    bound = (2.0 ** -40 + 4 * n * 2.0 ** -53) * (A.abs() @ x.t().abs())
    err = (r.t() - ref).abs()
    assert bool((err <= bound).all()), float((err / bound.clamp_min(1e-300)).max())
    if nrhs > 3:
        assert bool((r[1] == 0).all())


@pytest.mark.parametrize("nrhs", [16, 5])
def test_update_form_residual_error_bound(nrhs):
    """R <- R - A D with FP32 products (the refinement's update form) against torch FP64:
    entrywise |error| <= 2^-17 (|A| |D|)_i, columns of very different scale, a zero column
    leaves R exactly unchanged."""
    import ctypes
    n, nb = 4096, 512
    da = torch.empty(n * n, dtype=torch.float64, device="cuda")
    P.gen_kappa(da.data_ptr(), n, nb, 1e4, False, seed=5)
    g = torch.Generator("cuda").manual_seed(7)
    d = torch.rand(nrhs, n, dtype=torch.float64, device="cuda", generator=g) - 0.5
    d[1] *= 1e-12
    d[2] = 0.0
    r0 = torch.rand(nrhs, n, dtype=torch.float64, device="cuda", generator=g)
    mt = n // nb
    A = da.view(mt, mt, nb, nb).permute(1, 3, 0, 2).reshape(n, n)
    ref = r0.t() - A @ d.t()
    bound = (A.abs() @ d.t().abs()) * 2.0 ** -17 + 1e-15 * ref.abs()
    r = r0.clone()
    lib = P.lib()
    lib.palial_gpu_residual.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    assert lib.palial_gpu_residual(da.data_ptr(), n, nb, d.data_ptr(), None, r.data_ptr(), nrhs, 2, None) == 0
    torch.cuda.synchronize()
    err = (r.t() - ref).abs()
    assert bool((err <= bound).all()), (err / bound.clamp_min(1e-300)).max().item()
    assert torch.equal(r[2], r0[2])
    # the bound is not vacuous: the FP32 products do differ from FP64
    assert err[:, 0].max().item() > 0


def test_refinement_update_form_residual():
    """BF16x3 at N = 8192: the second residual takes the update form (the message counts it),
    and the solution's FP64 backward error meets the target as with full residuals only."""
    n, nb, nrhs = 8192, 512, 16
    a = O.gen_spd(0, n)
    b = O.gen_uniform(5, n, nrhs, stream=O.STREAM_RHS)
    da = torch.from_numpy(O.to_tiles(a, nb)).cuda()
    db = torch.from_numpy(np.asfortranarray(b).ravel(order="F")).cuda()
    at = torch.from_numpy(a).cuda()
    bt = torch.from_numpy(b).cuda()
    res = {}
    for r4 in (0, 3):
        dx = torch.zeros_like(db)
        o = P.make_opts(precision="bf16x3")
        o.reserved[4] = r4
        import ctypes
        st = P.Status()
        rc = P.lib().palial_gpu_solve_ir(0, da.data_ptr(), n, nb, db.data_ptr(), dx.data_ptr(), nrhs, ctypes.byref(o),
                                         ctypes.byref(st), None)
        assert rc == 0, st.message
        x = dx.view(nrhs, n).t()
        r = bt - at @ x
        eta = (r.abs().max(0).values / (at.abs().sum(1).max() * x.abs().max(0).values + bt.abs().max(0).values)).max()
        assert eta.item() <= 1e-14 * n
        msg = st.message.decode(errors="replace")
        res[r4] = (st.ir_iters, msg, x.clone())
    import re
    count = {k: int(re.search(r"(\d+) update-form", v[1]).group(1)) for k, v in res.items()}
    assert count[0] >= 1 and count[3] == 0, res
    assert res[0][0] == res[3][0]


def test_refinement_with_compensated_residual_reports_fp64_error():
    """Steering with the compensated residual and confirming in FP64 gives the same solution
    quality as FP64 residuals throughout (backward errors of both at the FP64 target)."""
    n, nb, nrhs = 4096, 512, 8
    a = O.gen_spd(0, n)
    b = O.gen_uniform(5, n, nrhs, stream=O.STREAM_RHS)
    da = torch.from_numpy(O.to_tiles(a, nb)).cuda()
    db = torch.from_numpy(np.asfortranarray(b).ravel(order="F")).cuda()
    xs = []
    for r4 in (0, 1):
        dx = torch.zeros_like(db)
        o = P.make_opts(precision="bf16")
        o.reserved[4] = r4
        import ctypes
        st = P.Status()
        rc = P.lib().palial_gpu_solve_ir(0, da.data_ptr(), n, nb, db.data_ptr(), dx.data_ptr(), nrhs, ctypes.byref(o),
                                         ctypes.byref(st), None)
        assert rc == 0 and st.backward_error <= 1e-14 * n, (r4, rc, st.backward_error)
        xs.append(dx.cpu().numpy())
    assert np.linalg.norm(xs[0] - xs[1]) / np.linalg.norm(xs[1]) < 1e-11


def _solve_lu(da, n, nb, db, nrhs, precision, rbt, maxit=30):
    import ctypes
    dx = torch.zeros_like(db)
    o = P.make_opts(precision=precision, ir_max_iter=maxit)
    o.reserved[6] = 1 if rbt else 0
    st = P.Status()
    rc = P.lib().palial_gpu_solve_ir(1, da.data_ptr(), n, nb, db.data_ptr(), dx.data_ptr(), nrhs, ctypes.byref(o),
                                     ctypes.byref(st), None)
    return rc, st, dx


def _block_antidiagonal(n):
    """[[0, B], [C, 0]] with B, C = I + 0.5 G / sqrt(n/2) (G uniform in [-1, 1)): well
    conditioned, but its leading entry is zero, so LU without pivoting breaks down at its
    first pivot."""
    h = n // 2
    g = O.gen_uniform(21, n)
    a = np.zeros((n, n))
    a[:h, h:] = np.eye(h) + 0.5 * g[:h, :h] / np.sqrt(h)
    a[h:, :h] = np.eye(h) + 0.5 * g[h:, h:] / np.sqrt(h)
    return a


@pytest.mark.parametrize("precision", ["bf16", "bf16x3"])
def test_random_butterfly_lu_matches_numpy(precision):
    """LU of U^T A V (depth-2 random butterflies) as the preconditioner, refinement against A.
    On a block anti-diagonal matrix the no-pivot LU of A itself breaks down (zero pivot); the
    butterflies mix row i with rows i + n/4, i + n/2, i + 3n/4, and the transformed matrix
    factors with growth near 1, so refinement reaches the FP64 target."""
    n, nb, nrhs = 2048, 256, 4
    a = _block_antidiagonal(n)
    b = O.gen_uniform(12, n, nrhs)
    da = torch.from_numpy(O.to_tiles(a, nb)).cuda()
    db = torch.from_numpy(np.asfortranarray(b).ravel(order="F")).cuda()
    rc_plain, _, _ = _solve_lu(da, n, nb, db, nrhs, precision, False)
    assert rc_plain != 0
    rc, st, dx = _solve_lu(da, n, nb, db, nrhs, precision, True)
    assert rc == 0, (rc, st.backward_error, st.ir_iters)
    x = dx.cpu().numpy().reshape(nrhs, n).T
    # forward error within kappa (2.3) times the backward-error target 1e-14 n
    assert np.linalg.norm(x - np.linalg.solve(a, b)) / np.linalg.norm(x) < 1e-10
    assert st.backward_error <= 1e-14 * n


def test_random_butterfly_on_dense_matrix_agrees():
    """On a dense A = U diag(s) V^T (orthogonal factors, kappa 1e2) both the plain no-pivot LU
    and the butterfly transform's LU precondition refinement to the FP64 target, and the two
    solutions agree: the transform changes the preconditioner, not the answer."""
    n, nb, nrhs = 4096, 512, 4
    da = torch.empty(n * n, dtype=torch.float64, device="cuda")
    P.gen_kappa(da.data_ptr(), n, nb, 1e2, False, seed=7)
    b = O.gen_uniform(5, n, nrhs, stream=O.STREAM_RHS)
    db = torch.from_numpy(np.asfortranarray(b).ravel(order="F")).cuda()
    rc_plain, st_plain, x_plain = _solve_lu(da, n, nb, db, nrhs, "bf16x3", False)
    rc, st, x_rbt = _solve_lu(da, n, nb, db, nrhs, "bf16x3", True)
    assert rc_plain == 0 and rc == 0, (rc_plain, rc)
    assert st.backward_error <= 1e-14 * n
    # both within kappa * (backward-error target 1e-14 n) of the exact solution
    assert (torch.linalg.vector_norm(x_rbt - x_plain) / torch.linalg.vector_norm(x_plain)).item() < 2 * 1e2 * 1e-14 * n


@pytest.mark.parametrize("alg,prec", [("cholesky", "bf16x3"), ("cholesky", "bf16"), ("cholesky", "fp8"),
                                      ("cholesky", "fp64"), ("lu", "bf16x3")])
def test_host_solve_matches_device_solve(alg, prec):
    """The host-buffer entry point (mixed Cholesky: the upper triangle arrives in row groups
    and the factorization starts on the first ones, catching up skipped updates in step order;
    FP64 Cholesky: upper triangle first) returns exactly the device-resident solve's X."""
    n, nb, nrhs = 4096, 512, 8
    a = O.gen_spd(0, n) if alg == "cholesky" else dominant(3, n)
    b = O.gen_uniform(5, n, nrhs, stream=O.STREAM_RHS)
    at = O.to_tiles(a, nb)
    bf = np.asfortranarray(b)
    da = torch.from_numpy(at).cuda()
    db = torch.from_numpy(bf.ravel(order="F")).cuda()
    dx = torch.zeros_like(db)
    st = P.solve_ir(alg, da.data_ptr(), n, nb, db.data_ptr(), dx.data_ptr(), nrhs, precision=prec)
    assert st.code == 0
    host_a = torch.from_numpy(at).pin_memory()
    xh = np.zeros((nrhs, n))
    sth = P.solve_ir_host(alg, host_a.numpy(), n, nb, np.ascontiguousarray(b.T), xh, nrhs, precision=prec)
    assert sth.code == 0 and sth.ir_iters == st.ir_iters
    assert np.array_equal(xh, dx.cpu().numpy().reshape(nrhs, n))


@pytest.mark.parametrize("prec", ["bf16x3", "fp64"])
def test_host_cholesky_reads_only_the_upper_triangle(prec):
    """Host-buffer Cholesky copies only the upper triangle and writes the lower one on the
    device from it: with NaN everywhere below the diagonal of the caller's buffer, the solve
    returns exactly the device-resident solve's X for the full symmetric matrix."""
    n, nb, nrhs = 4096, 512, 4
    a = O.gen_spd(0, n)
    b = O.gen_uniform(5, n, nrhs, stream=O.STREAM_RHS)
    da = torch.from_numpy(O.to_tiles(a, nb)).cuda()
    db = torch.from_numpy(np.asfortranarray(b).ravel(order="F")).cuda()
    dx = torch.zeros_like(db)
    st = P.solve_ir("cholesky", da.data_ptr(), n, nb, db.data_ptr(), dx.data_ptr(), nrhs, precision=prec)
    assert st.code == 0
    upper = a.copy()
    upper[np.tril_indices(n, -1)] = np.nan
    host_a = torch.from_numpy(O.to_tiles(upper, nb)).pin_memory()
    xh = np.zeros((nrhs, n))
    sth = P.solve_ir_host("cholesky", host_a.numpy(), n, nb, np.ascontiguousarray(b.T), xh, nrhs, precision=prec)
    assert sth.code == 0 and sth.ir_iters == st.ir_iters, sth.message
    assert np.array_equal(xh, dx.cpu().numpy().reshape(nrhs, n))


def test_update_reserve_gives_the_same_bits():
    """The SMs the rest-of-update launches leave to the critical chain change the launch shape
    only: the solution is bit-identical for every setting; bad settings are refused."""
    lib = P.lib()
    err_arg = -1  # PALIAL_ERR_ARG
    assert lib.palial_gpu_set_update_reserve(-1, 0) == err_arg
    assert lib.palial_gpu_set_update_reserve(8, -1) == err_arg
    n, nb, nrhs = 8192, 512, 4
    da = torch.empty(n * n, dtype=torch.float64, device="cuda")
    P.gen_spd(da.data_ptr(), n, nb, seed=3)
    db = torch.empty(n * nrhs, dtype=torch.float64, device="cuda")
    P.gen_dense(db.data_ptr(), n, nrhs, 5, P.STREAM_RHS)
    xs = []
    old = lib.palial_gpu_set_update_reserve(0, 0)
    try:
        for sms, below in ((0, 0), (24, 0), (60, 0), (16, 8)):
            lib.palial_gpu_set_update_reserve(sms, below)
            dx = torch.zeros_like(db)
            st = P.solve_ir("cholesky", da.data_ptr(), n, nb, db.data_ptr(), dx.data_ptr(), nrhs, precision="bf16x3")
            assert st.code == 0
            xs.append(dx)
    finally:
        lib.palial_gpu_set_update_reserve(old, 0)
    assert all(torch.equal(xs[0], x) for x in xs[1:])


@pytest.mark.parametrize("alg", ["cholesky", "lu"])
def test_fp32_and_tensor_core_panels_both_reach_the_target(alg):
    """BF16x3 factorizations solve their panels' block products as BF16x3 on the warp tensor
    cores by default; opts.reserved[5] bit 3 keeps them in FP32.  Both refine to the FP64-level
    backward error in the same small number of steps."""
    import ctypes
    n, nb, nrhs = 4096, 512, 4
    a = O.gen_spd(0, n) if alg == "cholesky" else dominant(3, n)
    b = O.gen_uniform(5, n, nrhs, stream=O.STREAM_RHS)
    da = torch.from_numpy(O.to_tiles(a, nb)).cuda()
    db = torch.from_numpy(np.asfortranarray(b).ravel(order="F")).cuda()
    iters = []
    for bit in (0, 8):
        dx = torch.zeros_like(db)
        o = P.make_opts(precision="bf16x3")
        o.reserved[5] = bit
        st = P.Status()
        rc = P.lib().palial_gpu_solve_ir(P.ALG[alg], da.data_ptr(), n, nb, db.data_ptr(), dx.data_ptr(), nrhs,
                                         ctypes.byref(o), ctypes.byref(st), None)
        assert rc == 0, st.message
        assert st.backward_error <= 1e-14 * n
        x = dx.cpu().numpy().reshape(nrhs, n).T
        assert np.linalg.norm(x - np.linalg.solve(a, b)) <= 1e-9 * np.linalg.norm(x)
        iters.append(st.ir_iters)
    assert max(iters) <= 3, iters


@pytest.mark.parametrize("nb", [256, 512])
def test_shared_memory_diagonal_kernel_gives_the_same_bits(nb):
    """The 256 x 256 Cholesky blocks factored with their upper triangle resident in shared
    memory give the factors of the staged kernel bit for bit (NB = 512: the two halves of each
    diagonal tile; NB = 256: whole tiles)."""
    n = 2048
    a = O.gen_spd(0, n)
    da = torch.from_numpy(O.to_tiles(a, nb)).cuda()
    lib = P.lib()
    outs = []
    old = lib.palial_gpu_set_diag_kernel(0)
    try:
        for kind in (0, 1):
            lib.palial_gpu_set_diag_kernel(kind)
            w = torch.empty(n * n, dtype=torch.float32, device="cuda")
            P.mp_factor("cholesky", da.data_ptr(), w.data_ptr(), n, nb, precision="bf16x3")
            outs.append(w)
    finally:
        lib.palial_gpu_set_diag_kernel(old)
    u = O.from_tiles(outs[0].double().cpu().numpy(), n, nb)
    assert np.array_equal(np.triu(u), np.triu(O.from_tiles(outs[1].double().cpu().numpy(), n, nb)))
    assert np.linalg.norm(np.triu(u).T @ np.triu(u) - a) <= 1e-3 * np.linalg.norm(a)


def test_fp64_to_fp32_conversion_rounds_like_the_hardware():
    """The working-copy conversion rounds by integer operations on the bit pattern: equal bits to
    torch's FP32 cast (round to nearest even) on random values, exact ties in both directions,
    values near the FP32 overflow and underflow limits, zeros and non-finite values."""
    n, nb = 512, 256
    g = torch.Generator().manual_seed(3)
    a = torch.randn(n * n, dtype=torch.float64, generator=g) * torch.exp2(torch.randint(-60, 60, (n * n,),
                                                                                        generator=g).double())
    # exact ties: 24 significant bits + a 1 in the 25th place, odd and even last kept bit
    m = torch.randint(1 << 23, 1 << 24, (4096,), generator=g, dtype=torch.int64)
    ties = (m.double() * 2 + 1) * torch.exp2(torch.randint(-100, 100, (4096,), generator=g).double() - 24)
    a[:4096] = ties
    special = torch.tensor([0.0, -0.0, 3.4e38, -3.4e38, 3.4028235e38, 1e39, -1e39, 1.2e-38, 1e-40, -1e-44, 1e-50,
                            float("inf"), -float("inf"), float("nan")], dtype=torch.float64)
    a[4096:4096 + len(special)] = special
    da = a.cuda()
    w = torch.empty(n * n, dtype=torch.float32, device="cuda")
    assert P.lib().palial_gpu_f64_to_f32(ctypes.c_void_p(da.data_ptr()), ctypes.c_void_p(w.data_ptr()), n, nb, 0) == 0
    ref = a.float()
    got = w.cpu()
    same = (got.view(torch.int32) == ref.view(torch.int32)) | (torch.isnan(got) & torch.isnan(ref))
    assert bool(same.all()), int((~same).sum())
