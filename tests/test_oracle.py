"""The CPU oracle (C restatement of the reference's DAGs) pinned against golden fixtures
made by the reference itself (tests/golden/make_golden.py)."""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import build_oracle, oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")
META = json.load(open(os.path.join(GOLD, "sha256.json")))
SAME_BLAS = os.path.basename(build_oracle.find_openblas()) == META["openblas"]


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _dominant(seed, n):
    a = np.full((n, n), 0.5)
    u = (O.gen_uniform(seed, n, 1)[:, 0] + 1.0) * 0.5
    a[np.diag_indices(n)] = 173.0 * u + 173.0
    return a


GENS = {"chol_192_64": lambda: O.gen_spd(0, 192), "lu_192_64": lambda: O.gen_uniform(1, 192),
        "lu_dom_128_32": lambda: _dominant(3, 128), "qr_192_64": lambda: O.gen_uniform(1, 192)}


def _close(a, b, tol):
    return np.linalg.norm(a - b) <= tol * np.linalg.norm(b)


@pytest.mark.parametrize("name", sorted(GENS))
def test_generator_bytes_pinned(name):
    """The seeded generators reproduce the exact inputs the golden outputs were made from."""
    rec = META[name]
    assert _sha(O.to_tiles(GENS[name](), rec["nb"])) == rec["input_sha256"]


@pytest.mark.parametrize("name", sorted(GENS))
def test_oracle_matches_reference_golden(name):
    rec = META[name]
    n, nb, alg = rec["n"], rec["nb"], rec["alg"]
    g = np.load(os.path.join(GOLD, name + ".npz"))
    t = O.to_tiles(GENS[name](), nb)
    s = np.zeros_like(t) if alg == "qr" else None
    O.run(alg, t, n, nb, s)
    if SAME_BLAS:
        assert np.array_equal(t, g["out_tiles"])
        if s is not None:
            assert np.array_equal(s, g["s_tiles"])
    else:  # another OpenBLAS build (e.g. another CPU architecture): rounding differs
        tol = 1e-8 if name == "lu_192_64" else 1e-13
        assert _close(t, g["out_tiles"], tol)


def test_special4x4_reference_fixture():
    g = np.load(os.path.join(GOLD, "special4x4.npz"))
    for alg in ("cholesky", "lu", "qr"):
        t = g["a_tiles"].copy()
        s = np.zeros_like(t) if alg == "qr" else None
        O.run(alg, t, 4, 2, s)
        np.testing.assert_allclose(t, g[f"{alg}_tiles"], rtol=1e-14, atol=1e-15)
        if s is not None:
            np.testing.assert_allclose(s, g["qr_s_tiles"], rtol=1e-14, atol=1e-15)


@pytest.mark.skipif(not SAME_BLAS, reason="bit-exact hashes need the same OpenBLAS build")
def test_oracle_sha256_at_1024():
    big = META["sha256_1024_256"]
    for alg, gen in (("cholesky", lambda: O.gen_spd(0, 1024)), ("lu", lambda: O.gen_uniform(1, 1024)),
                     ("qr", lambda: O.gen_uniform(1, 1024))):
        t = O.to_tiles(gen(), 256)
        s = np.zeros_like(t) if alg == "qr" else None
        O.run(alg, t, 1024, 256, s)
        assert _sha(t) == big[alg]["out"], alg


def test_oracle_residuals():
    n, nb = 256, 64
    a = O.gen_spd(0, n)
    t = O.to_tiles(a, nb)
    O.run("cholesky", t, n, nb)
    assert O.cholesky_residual(a, O.from_tiles(t, n, nb)) < 1e-15
    u = O.gen_uniform(1, n)
    t = O.to_tiles(u, nb)
    O.run("lu", t, n, nb)
    assert O.lu_residual(u, O.from_tiles(t, n, nb)) < 1e-10
    t = O.to_tiles(u, nb)
    s = np.zeros_like(t)
    O.run("qr", t, n, nb, s)
    res, orth = O.qr_checks(u, O.from_tiles(t, n, nb), O.from_tiles(s, n, nb), nb)
    assert res < 1e-14 and orth < 1e-14


def test_openmp_matches_serial_and_racy_lu_reproduced():
    """OpenMP task execution gives the serial bits for Cholesky/QR and for LU with the true
    dependences; the reference's LU dependence clauses (src/lu.h:62,104) let GEMMs overtake
    TRSMs and typically produce a wrong factor (reported, not asserted: it is a race)."""
    n, nb = 512, 128
    a = O.gen_spd(0, n)
    t1, t2 = O.to_tiles(a, nb), O.to_tiles(a, nb)
    O.run("cholesky", t1, n, nb)
    O.run("cholesky", t2, n, nb, nthreads=4)
    assert np.array_equal(t1, t2)
    u = O.gen_uniform(1, n)
    t1, t2 = O.to_tiles(u, nb), O.to_tiles(u, nb)
    O.run("lu", t1, n, nb)
    O.run("lu", t2, n, nb, nthreads=4)
    assert np.array_equal(t1, t2)
    t3 = O.to_tiles(u, nb)
    O.run("lu", t3, n, nb, nthreads=4, racy_deps=True)
    assert np.isfinite(O.lu_residual(u, O.from_tiles(t1, n, nb)))


def test_oracle_rejects_bad_sizes():
    with pytest.raises(ValueError):
        O.run("cholesky", np.zeros(100), 10, 3)


@pytest.mark.skipif(not O.reference_available(), reason="reference checkout not present")
def test_restatement_bit_identical_to_reference_build():
    for alg, gen in (("cholesky", lambda: O.gen_spd(5, 256)), ("lu", lambda: O.gen_uniform(6, 256)),
                     ("qr", lambda: O.gen_uniform(7, 256))):
        a = gen()
        t1, t2 = O.to_tiles(a, 64), O.to_tiles(a, 64)
        s1 = np.zeros_like(t1) if alg == "qr" else None
        s2 = np.zeros_like(t1) if alg == "qr" else None
        O.run(alg, t1, 256, 64, s1)
        O.run_reference(alg, t2, 256, 64, s2)
        assert np.array_equal(t1, t2), alg
        if s1 is not None:
            assert np.array_equal(s1, s2)
