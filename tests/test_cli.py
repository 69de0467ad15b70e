"""The palial command line: the reference's argument handling (palial_src/main.c:57-105) is
checked on CPU (these paths never touch the GPU); the runs themselves on the GPU."""
import json
import os
import subprocess

import numpy as np
import pytest

import palial_gb300 as P

BIN = os.path.join(os.path.dirname(P.LIB_PATH), "..", "bin", "palial")


def run(*args, timeout=600):
    r = subprocess.run([BIN, *args], capture_output=True, text=True, timeout=timeout)
    return r.returncode, r.stdout


def test_binary_built():
    assert os.path.exists(BIN)


def test_missing_arguments():
    assert run() == (0, "Missing arguments.\nAborting...\n")


def test_invalid_option():
    assert run("-x") == (0, "Invalid arguments.\nAborting...\n")
    assert run("-a", "cholesky", "-m", "1024", "-b", "256", "--precision", "fp16") == \
        (0, "Invalid arguments.\nAborting...\n")


def test_help():
    assert run("-h") == (0, "HELP\n")


@pytest.mark.parametrize("m,b", [("1000", "256"), ("1024", "0"), ("0", "256")])
def test_tile_size_must_divide(m, b):
    assert run("-a", "cholesky", "-m", m, "-b", b) == (0, "Tile size does not divide the matrix size. Aborting...\n")


def test_unknown_algorithm_does_nothing():
    assert run("-a", "svd", "-m", "1024", "-b", "256") == (0, "")


def test_too_many_rhs_rejected():
    assert run("-a", "lu", "-m", "1024", "-b", "256", "--rhs", "17")[1].startswith("Invalid arguments.")
    assert run("-a", "qr", "-m", "1024", "-b", "256", "--rhs", "4", "--precision", "bf16")[1].startswith("Invalid")


def _json(out):
    return json.loads(out.strip().splitlines()[-1])


@pytest.mark.gpu
@pytest.mark.parametrize("alg", ["cholesky", "lu", "qr"])
def test_factor_runs_and_checks(alg):
    rc, out = run("-a", alg, "-m", "2048", "-b", "512", "--check", "--clocks")
    j = _json(out)
    assert rc == 0 and j["code"] == 0 and j["tflops"] > 0 and 0 <= j["residual_probe"] < 1e-14
    assert j["clocks"]["sm_mhz_device"] > 0


@pytest.mark.gpu
@pytest.mark.parametrize("alg,prec,nrhs", [("cholesky", "bf16", 4), ("lu", "fp64", 2), ("cholesky", "auto", 1),
                                           ("qr", "fp64", 3)])
def test_solve_mode(alg, prec, nrhs):
    gen = "spd" if alg == "cholesky" else "ref"
    rc, out = run("-a", alg, "-m", "2048", "-b", "512", "--gen", gen, "--precision", prec, "--rhs", str(nrhs))
    j = _json(out)
    assert rc == 0 and j["mode"] == "solve" and j["code"] in (0, 1) and j["nrhs"] == nrhs
    if alg != "qr":
        assert j["backward_error"] <= 1e-14 * 2048


@pytest.mark.gpu
def test_batch_mode():
    rc, out = run("--batch", "40", "--autotune")
    j = _json(out)
    assert rc == 0 and j["batch"] == 40 and j["matrices_per_s"] > 0
    assert sum(c["count"] for c in j["classes"]) == 40


@pytest.mark.gpu
def test_batch_solve_mode():
    rc, out = run("--batch", "40", "--solve")
    j = _json(out)
    assert rc == 0 and j["batch_solve"] == 40 and j["converged"] and j["matrices_per_s"] > 0
    assert j["max_backward_error"] <= 1e-14 * 2048 and len(j["choice"]) == 12


@pytest.mark.gpu
def test_trace_file(tmp_path):
    f = tmp_path / "t.txt"
    rc, out = run("-a", "cholesky", "-m", "2048", "-b", "512", "--block", "512", "--trace", str(f), "--quiet")
    assert rc == 0 and out == ""
    lines = f.read_text().splitlines()
    assert len(lines) == 4 + 6 + 6 + 4 and lines[0].startswith("potrf000, ")


def test_load_rejects_bad_or_mismatched_files(tmp_path):
    f = tmp_path / "a.palt"
    assert run("-a", "lu", "--load", str(f))[1].startswith("Invalid arguments.")  # missing file
    n, nb = 256, 128
    P.tiles_write(str(f), np.zeros(n * n), n, nb)
    assert run("-a", "lu", "-m", "512", "--load", str(f))[1].startswith("Invalid arguments.")
    assert run("-a", "lu", "-b", "64", "--load", str(f))[1].startswith("Invalid arguments.")


def test_butterfly_needs_lu_solve():
    assert run("-a", "cholesky", "-m", "1024", "-b", "256", "--rhs", "1", "--butterfly", "3")[1].startswith("Invalid")
    assert run("-a", "lu", "-m", "1024", "-b", "256", "--butterfly", "3")[1].startswith("Invalid")


@pytest.mark.gpu
def test_save_load_roundtrip(tmp_path):
    """The generated input saved, loaded back and factored gives the same factors (bit for bit:
    the schedule-independent FP64 path), and the saved factors read back as a tile matrix."""
    src, f1, f2 = tmp_path / "in.palt", tmp_path / "f1.palt", tmp_path / "f2.palt"
    rc, out = run("-a", "lu", "-m", "1024", "-b", "256", "--gen", "uniform", "--seed", "4", "--save", str(src),
                  "--save-result", str(f1))
    assert rc == 0 and _json(out)["code"] == 0
    rc, out = run("-a", "lu", "--load", str(src), "--save-result", str(f2))
    j = _json(out)
    assert rc == 0 and j["code"] == 0 and (j["n"], j["nb"]) == (1024, 256)
    a, n, nb = P.tiles_read(str(f1))
    b, _, _ = P.tiles_read(str(f2))
    assert (n, nb) == (1024, 256) and np.array_equal(a, b)
    orig, _, _ = P.tiles_read(str(src))
    assert not np.array_equal(orig, a)


@pytest.mark.gpu
def test_butterfly_solve_mode(tmp_path):
    """A block anti-diagonal matrix written as a tile file: the plain no-pivot LU fails at its
    zero pivot, the butterfly-preconditioned solve reaches the FP64 target."""
    from oracle import oracle as O
    n, nb, h = 1024, 256, 512
    g = O.gen_uniform(21, n)
    a = np.zeros((n, n))
    a[:h, h:] = np.eye(h) + 0.5 * g[:h, :h] / np.sqrt(h)
    a[h:, :h] = np.eye(h) + 0.5 * g[h:, h:] / np.sqrt(h)
    f = tmp_path / "a.palt"
    P.tiles_write(str(f), O.to_tiles(a, nb), n, nb)
    rc, out = run("--load", str(f), "-a", "lu", "--precision", "bf16x3", "--rhs", "2")
    assert rc == 1 and _json(out)["code"] < 0
    rc, out = run("--load", str(f), "-a", "lu", "--precision", "bf16x3", "--rhs", "2", "--butterfly", "5")
    j = _json(out)
    assert rc == 0 and j["code"] in (0, 1) and j["backward_error"] <= 1e-14 * n
