"""Host logic of the device scheduler: task counts, dependence validity, emulation with
random durations, and the C ABI exports.  No GPU needed (no compute calls)."""
import re

import numpy as np
import os

import pytest

import palial_gb300 as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol():
    names = set()
    for hdr in os.listdir(os.path.join(ROOT, "include")):
        if hdr.endswith(".h"):
            src = open(os.path.join(ROOT, "include", hdr)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            # prototypes only: a return type before the name, ';' after the parameter list
            # (header-defined helpers of palial_entry.h, calls inside them and the caller's weak
            # trace hooks are not exports)
            names |= set(re.findall(r"^[ \t]*(?:\w+[ \t\*]+)+(palial_\w+)\s*\((?:[^;{()]|\([^()]*\))*\)\s*;", src,
                                    flags=re.M))
    assert names
    lib = P.lib()
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


@pytest.mark.parametrize("mt", [1, 2, 3, 5, 8])
def test_cholesky_task_counts(mt):
    d = P.dag_info("cholesky", 512 * mt, 512, block=512)
    c = d["type_counts"]
    assert c[0] == mt and c[1] == mt * (mt - 1) // 2 and c[2] == mt * (mt - 1) // 2
    assert c[3] == mt * (mt - 1) * (mt - 2) // 6


@pytest.mark.parametrize("mt", [1, 2, 4, 7])
def test_lu_task_counts(mt):
    c = P.dag_info("lu", 256 * mt, 256, block=256)["type_counts"]
    assert c[4] == mt and c[5] == mt * (mt - 1) // 2 and c[6] == mt * (mt - 1) // 2
    assert c[7] == (mt - 1) * mt * (2 * mt - 1) // 6


@pytest.mark.parametrize("mt", [1, 2, 4, 6])
def test_qr_task_counts(mt):
    c = P.dag_info("qr", 128 * mt, 128)["type_counts"]
    assert c[8] == mt and c[9] == mt * (mt - 1) // 2 and c[10] == mt * (mt - 1) // 2
    assert c[11] == sum((mt - 1 - k) ** 2 for k in range(mt))


@pytest.mark.parametrize("alg", ["cholesky", "lu", "qr"])
@pytest.mark.parametrize("priority", [0, 1])
@pytest.mark.parametrize("workers", [1, 3, 152])
def test_dag_validates(alg, priority, workers):
    assert P.dag_validate(alg, 2048, 256, block=128 if alg != "qr" else 0, priority=priority,
                          nworkers=workers, seed=workers) == ""


def test_critical_path_order_beats_program_order_in_model():
    a = P.dag_info("cholesky", 16384, 512, priority=0, nworkers=152)
    b = P.dag_info("cholesky", 16384, 512, priority=1, nworkers=152)
    assert a["makespan_s"] <= b["makespan_s"] * 1.0001


def test_bad_sizes_rejected():
    with pytest.raises(P.PalialError):
        P.dag_info("cholesky", 1000, 512)


def test_batch_sizes_log_uniform_and_split():
    from palial_gb300 import batched as B
    ns, algs = B.batch_sizes(2000, 2)
    assert ns.min() >= 32 and ns.max() < 2048
    # log-uniform: about 1/6 of the mass in each octave pair of [32, 2048)
    counts = np.bincount([B.size_class(int(n)) for n in ns], minlength=6)
    assert all(abs(c / 2000 - 1 / 6) < 0.05 for c in counts)
    assert (algs == np.arange(2000) % 2).all()
    ns2, _ = B.batch_sizes(2000, 2)
    assert (ns == ns2).all()


def test_batch_dag_validates_and_isolates_matrices():
    import ctypes
    from palial_gb300 import batched as B
    ns, algs = B.batch_sizes(60, 3)
    bs = [64 if n < 256 else 128 for n in ns]
    npad = [B.padded(int(n), b) for n, b in zip(ns, bs)]
    arr = lambda x: (ctypes.c_int * len(x))(*[int(v) for v in x])  # noqa: E731
    buf = ctypes.create_string_buffer(256)
    rc = P.lib().palial_dag_batch_validate(60, arr(algs), arr(npad), arr(bs), arr(bs), 152, 5, buf, 256)
    assert rc == 0, buf.value
    # 64-blocks inside larger tiles (the batched solves' FP64 factorizations)
    tiles = [64 if n < 128 else (128 if n < 1024 else 256) for n in ns]
    npad = [B.padded(int(n), t) for n, t in zip(ns, tiles)]
    rc = P.lib().palial_dag_batch_validate(60, arr(algs), arr(npad), arr(tiles), arr([64] * 60), 152, 7, buf, 256)
    assert rc == 0, buf.value


def _names(alg, n, nb, block):
    import ctypes
    lib = P.lib()
    lib.palial_dag_names.restype = ctypes.c_longlong
    lib.palial_dag_names.argtypes = [ctypes.c_int] * 4 + [ctypes.c_char_p, ctypes.c_longlong]
    need = lib.palial_dag_names({"cholesky": 0, "lu": 1, "qr": 2}[alg], n, nb, block, None, 0)
    buf = ctypes.create_string_buffer(need)
    lib.palial_dag_names({"cholesky": 0, "lu": 1, "qr": 2}[alg], n, nb, block, buf, need)
    return buf.value.decode().split()


def test_task_names_equal_reference_published_trace():
    """The reference's own trace of Cholesky N=8192 NB=512 (exp/data, first column): same
    names, same creation order, stale loop variables included (potrf11615 ...)."""
    gold = open(os.path.join(ROOT, "tests", "golden", "trace_names_cholesky_8192_512.txt")).read().split()
    assert _names("cholesky", 8192, 512, 512) == gold
    assert "potrf11615" in gold


def test_task_names_lu_qr_follow_loop_rule():
    """Names from the reference's loops (src/lu.h:14-144, src/qr.h:18-158): k, m, n are
    function-scope ints, so a name takes whatever value the last finished loop left."""
    lu = _names("lu", 2048, 512, 512)
    assert lu[:9] == ["getrf000", "trsm010", "trsm020", "trsm030", "trsm041", "gemm011", "gemm021",
                      "gemm031", "trsm042"]
    assert lu[16] == "getrf144" and len(lu) == 4 + 6 + 6 + 14
    qr = _names("qr", 1024, 512, 512)
    assert qr == ["geqrt000", "ormqr001", "tsqrt012", "tsmqr011", "geqrt122"]
