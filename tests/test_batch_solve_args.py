"""Batched solves: the argument checks, which run on the host before the device is touched,
and the loud failure without a device (no CPU fallback)."""
import ctypes

import pytest

import palial_gb300 as P
from palial_gb300 import batched as B

FAKE = 1 << 20  # a 16-byte aligned address that is never dereferenced


def _solve(ns, nbs, algs=None, precs=None, ptr=FAKE):
    count = len(ns)
    algs = algs or [0] * count
    return B.solve(algs, ns, nbs, [ptr] * count, [ptr] * count, [ptr] * count, precs=precs)


@pytest.mark.parametrize("ns,nbs,kw", [
    ([128], [48], {}),                       # tile not a multiple of 64
    ([192], [128], {}),                      # tile does not divide n
    ([8192], [256], {}),                     # above the 4096 limit of the correction solve
    ([128], [64], {"algs": [2]}),            # QR has no batched solve
    ([128], [64], {"precs": ["bf16"]}),      # FP32 or FP64 factorizations only
    ([128], [64], {"ptr": FAKE + 8}),        # A not 16-byte aligned
])
def test_bad_arguments_rejected_before_the_device(ns, nbs, kw):
    with pytest.raises(P.PalialError) as e:
        _solve(ns, nbs, **kw)
    assert e.value.code == -1


def test_empty_batches_rejected():
    lib = P.lib()
    st = P.Status()
    assert lib.palial_gpu_batched_solve(0, None, None, None, None, None, None, None, None, ctypes.byref(st), None,
                                        None, None) == -1
    assert lib.palial_gpu_batched_f32(0, None, None, None, None, None, None, None, ctypes.byref(st), None, None) == -1
    assert lib.palial_gpu_batch_solve_autotune(0, None, None, 0, 1, None, None, None, ctypes.byref(st)) == -1
    rep = B.SolveReport()
    assert lib.palial_gpu_batch_solve_synthetic(0, 2, 0, 1, 0, None, None, 1, None, ctypes.byref(st),
                                                ctypes.byref(rep)) == -1


def test_valid_arguments_need_a_device():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    with pytest.raises(P.PalialError) as e:
        _solve([128, 256], [64, 128], algs=[0, 1], precs=["fp32", "fp64"])
    assert e.value.code == -5
