"""Batched uneven factorizations in one persistent launch (+ CUDA graph), with a per-size-class
autotuner.

The batch (``batch_sizes``): ``count`` matrices, N_i = floor(32 * 64**u_i) with u_i uniform in
[0, 1) (log-uniform in [32, 2048)) from a counter-based generator (seed, index i); even i are
SPD (B B^T + N I, Cholesky), odd i are uniform [-1, 1) (no-pivot LU).  Each matrix is stored
in its own tile-layout buffer padded to a multiple of its block size (identity padding for LU,
N*I for Cholesky: the leading factor is exact).  All matrices' task DAGs run in a single
persistent scheduler launch, optionally replayed from a CUDA graph.

The autotuner times each size class alone with every candidate block size and keeps the
fastest; the per-class choice is then used for the whole batch.

Batched solves (``solve``, ``solve_synthetic``): A_i x_i = b_i to FP64-level backward error,
each matrix factored in FP32 (all FP32 matrices in one persistent launch of the FP32 task
scheduler) or FP64 and refined with FP64 residuals; a matrix whose FP32 factorization breaks
down or whose refinement stalls is refactored in FP64.  The solve autotuner picks block size
and precision per (algorithm, size class).
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import PREC, PalialError, Status, lib, make_opts

CLASS_EDGES = (32, 64, 128, 256, 512, 1024, 2048)
CANDIDATE_BS = (64, 128, 256)


class SolveReport(ctypes.Structure):
    _fields_ = [("count", ctypes.c_int), ("bs_of_class", ctypes.c_int * 12), ("prec_of_class", ctypes.c_int * 12),
                ("fallbacks", ctypes.c_int), ("butterflies", ctypes.c_int), ("max_iters", ctypes.c_int),
                ("not_converged", ctypes.c_int),
                ("seconds", ctypes.c_double), ("matrices_per_s", ctypes.c_double), ("tflops", ctypes.c_double),
                ("max_backward_error", ctypes.c_double), ("autotune_seconds", ctypes.c_double),
                ("autotune_s", ctypes.c_double * 108), ("phase_seconds", ctypes.c_double * 3)]


class BatchReport(ctypes.Structure):
    _fields_ = [("count", ctypes.c_int), ("bs_of_class", ctypes.c_int * 6), ("count_of_class", ctypes.c_int * 6),
                ("seconds", ctypes.c_double), ("matrices_per_s", ctypes.c_double), ("tflops", ctypes.c_double),
                ("p50_ms", ctypes.c_double * 6), ("p99_ms", ctypes.c_double * 6),
                ("autotune_seconds", ctypes.c_double), ("autotune_s", ctypes.c_double * 18)]


def _ints(a) -> ctypes.Array:
    a = [int(x) for x in a]
    return (ctypes.c_int * max(1, len(a)))(*a)


def batch_sizes(count: int = 2000, seed: int = 2) -> tuple[np.ndarray, np.ndarray]:
    """(N_i, alg_i) of the synthetic batch (the library's generator): N log-uniform in
    [32, 2048), alg 0 (Cholesky, SPD) for even i, 1 (LU) for odd i."""
    ns = (ctypes.c_int * max(1, count))()
    algs = (ctypes.c_int * max(1, count))()
    _check_rc(lib().palial_gpu_batch_sizes(count, ctypes.c_uint64(seed), ns, algs))
    return np.array(ns[:count], dtype=np.int64), np.array(algs[:count], dtype=np.int64)


def partition(ns, algs, world: int) -> np.ndarray:
    """Size-balanced owner rank of every matrix (the library's LPT partition; identical on
    every rank, so sharding a batch needs no collective)."""
    count = len(ns)
    out = (ctypes.c_int * max(1, count))()
    _check_rc(lib().palial_gpu_batch_partition(count, _ints(ns), _ints(algs), world, out))
    return np.array(out[:count], dtype=np.int64)


def _check_rc(rc: int) -> None:
    if rc:
        raise PalialError(rc, "batch call failed")


def size_class(n: int) -> int:
    for c in range(len(CLASS_EDGES) - 1):
        if n < CLASS_EDGES[c + 1]:
            return c
    return len(CLASS_EDGES) - 2


def class_label(c: int) -> str:
    return f"[{CLASS_EDGES[c]},{CLASS_EDGES[c + 1]})"


def _dense(t: np.ndarray, n: int, nb: int) -> np.ndarray:
    """Tile-layout buffer (tile (m, k) at nb*nb*(m + (n/nb)*k), column-major inside) -> the
    dense n x n matrix indexed [row, col]."""
    mt = n // nb
    return np.ascontiguousarray(t.reshape(mt, mt, nb, nb).transpose(1, 3, 0, 2).reshape(n, n))


def padded(n: int, bs: int) -> int:
    return int(math.ceil(n / bs) * bs)


class Batch:
    """Device buffers of one batch (torch provides the memory) and its launch arguments."""

    def __init__(self, torch, ns, algs, bs_of_class: dict, seed: int = 2, index_base: int = 0, indices=None):
        self.torch = torch
        self.ns = np.asarray(ns, dtype=np.int64)
        # batch index of every matrix (its generator seed): index_base + i unless given
        self.indices = (np.arange(len(self.ns)) + index_base) if indices is None else np.asarray(indices)
        self.algs = np.asarray(algs, dtype=np.int64)
        self.count = len(self.ns)
        self.bs = np.array([bs_of_class[size_class(int(n))] for n in self.ns], dtype=np.int32)
        self.np_ = np.array([padded(int(n), int(b)) for n, b in zip(self.ns, self.bs)], dtype=np.int32)
        sizes = self.np_.astype(np.int64) ** 2
        offs = np.concatenate([[0], np.cumsum(sizes)])
        self.buf = torch.empty(int(offs[-1]), dtype=torch.float64, device="cuda")
        base = self.buf.data_ptr()
        self.ptrs = (ctypes.c_void_p * self.count)(*[base + 8 * int(o) for o in offs[:-1]])
        self.offs = offs
        for i in range(self.count):
            rc = lib().palial_gpu_gen_batch_matrix(self.ptrs[i], 1 if self.algs[i] == 0 else 0, int(self.ns[i]),
                                                   int(self.np_[i]), int(self.bs[i]),
                                                   seed * 100000 + int(self.indices[i]), None)
            if rc:
                raise PalialError(rc, f"generating matrix {i}")
        torch.cuda.synchronize()
        self.pristine = self.buf.clone()
        self.flops = float(sum(n ** 3 / 3.0 if a == 0 else 2.0 * n ** 3 / 3.0 for n, a in zip(self.ns, self.algs)))
        self._args = [(ctypes.c_int * self.count)(*[int(x) for x in arr])
                      for arr in (self.algs, self.np_, self.bs, self.bs)]

    def reset(self):
        self.buf.copy_(self.pristine)

    def run(self, graph: bool = True, completion: bool = False) -> tuple[Status, np.ndarray | None]:
        o = make_opts()
        o.reserved[2] = 1 if graph else 0
        st = Status()
        comp = (ctypes.c_double * self.count)() if completion else None
        a, n, nb, bs = self._args
        rc = lib().palial_gpu_batched(self.count, a, n, nb, bs, self.ptrs, ctypes.byref(o), ctypes.byref(st),
                                      comp, None)
        st.code = rc
        if rc < 0:
            raise PalialError(rc, st.message.decode(errors="replace"))
        return st, (np.frombuffer(comp, dtype=np.float64).copy() if completion else None)

    def factor(self, i: int) -> np.ndarray:
        """Factored matrix i, leading n x n block, as a dense [row, col] array (host)."""
        t = self.buf[int(self.offs[i]):int(self.offs[i + 1])].cpu().numpy()
        n, npad, bs = int(self.ns[i]), int(self.np_[i]), int(self.bs[i])
        return _dense(t, npad, bs)[:n, :n]

    def original(self, i: int) -> np.ndarray:
        t = self.pristine[int(self.offs[i]):int(self.offs[i + 1])].cpu().numpy()
        n, npad, bs = int(self.ns[i]), int(self.np_[i]), int(self.bs[i])
        return _dense(t, npad, bs)[:n, :n]


def autotune(torch, ns, algs, candidates=CANDIDATE_BS, reps: int = 2, seed: int = 2) -> tuple[dict, dict]:
    """Per size class, the fastest candidate block size (the library's autotuner: each class's
    matrices alone in a batched launch per candidate).  Returns (choice, timings) with
    choice[class] = block size and timings[(class, bs)] = seconds.  `torch` and `candidates`
    are accepted for the older signature; the candidates are 64, 128, 256."""
    del torch, candidates
    ns = np.asarray(ns)
    algs = np.asarray(algs)
    cls = (ctypes.c_int * 6)()
    tim = (ctypes.c_double * 18)()
    st = Status()
    rc = lib().palial_gpu_batch_autotune(len(ns), _ints(ns), _ints(algs), ctypes.c_uint64(seed), reps, cls, tim,
                                         ctypes.byref(st))
    if rc:
        raise PalialError(rc, st.message.decode(errors="replace"))
    present = sorted({size_class(int(n)) for n in ns})
    choice = {c: int(cls[c]) for c in present}
    timings = {(c, bs): float(tim[c * 3 + j]) for c in present for j, bs in enumerate(CANDIDATE_BS)
               if tim[c * 3 + j] >= 0}
    return choice, timings


def synthetic(count: int = 2000, seed: int = 2, rank: int = 0, world: int = 1, autotune: bool = True,
              bs_of_class=None, reps: int = 3) -> dict:
    """Run this rank's share of the synthetic batch entirely inside the library; returns the
    report as a dict."""
    rep = BatchReport()
    st = Status()
    cls = (ctypes.c_int * 6)(*bs_of_class) if bs_of_class is not None else None
    rc = lib().palial_gpu_batch_synthetic(count, ctypes.c_uint64(seed), rank, world, int(autotune), cls, reps,
                                          ctypes.byref(make_opts()), ctypes.byref(st), ctypes.byref(rep))
    if rc:
        raise PalialError(rc, st.message.decode(errors="replace"))
    out = {f: getattr(rep, f) for f, _ in BatchReport._fields_}
    for f in ("bs_of_class", "count_of_class", "p50_ms", "p99_ms", "autotune_s"):
        out[f] = list(out[f])
    return out


def _ptrs(ptrs) -> ctypes.Array:
    return (ctypes.c_void_p * max(1, len(ptrs)))(*[int(p) for p in ptrs])


def factor_f32(algs, ns, nbs, ptrs, bss=None) -> tuple[Status, np.ndarray]:
    """FP32 factorizations of FP32 tile-layout device buffers in one persistent launch (the
    batched solves' factorization).  Returns (status, breakdown flags per matrix)."""
    count = len(ns)
    flags = (ctypes.c_int * max(1, count))()
    st = Status()
    rc = lib().palial_gpu_batched_f32(count, _ints(algs), _ints(ns), _ints(nbs), _ints(nbs if bss is None else bss),
                                      _ptrs(ptrs), flags, ctypes.byref(make_opts()), ctypes.byref(st), None, None)
    st.code = rc
    if rc < 0:
        raise PalialError(rc, st.message.decode(errors="replace"))
    return st, np.array(flags[:count], dtype=np.int64)


def solve(algs, ns, nbs, a_ptrs, b_ptrs, x_ptrs, precs=None, ir_tol: float = 0.0, ir_max_iter: int = 0,
          allow_not_converged: bool = False) -> tuple[Status, np.ndarray, np.ndarray]:
    """Batched solves A_i x_i = b_i (device buffers: A in the tile layout with tile nbs[i], b and
    x of ns[i] doubles).  precs[i]: "fp32" (default), "bf16x3" (FP32 with its updates on the tensor
    cores as BF16x3 products) or "fp64" factorization.  Returns (status,
    iters, backward errors); iters[i] < 0 marks a matrix refactored in FP64 after its FP32
    attempt (-(steps + 1))."""
    count = len(ns)
    pr = None if precs is None else _ints([PREC[p] if isinstance(p, str) else int(p) for p in precs])
    iters = (ctypes.c_int * max(1, count))()
    berr = (ctypes.c_double * max(1, count))()
    st = Status()
    o = make_opts(ir_tol=ir_tol, ir_max_iter=ir_max_iter)
    rc = lib().palial_gpu_batched_solve(count, _ints(algs), _ints(ns), _ints(nbs), _ptrs(a_ptrs), _ptrs(b_ptrs),
                                        _ptrs(x_ptrs), pr, ctypes.byref(o), ctypes.byref(st), iters, berr, None)
    st.code = rc
    if rc < 0 and not (allow_not_converged and rc == -6):
        raise PalialError(rc, st.message.decode(errors="replace"))
    return st, np.array(iters[:count], dtype=np.int64), np.array(berr[:count], dtype=np.float64)


def solve_synthetic(count: int = 2000, seed: int = 2, rank: int = 0, world: int = 1, autotune: bool = True,
                    bs12=None, prec12=None, reps: int = 3, butterflies: int = 0) -> dict:
    """Batched solves of this rank's share of the synthetic batch, inside the library; block and
    precision per [alg * 6 + size class] from the autotuner or the arguments.  butterflies: 0 =
    an FP32 LU that fails gets a second attempt on its random-butterfly transform, 1 = every
    FP32 LU on its transform from the start, -1 = never.  Returns the report as a dict."""
    rep = SolveReport()
    st = Status()
    b12 = (ctypes.c_int * 12)(*bs12) if bs12 is not None else None
    p12 = (ctypes.c_int * 12)(*prec12) if prec12 is not None else None
    o = make_opts()
    o.reserved[6] = butterflies
    rc = lib().palial_gpu_batch_solve_synthetic(count, ctypes.c_uint64(seed), rank, world, int(autotune), b12, p12,
                                                reps, ctypes.byref(o), ctypes.byref(st), ctypes.byref(rep))
    if rc and rc != -6:
        raise PalialError(rc, st.message.decode(errors="replace"))
    out = {f: getattr(rep, f) for f, _ in SolveReport._fields_}
    for f in ("bs_of_class", "prec_of_class", "autotune_s", "phase_seconds"):
        out[f] = list(out[f])
    out["rc"] = rc
    return out
