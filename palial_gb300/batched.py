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
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import PalialError, Status, lib, make_opts

CLASS_EDGES = (32, 64, 128, 256, 512, 1024, 2048)
CANDIDATE_BS = (64, 128, 256)

_M1, _M2, _M3, _K1 = (np.uint64(0x9E3779B97F4A7C15), np.uint64(0xBF58476D1CE4E5B9),
                      np.uint64(0x94D049BB133111EB), np.uint64(0xD1B54A32D192ED03))


def _mix(z):
    with np.errstate(over="ignore"):
        z = z + _M1
        z = (z ^ (z >> np.uint64(30))) * _M2
        z = (z ^ (z >> np.uint64(27))) * _M3
        return z ^ (z >> np.uint64(31))


def batch_sizes(count: int = 2000, seed: int = 2) -> tuple[np.ndarray, np.ndarray]:
    """(N_i, alg_i): N log-uniform in [32, 2048), alg 0 (Cholesky, SPD) for even i, 1 (LU)."""
    with np.errstate(over="ignore"):
        key = _mix(np.array([np.uint64(seed) * _K1 + np.uint64(6)], dtype=np.uint64))[0]
        r = _mix(key + np.arange(count, dtype=np.uint64))
    u = (r >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
    ns = np.minimum(np.floor(32.0 * 64.0 ** u).astype(np.int64), 2047)
    algs = (np.arange(count) % 2).astype(np.int64)
    return ns, algs


def size_class(n: int) -> int:
    for c in range(len(CLASS_EDGES) - 1):
        if n < CLASS_EDGES[c + 1]:
            return c
    return len(CLASS_EDGES) - 2


def class_label(c: int) -> str:
    return f"[{CLASS_EDGES[c]},{CLASS_EDGES[c + 1]})"


def padded(n: int, bs: int) -> int:
    return int(math.ceil(n / bs) * bs)


class Batch:
    """Device buffers of one batch (torch provides the memory) and its launch arguments."""

    def __init__(self, torch, ns, algs, bs_of_class: dict, seed: int = 2, index_base: int = 0):
        self.torch = torch
        self.ns = np.asarray(ns, dtype=np.int64)
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
                                                   int(self.np_[i]), int(self.bs[i]), seed * 100000 + index_base + i,
                                                   None)
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
        from oracle.oracle import from_tiles  # noqa: WPS433 (layout helper only)
        t = self.buf[int(self.offs[i]):int(self.offs[i + 1])].cpu().numpy()
        n, npad, bs = int(self.ns[i]), int(self.np_[i]), int(self.bs[i])
        return from_tiles(t, npad, bs)[:n, :n]

    def original(self, i: int) -> np.ndarray:
        from oracle.oracle import from_tiles  # noqa: WPS433
        t = self.pristine[int(self.offs[i]):int(self.offs[i + 1])].cpu().numpy()
        n, npad, bs = int(self.ns[i]), int(self.np_[i]), int(self.bs[i])
        return from_tiles(t, npad, bs)[:n, :n]


def autotune(torch, ns, algs, candidates=CANDIDATE_BS, reps: int = 2, seed: int = 2) -> tuple[dict, dict]:
    """Per size class, time the class's matrices alone with each candidate block size (one
    launch per repetition after a warm-up) and keep the fastest.  Returns (choice, timings)."""
    ns = np.asarray(ns)
    algs = np.asarray(algs)
    classes = sorted({size_class(int(n)) for n in ns})
    choice, timings = {}, {}
    for c in classes:
        idx = [i for i in range(len(ns)) if size_class(int(ns[i])) == c]
        best = None
        for bs in candidates:
            if bs > max(64, CLASS_EDGES[c + 1]):
                continue
            b = Batch(torch, ns[idx], algs[idx], {c: bs}, seed=seed, index_base=idx[0])
            times = []
            for r in range(reps + 1):
                b.reset()
                st, _ = b.run(graph=True)
                if r > 0:
                    times.append(st.seconds)
            t = min(times)
            timings[(c, bs)] = t
            if best is None or t < best[1]:
                best = (bs, t)
            del b
            torch.cuda.empty_cache()
        choice[c] = best[0]
    return choice, timings
