"""CPU oracle: loader, seeded generators, tile layout helpers and residual checks.

TEST INFRASTRUCTURE ONLY.  Used by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg as the checker.  The GPU library never imports it.

* ``run(alg, a_tiles, ...)`` calls the C restatement of the reference's DAGs
  (palial_oracle.c) over SciPy's OpenBLAS, serially (parity) or as OpenMP tasks (timing).
* ``run_reference(...)`` calls the reference's own sources compiled by build_oracle.py
  into oracle/_ref/ (only where a reference checkout exists).
* Generators are counter-based (splitmix64 of the global column-major index), so the GPU
  generators in the product reproduce the same bytes.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

# The tile kernels must run single-threaded inside OpenMP tasks (the reference's runs set
# OPENBLAS_NUM_THREADS=1); SciPy's OpenBLAS reads this when it is first loaded.
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")

HERE = os.path.dirname(os.path.abspath(__file__))
ALG = {"cholesky": 0, "lu": 1, "qr": 2}

# --------------------------------------------------------------------------------------
# Loading
# --------------------------------------------------------------------------------------
_lib = None
_ref = {}


def _dp():
    return ctypes.POINTER(ctypes.c_double)


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            from . import build_oracle  # noqa: WPS433
            build_oracle.build_oracle()
        _lib = ctypes.CDLL(path)
        _lib.orc_run.restype = ctypes.c_double
        _lib.orc_run.argtypes = [ctypes.c_int] * 3 + [_dp(), _dp(), ctypes.c_int, ctypes.c_int]
        _lib.orc_max_threads.restype = ctypes.c_int
        for name, nargs in (("orc_dgetrf_nopiv", None),):
            getattr(_lib, name).restype = ctypes.c_int
    return _lib


def reference_available() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libpalial_ref_serial.so"))


def ref_lib(openmp: bool = False):
    key = "omp" if openmp else "serial"
    if key not in _ref:
        path = os.path.join(HERE, "_ref", f"libpalial_ref_{key}.so")
        h = ctypes.CDLL(path)
        h.ref_run.restype = ctypes.c_double
        h.ref_run.argtypes = [ctypes.c_int] * 3 + [_dp(), _dp(), ctypes.c_int]
        _ref[key] = h
    return _ref[key]


def _ptr(a: np.ndarray | None):
    if a is None:
        return ctypes.cast(None, _dp())
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp())


def run(alg: str, a_tiles: np.ndarray, n: int, nb: int, s_tiles: np.ndarray | None = None,
        nthreads: int = 1, racy_deps: bool = False) -> float:
    """Run the restated reference DAG in place on tile-layout buffers; returns seconds."""
    t = lib().orc_run(ALG[alg], n, nb, _ptr(a_tiles), _ptr(s_tiles), int(nthreads), int(racy_deps))
    if t < 0:
        raise ValueError("oracle rejected the arguments (N % NB != 0, or QR without S)")
    return t


def run_reference(alg: str, a_tiles: np.ndarray, n: int, nb: int,
                  s_tiles: np.ndarray | None = None, nthreads: int = 1, openmp: bool = False) -> float:
    """Run the reference's own compiled sources in place on tile-layout buffers."""
    h = ref_lib(openmp)
    return h.ref_run(ALG[alg], n, nb, _ptr(a_tiles), _ptr(s_tiles), int(nthreads))


# --------------------------------------------------------------------------------------
# Tile layout (include/tile_address.h:9-17)
# --------------------------------------------------------------------------------------
def to_tiles(a: np.ndarray, nb: int) -> np.ndarray:
    """Full M x N matrix (indexed a[i, j]) -> flat tile-layout buffer: tile (m, n) at element
    nb*nb*(m + (M/nb)*n), column-major inside (reference include/tile_address.h:9-17)."""
    mt, nt = a.shape[0] // nb, a.shape[1] // nb
    return np.ascontiguousarray(a.reshape(mt, nb, nt, nb).transpose(2, 0, 3, 1)).ravel()


def from_tiles(t: np.ndarray, n: int, nb: int, cols: int | None = None) -> np.ndarray:
    """Flat tile-layout buffer -> full n x cols (default n x n) matrix indexed [i, j]."""
    cols = n if cols is None else cols
    mt, nt = n // nb, cols // nb
    return np.ascontiguousarray(t.reshape(nt, mt, nb, nb).transpose(1, 3, 0, 2).reshape(n, cols))


# --------------------------------------------------------------------------------------
# Counter-based generators (identical bytes on CPU and GPU)
# --------------------------------------------------------------------------------------
_M1 = np.uint64(0x9E3779B97F4A7C15)
_M2 = np.uint64(0xBF58476D1CE4E5B9)
_M3 = np.uint64(0x94D049BB133111EB)
_K1 = np.uint64(0xD1B54A32D192ED03)

STREAM_UNIFORM, STREAM_SPD, STREAM_RHS, STREAM_HOUSE = 0, 1, 2, 3


def _mix(z):
    with np.errstate(over="ignore"):
        z = z + _M1
        z = (z ^ (z >> np.uint64(30))) * _M2
        z = (z ^ (z >> np.uint64(27))) * _M3
        return z ^ (z >> np.uint64(31))


def stream_key(seed: int, stream: int) -> np.uint64:
    with np.errstate(over="ignore"):
        return _mix(np.array([np.uint64(seed) * _K1 + np.uint64(stream)], dtype=np.uint64))[0]


def rand_u64(seed: int, stream: int, idx: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        return _mix(stream_key(seed, stream) + idx.astype(np.uint64))


def uniform_from_bits(r: np.ndarray) -> np.ndarray:
    """Top 53 bits -> double uniform in [-1, 1): (r >> 11) * 2^-52 - 1 (exact)."""
    return (r >> np.uint64(11)).astype(np.float64) * (2.0 ** -52) - 1.0


def int8_from_bits(r: np.ndarray) -> np.ndarray:
    """Top 8 bits -> integer in [-128, 127]."""
    return (r >> np.uint64(56)).astype(np.int64) - 128


def _global_index(rows: int, cols: int) -> np.ndarray:
    i = np.arange(rows, dtype=np.uint64)[:, None]
    j = np.arange(cols, dtype=np.uint64)[None, :]
    return i + j * np.uint64(rows)


def gen_uniform(seed: int, n: int, cols: int | None = None, stream: int = STREAM_UNIFORM) -> np.ndarray:
    """Matrix (n x cols) with iid entries uniform in [-1, 1); entry (i, j) uses index i + j*n."""
    cols = n if cols is None else cols
    return uniform_from_bits(rand_u64(seed, stream, _global_index(n, cols)))


def gen_spd_int(seed: int, n: int) -> np.ndarray:
    """Integer matrix K (n x n) in [-128, 127]; B = K / 128 is uniform on a 2^-7 grid in [-1, 1)."""
    return int8_from_bits(rand_u64(seed, STREAM_SPD, _global_index(n, n)))


def gen_spd(seed: int, n: int) -> np.ndarray:
    """A = B B^T + n I with B = K/128, computed exactly (integer products, exact sums)."""
    k = gen_spd_int(seed, n).astype(np.float64)
    g = k @ k.T                    # exact: |entries| <= 2^29, integer-valued
    a = g * (2.0 ** -14)           # exact power-of-two scaling
    a[np.diag_indices(n)] += float(n)
    return a


# --------------------------------------------------------------------------------------
# Checks
# --------------------------------------------------------------------------------------
def fro(x: np.ndarray) -> float:
    return float(np.linalg.norm(x))


def cholesky_residual(a: np.ndarray, u: np.ndarray) -> float:
    """||A - U^T U||_F / ||A||_F with U = upper triangle of the factored matrix."""
    uu = np.triu(u)
    return fro(a - uu.T @ uu) / fro(a)


def lu_residual(a: np.ndarray, f: np.ndarray) -> float:
    """||A - L U||_F / ||A||_F with L unit lower (strict lower of f) and U upper of f."""
    l = np.tril(f, -1) + np.eye(f.shape[0])
    return fro(a - l @ np.triu(f)) / fro(a)


def qr_apply_qt(f: np.ndarray, s: np.ndarray, nb: int, c: np.ndarray) -> np.ndarray:
    """Apply Q^T of the flat-tree tile QR (factors f, T factors s, both full matrices) to c.

    Follows the transform order of src/qr.h:15-192: for each k, the GEQRT block reflector
    of tile row k, then the TS block reflectors coupling tile rows k and m > k.  f may be tall
    (rows x cols factors of the same algorithm on a rectangular tile grid).
    """
    mt, nt = f.shape[0] // nb, f.shape[1] // nb
    c = c.copy()
    blk = lambda i: slice(i * nb, (i + 1) * nb)  # noqa: E731
    for k in range(nt):
        v = np.tril(f[blk(k), blk(k)], -1) + np.eye(nb)
        t = np.triu(s[blk(k), blk(k)])
        c[blk(k)] -= v @ (t.T @ (v.T @ c[blk(k)]))
        for m in range(k + 1, mt):
            v2 = f[blk(m), blk(k)]
            t2 = np.triu(s[blk(m), blk(k)])
            w = t2.T @ (c[blk(k)] + v2.T @ c[blk(m)])
            c[blk(k)] -= w
            c[blk(m)] -= v2 @ w
    return c


def r_upper(f: np.ndarray, nb: int) -> np.ndarray:
    """R of the tile QR: the upper triangle of the top cols x cols tile block of the factors."""
    cols = f.shape[1]
    return np.triu(f[:cols, :cols])


def qr_solve(f: np.ndarray, s: np.ndarray, nb: int, b: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Solve / least squares with the tile QR factors: y = Q^T b, x = R^-1 y(0:cols); returns
    (x, ||y(cols:rows)||_2 per column)."""
    import scipy.linalg as sl

    cols = f.shape[1]
    y = qr_apply_qt(f, s, nb, b.reshape(f.shape[0], -1))
    x = sl.solve_triangular(r_upper(f, nb), y[:cols], lower=False)
    return x, np.linalg.norm(y[cols:], axis=0)


def qr_checks(a: np.ndarray, f: np.ndarray, s: np.ndarray, nb: int) -> tuple[float, float]:
    """(||Q^T A - R||_F / ||A||_F, ||Q^T Q - I||_F / sqrt(n)) for the tile QR."""
    n = a.shape[0]
    r = np.triu(f)
    # R lives in the upper triangle of the tile matrix (diagonal tiles: upper triangle;
    # tiles above the diagonal: full).  Below-diagonal tiles hold V.
    mt = n // nb
    rr = np.zeros_like(f)
    for k in range(mt):
        for j in range(k, mt):
            blkk = f[k * nb:(k + 1) * nb, j * nb:(j + 1) * nb]
            rr[k * nb:(k + 1) * nb, j * nb:(j + 1) * nb] = np.triu(blkk) if j == k else blkk
    del r
    qta = qr_apply_qt(f, s, nb, a)
    res = fro(qta - rr) / fro(a)
    qt = qr_apply_qt(f, s, nb, np.eye(n))
    orth = fro(qt @ qt.T - np.eye(n)) / np.sqrt(n)
    return res, orth


def r_factor(f: np.ndarray, nb: int) -> np.ndarray:
    n = f.shape[0]
    mt = n // nb
    rr = np.zeros_like(f)
    for k in range(mt):
        for j in range(k, mt):
            blkk = f[k * nb:(k + 1) * nb, j * nb:(j + 1) * nb]
            rr[k * nb:(k + 1) * nb, j * nb:(j + 1) * nb] = np.triu(blkk) if j == k else blkk
    return rr
