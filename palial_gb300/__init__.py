"""palial_gb300 -- GB300 (sm_103a) tiled dense Cholesky / LU / QR behind PALIAL's interface.

Python mirror of the reference's entry points (reference src/cholesky.h:12 ``cholesky(A)``,
src/lu.h:11 ``lu(A)``, src/qr.h:15 ``qr(A, S)``) over the C ABI of libpalial_gpu.so
(include/palial_gpu.h).  Matrices are flat float64 buffers in the reference's tile layout
(include/tile_address.h:9-17); factorizations run in place, on the GPU only.  There is no CPU
fallback: if the library or a device is missing, every call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libpalial_gpu.so")

PALIAL_OK = 0
ERR = {
    -1: "bad argument", -2: "CUDA error", -3: "matrix is not positive definite",
    -4: "device dependency wait timed out", -5: "no CUDA device", -6: "refinement did not converge",
    -7: "device allocation failed", 1: "exact zero pivot skipped",
}
ALG = {"cholesky": 0, "lu": 1, "qr": 2}
PREC = {"fp64": 0, "bf16": 1, "fp8": 2, "bf16x3": 3, "auto": 4, "fp32": 5, "tf32x3": 6}
PREC_NAME = {v: k for k, v in PREC.items()}
PREC_NAME[100 + PREC["bf16x3"]] = "bf16x3-rbt"  # AUTO ladder rung: BF16x3 on the butterfly transform


class PalialError(RuntimeError):
    def __init__(self, code: int, msg: str = ""):
        super().__init__(f"palial error {code} ({ERR.get(code, '?')}): {msg}")
        self.code = code


class Desc(ctypes.Structure):
    """Same layout as the reference's MATRIX_desc (include/descriptor.h:13-20)."""
    _fields_ = [("tile_size", ctypes.c_int), ("matrix_nelements", ctypes.c_long),
                ("tile_nelements", ctypes.c_long), ("matrix_size", ctypes.c_int),
                ("matrix", ctypes.c_void_p)]


class Opts(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("block", ctypes.c_int), ("workers_per_sm", ctypes.c_int),
                ("max_sms", ctypes.c_int), ("priority", ctypes.c_int), ("trace", ctypes.c_int),
                ("timeout_s", ctypes.c_double), ("shuffle_seed", ctypes.c_uint), ("ir_max_iter", ctypes.c_int),
                ("ir_tol", ctypes.c_double), ("gmres", ctypes.c_int), ("reserved", ctypes.c_int * 8)]


class Status(ctypes.Structure):
    _fields_ = [("code", ctypes.c_int), ("cuda_error", ctypes.c_int), ("task", ctypes.c_int),
                ("tile_m", ctypes.c_int), ("tile_n", ctypes.c_int), ("column", ctypes.c_int),
                ("ntasks", ctypes.c_longlong), ("seconds", ctypes.c_double), ("total_seconds", ctypes.c_double),
                ("tflops", ctypes.c_double), ("ir_iters", ctypes.c_int), ("gmres_iters", ctypes.c_int),
                ("backward_error", ctypes.c_double), ("kappa_est", ctypes.c_double),
                ("factor_seconds", ctypes.c_double), ("shift", ctypes.c_double),
                ("precision_used", ctypes.c_int), ("fallbacks", ctypes.c_int), ("butterflies", ctypes.c_int),
                ("message", ctypes.c_char * 160)]

    def as_dict(self) -> dict:
        d = {f: getattr(self, f) for f, _ in self._fields_ if f != "message"}
        d["message"] = self.message.decode(errors="replace")
        return d


_lib = None


def lib() -> ctypes.CDLL:
    """Load libpalial_gpu.so (built by palial_gb300/build.py); raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise PalialError(-5, f"{LIB_PATH} not built (run __graft_entry__.build())")
        h = ctypes.CDLL(LIB_PATH)
        vp, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        h.palial_gpu_init.argtypes = [i]
        h.palial_gpu_factor_dev.argtypes = [i, vp, vp, i, i, ctypes.POINTER(Opts), ctypes.POINTER(Status), vp]
        h.palial_gpu_cholesky.argtypes = [ctypes.POINTER(Desc), ctypes.POINTER(Opts), ctypes.POINTER(Status)]
        h.palial_gpu_lu.argtypes = [ctypes.POINTER(Desc), vp, ctypes.POINTER(Opts), ctypes.POINTER(Status)]
        h.palial_gpu_qr.argtypes = [ctypes.POINTER(Desc), ctypes.POINTER(Desc), ctypes.POINTER(Opts),
                                    ctypes.POINTER(Status)]
        h.palial_gpu_gen_uniform.argtypes = [vp, i, i, ctypes.c_uint64, vp]
        h.palial_gpu_gen_spd.argtypes = [vp, i, i, ctypes.c_uint64, vp]
        h.palial_gpu_gen_dense.argtypes = [vp, ctypes.c_longlong, i, ctypes.c_uint64, i, vp]
        h.palial_gpu_residual_probe.argtypes = [i, vp, vp, vp, i, i, i, ctypes.c_uint64, ctypes.POINTER(d)]
        h.palial_gpu_trace_dump.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        h.palial_gpu_trace_count.restype = ctypes.c_longlong
        h.palial_dag_info.restype = ctypes.c_longlong
        h.palial_dag_info.argtypes = [i, i, i, i, i, i, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(d),
                                      ctypes.POINTER(d)]
        h.palial_dag_validate.argtypes = [i, i, i, i, i, i, ctypes.c_uint, ctypes.c_char_p, i]
        for name in ("palial_gpu_tile_dpotrf", "palial_gpu_tile_dgetrf"):
            getattr(h, name).argtypes = [i, vp, i]
        h.palial_gpu_tile_dtrsm.argtypes = [i, i, vp, vp, i]
        h.palial_gpu_tile_dsyrk.argtypes = [i, vp, vp, i]
        h.palial_gpu_tile_dgemm.argtypes = [i, i, vp, vp, vp, i]
        h.palial_gpu_tile_dgeqrt.argtypes = [i, vp, vp, i]
        h.palial_gpu_tile_dormqr.argtypes = [i, vp, vp, vp, i]
        h.palial_gpu_tile_dtsqrt.argtypes = [i, vp, vp, vp, i]
        h.palial_gpu_tile_dtsmqr.argtypes = [i, vp, vp, vp, vp, i]
        h.palial_gpu_tile_dtsmqr_noalloc.argtypes = [i, vp, vp, vp, vp, i, vp]
        h.palial_gpu_tile_sgeqrt.argtypes = [i, vp, vp, i]
        h.palial_gpu_tile_sormqr.argtypes = [i, vp, vp, vp, i]
        h.palial_gpu_tile_stsqrt.argtypes = [i, vp, vp, vp, i]
        h.palial_gpu_tile_stsmqr.argtypes = [i, vp, vp, vp, vp, i]
        h.palial_gpu_error_string.restype = ctypes.c_char_p
        h.palial_gpu_kernel_launches.restype = ctypes.c_longlong
        h.palial_gpu_solve_ir.argtypes = [i, vp, i, i, vp, vp, i, ctypes.POINTER(Opts), ctypes.POINTER(Status), vp]
        h.palial_gpu_mp_factor.argtypes = [i, vp, vp, i, i, ctypes.POINTER(Opts), ctypes.POINTER(Status), vp]
        h.palial_gpu_mp_update_step.argtypes = [i, i, vp, i, i, i]
        h.palial_gpu_gen_kappa.argtypes = [vp, i, i, d, i, ctypes.c_uint64, vp]
        h.palial_gpu_batched.argtypes = [i, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                         ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                         ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(Opts), ctypes.POINTER(Status),
                                         ctypes.POINTER(ctypes.c_double), vp]
        h.palial_gpu_gen_batch_matrix.argtypes = [vp, i, i, i, i, ctypes.c_uint64, vp]
        h.palial_dag_batch_validate.argtypes = [i, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                                ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), i,
                                                ctypes.c_uint, ctypes.c_char_p, i]
        h.palial_gpu_solve_ir_host.argtypes = [i, ctypes.POINTER(Desc), vp, vp, i, ctypes.POINTER(Opts),
                                               ctypes.POINTER(Status)]
        h.palial_gpu_qr_solve.argtypes = [i, i, i, vp, vp, vp, i, vp, ctypes.POINTER(Opts), ctypes.POINTER(Status),
                                          vp]
        h.palial_gpu_qr_solve_host.argtypes = [i, i, i, vp, vp, vp, i, vp, ctypes.POINTER(Opts),
                                               ctypes.POINTER(Status)]
        h.palial_dag_qr_solve_validate.restype = ctypes.c_longlong
        h.palial_dag_qr_solve_validate.argtypes = [i, i, i, i, i, ctypes.c_uint, ctypes.POINTER(ctypes.c_longlong),
                                                   ctypes.c_char_p, i]
        h.palial_dag_qr_apply_validate.restype = ctypes.c_longlong
        h.palial_dag_qr_apply_validate.argtypes = [i, i, i, i, ctypes.c_uint, ctypes.POINTER(ctypes.c_longlong),
                                                   ctypes.c_char_p, i]
        h.palial_gpu_qr_solve_ir.argtypes = [i, i, vp, vp, vp, i, ctypes.POINTER(Opts), ctypes.POINTER(Status), vp]
        h.palial_gpu_batch_sizes.argtypes = [i, ctypes.c_uint64, vp, vp]
        h.palial_gpu_batch_partition.argtypes = [i, vp, vp, i, vp]
        h.palial_gpu_batch_autotune.argtypes = [i, vp, vp, ctypes.c_uint64, i, vp, vp, ctypes.POINTER(Status)]
        h.palial_gpu_batch_synthetic.argtypes = [i, ctypes.c_uint64, i, i, i, vp, i, ctypes.POINTER(Opts),
                                                 ctypes.POINTER(Status), vp]
        h.palial_gpu_batched_f32.argtypes = [i, vp, vp, vp, vp, vp, vp, ctypes.POINTER(Opts), ctypes.POINTER(Status),
                                             vp, vp]
        h.palial_gpu_batched_solve.argtypes = [i, vp, vp, vp, vp, vp, vp, vp, ctypes.POINTER(Opts),
                                               ctypes.POINTER(Status), vp, vp, vp]
        h.palial_gpu_batch_solve_autotune.argtypes = [i, vp, vp, ctypes.c_uint64, i, vp, vp, vp,
                                                      ctypes.POINTER(Status)]
        h.palial_gpu_batch_solve_synthetic.argtypes = [i, ctypes.c_uint64, i, i, i, vp, vp, i, ctypes.POINTER(Opts),
                                                       ctypes.POINTER(Status), vp]
        h.palial_gpu_colmajor_to_tiles.argtypes = [vp, ctypes.c_longlong, i, vp, i, i, d, vp]
        h.palial_gpu_tiles_to_colmajor.argtypes = [vp, i, i, vp, ctypes.c_longlong, i, vp]
        h.palial_gpu_solve_colmajor.argtypes = [i, i, vp, ctypes.c_longlong, vp, ctypes.c_longlong, vp,
                                                ctypes.c_longlong, i, i, ctypes.POINTER(Opts), ctypes.POINTER(Status),
                                                vp]
        h.palial_tiles_write.argtypes = [ctypes.c_char_p, ctypes.POINTER(Desc)]
        h.palial_gpu_row_groups.argtypes = [i, i, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                            ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), i]
        h.palial_gpu_check_solve_tasks.argtypes = [i, i, i]
        h.palial_gpu_check_arrival_plan.argtypes = [i, i, i]
        h.palial_tiles_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                        vp]
        _lib = h
    return _lib


def make_opts(precision: str | int = "fp64", block: int = 0, workers_per_sm: int = 0, max_sms: int = 0,
              priority: int = 0, trace: bool = False, timeout_s: float = 0.0, shuffle_seed: int = 0,
              ir_max_iter: int = 0, ir_tol: float = 0.0, gmres: int = 0) -> Opts:
    o = Opts()
    o.precision = PREC[precision] if isinstance(precision, str) else int(precision)
    o.block, o.workers_per_sm, o.max_sms, o.priority = block, workers_per_sm, max_sms, priority
    o.trace, o.timeout_s, o.shuffle_seed = int(trace), timeout_s, shuffle_seed
    o.ir_max_iter, o.ir_tol, o.gmres = ir_max_iter, ir_tol, gmres
    return o


def _check(rc: int, st: Status | None, allow=(PALIAL_OK,)) -> None:
    if rc not in allow:
        raise PalialError(rc, st.message.decode(errors="replace") if st is not None else "")


def init(device: int = 0) -> None:
    _check(lib().palial_gpu_init(device), None)


def desc(buf: np.ndarray, n: int, nb: int) -> Desc:
    assert buf.dtype == np.float64 and buf.flags["C_CONTIGUOUS"] and buf.size == n * n
    return Desc(nb, n * n, nb * nb, n, buf.ctypes.data)


# ---- reference entry points (host buffers, in place) ------------------------------------
def cholesky(a_tiles: np.ndarray, n: int, nb: int, **kw) -> Status:
    """Upper tile Cholesky A = U^T U in place (reference src/cholesky.h:12)."""
    st = Status()
    rc = lib().palial_gpu_cholesky(ctypes.byref(desc(a_tiles, n, nb)), ctypes.byref(make_opts(**kw)),
                                   ctypes.byref(st))
    _check(rc, st)
    return st


def lu(a_tiles: np.ndarray, n: int, nb: int, **kw) -> tuple[Status, np.ndarray]:
    """No-pivot tile LU in place (reference src/lu.h:11); returns (status, ipiv = 1..N)."""
    st = Status()
    ipiv = np.zeros(n, dtype=np.int32)
    rc = lib().palial_gpu_lu(ctypes.byref(desc(a_tiles, n, nb)), ipiv.ctypes.data, ctypes.byref(make_opts(**kw)),
                             ctypes.byref(st))
    _check(rc, st, allow=(PALIAL_OK, 1))
    return st, ipiv


def qr(a_tiles: np.ndarray, s_tiles: np.ndarray, n: int, nb: int, **kw) -> Status:
    """Flat-tree TS tile QR in place (reference src/qr.h:15); T factors go to S."""
    st = Status()
    rc = lib().palial_gpu_qr(ctypes.byref(desc(a_tiles, n, nb)), ctypes.byref(desc(s_tiles, n, nb)),
                             ctypes.byref(make_opts(**kw)), ctypes.byref(st))
    _check(rc, st)
    return st


def factor_dev(alg: str, d_a: int, d_s: int | None, n: int, nb: int, stream: int = 0, allow_warn: bool = True,
               **kw) -> Status:
    """Factor a DEVICE-resident tile matrix (pointer from e.g. torch's data_ptr())."""
    st = Status()
    rc = lib().palial_gpu_factor_dev(ALG[alg], d_a, d_s or None, n, nb, ctypes.byref(make_opts(**kw)),
                                     ctypes.byref(st), stream or None)
    _check(rc, st, allow=(PALIAL_OK, 1) if allow_warn else (PALIAL_OK,))
    return st


def solve_ir(alg: str, d_a: int, n: int, nb: int, d_b: int, d_x: int, nrhs: int, stream: int = 0,
             raise_on_error: bool = True, **kw) -> Status:
    """Mixed-precision (or FP64) factorization + iterative refinement: A X = B on the device."""
    st = Status()
    rc = lib().palial_gpu_solve_ir(ALG[alg], d_a, n, nb, d_b, d_x, nrhs, ctypes.byref(make_opts(**kw)),
                                   ctypes.byref(st), stream or None)
    if raise_on_error:
        _check(rc, st, allow=(PALIAL_OK, 1))
    st.code = rc
    return st


def solve_ir_host(alg: str, a_tiles: np.ndarray, n: int, nb: int, b: np.ndarray, x: np.ndarray, nrhs: int,
                  raise_on_error: bool = True, **kw) -> Status:
    """Host-buffer solve: a_tiles (tile layout), b and x (n x nrhs, column-major float64)."""
    st = Status()
    rc = lib().palial_gpu_solve_ir_host(ALG[alg], ctypes.byref(desc(a_tiles, n, nb)), b.ctypes.data, x.ctypes.data,
                                        nrhs, ctypes.byref(make_opts(**kw)), ctypes.byref(st))
    if raise_on_error:
        _check(rc, st, allow=(PALIAL_OK, 1))
    st.code = rc
    return st


def qr_solve(d_a: int, rows: int, cols: int, nb: int, d_b: int, d_x: int, nrhs: int, d_resid: int | None = None,
             stream: int = 0, **kw) -> Status:
    """A X = B (rows == cols) or least squares min ||A X - B||_2 (rows > cols) through the tile
    QR, on device buffers: A tile layout (rows x cols), B rows x nrhs and X cols x nrhs
    column-major, d_resid (optional) nrhs residual 2-norms."""
    st = Status()
    rc = lib().palial_gpu_qr_solve(rows, cols, nb, d_a, d_b, d_x, nrhs, d_resid or None,
                                   ctypes.byref(make_opts(**kw)), ctypes.byref(st), stream or None)
    _check(rc, st)
    return st


def qr_solve_host(a_tiles: np.ndarray, rows: int, cols: int, nb: int, b: np.ndarray, **kw):
    """Host-buffer QR solve: returns (X cols x nrhs, residual norms, status)."""
    b = np.asfortranarray(b.reshape(rows, -1), dtype=np.float64)
    nrhs = b.shape[1]
    x = np.zeros((cols, nrhs), dtype=np.float64, order="F")
    resid = np.zeros(nrhs)
    st = Status()
    rc = lib().palial_gpu_qr_solve_host(rows, cols, nb, np.ascontiguousarray(a_tiles).ctypes.data, b.ctypes.data,
                                        x.ctypes.data, nrhs, resid.ctypes.data, ctypes.byref(make_opts(**kw)),
                                        ctypes.byref(st))
    _check(rc, st)
    return x, resid, st


def tiles_write(path: str, a_tiles: np.ndarray, n: int, nb: int) -> None:
    """Write a tile-layout matrix in the library's tiled-matrix file format."""
    a = np.ascontiguousarray(a_tiles, dtype=np.float64)
    _check(lib().palial_tiles_write(path.encode(), ctypes.byref(desc(a, n, nb))), None)


def tiles_read(path: str) -> tuple[np.ndarray, int, int]:
    """Read a tiled-matrix file: (tile-layout buffer, n, nb)."""
    n, nb = ctypes.c_int(), ctypes.c_int()
    _check(lib().palial_tiles_read(path.encode(), ctypes.byref(n), ctypes.byref(nb), None), None)
    out = np.empty(n.value * n.value, dtype=np.float64)
    _check(lib().palial_tiles_read(path.encode(), ctypes.byref(n), ctypes.byref(nb), out.ctypes.data), None)
    return out, n.value, nb.value


def solve_colmajor(alg: str, n: int, d_a: int, lda: int, d_b: int, ldb: int, d_x: int, ldx: int, nrhs: int,
                   nb: int = 512, stream: int = 0, raise_on_error: bool = True, **kw) -> Status:
    """A X = B for a column-major device A of any n (padded to a multiple of nb internally)."""
    st = Status()
    rc = lib().palial_gpu_solve_colmajor(ALG[alg], n, d_a, lda, d_b, ldb, d_x, ldx, nrhs, nb,
                                         ctypes.byref(make_opts(**kw)), ctypes.byref(st), stream or None)
    if raise_on_error:
        _check(rc, st, allow=(PALIAL_OK, 1))
    st.code = rc
    return st


def qr_solve_dag(rows: int, cols: int, nb: int, nrhs: int, nworkers: int = 152, seed: int = 0) -> dict:
    """Host only: build and validate the QR solve DAG; records and logical task counts per type."""
    counts = (ctypes.c_longlong * 16)()
    msg = ctypes.create_string_buffer(256)
    nrec = lib().palial_dag_qr_solve_validate(rows, cols, nb, nrhs, nworkers, seed, counts, msg, 256)
    return {"records": nrec, "type_counts": list(counts), "message": msg.value.decode()}


def qr_apply_dag(n: int, nb: int, nrhs: int, nworkers: int = 152, seed: int = 0) -> dict:
    """Host only: build and validate the apply-only QR solve DAG of the mixed-precision QR
    refinement (Q^T and R^-1 on the extra tile column); records and logical task counts."""
    counts = (ctypes.c_longlong * 16)()
    msg = ctypes.create_string_buffer(256)
    nrec = lib().palial_dag_qr_apply_validate(n, nb, nrhs, nworkers, seed, counts, msg, 256)
    return {"records": nrec, "type_counts": list(counts), "message": msg.value.decode()}


def qr_solve_ir(d_a: int, n: int, nb: int, d_b: int, d_x: int, nrhs: int, stream: int = 0,
                allow_not_converged: bool = False, **kw) -> Status:
    """Mixed-precision QR solve of a square A X = B on device buffers (A tile layout, B and X
    n x nrhs column-major): FP32 tile QR + FP64 refinement, the FP64 QR solve when the
    refinement stalls.  status.precision_used = the precision that produced X (5 FP32, 0 FP64)."""
    st = Status()
    rc = lib().palial_gpu_qr_solve_ir(n, nb, d_a, d_b, d_x, nrhs, ctypes.byref(make_opts(**kw)), ctypes.byref(st),
                                      stream or None)
    _check(rc, st, allow=(PALIAL_OK, -6) if allow_not_converged else (PALIAL_OK,))
    st.code = rc
    return st


def mp_factor(alg: str, d_a: int, d_w: int, n: int, nb: int, stream: int = 0, **kw) -> Status:
    st = Status()
    rc = lib().palial_gpu_mp_factor(ALG[alg], d_a, d_w, n, nb, ctypes.byref(make_opts(**kw)), ctypes.byref(st),
                                    stream or None)
    _check(rc, st, allow=(PALIAL_OK, 1))
    return st


def gen_kappa(d_a: int, n: int, nb: int, kappa: float, symmetric: bool, seed: int = 0, stream: int = 0) -> None:
    _check(lib().palial_gpu_gen_kappa(d_a, n, nb, float(kappa), int(symmetric), seed, stream or None), None)


def gen_uniform(d_a: int, n: int, nb: int, seed: int, stream: int = 0) -> None:
    _check(lib().palial_gpu_gen_uniform(d_a, n, nb, seed, stream or None), None)


STREAM_RHS = 2  # generator stream of right-hand sides


def gen_dense(d_x: int, rows: int, cols: int, seed: int, stream_id: int = STREAM_RHS, stream: int = 0) -> None:
    """Dense column-major rows x cols uniform [-1, 1) block on the device (the generator the
    right-hand sides of the benchmarks use)."""
    _check(lib().palial_gpu_gen_dense(d_x, rows, cols, seed, stream_id, stream or None), None)


def gen_spd(d_a: int, n: int, nb: int, seed: int, stream: int = 0) -> None:
    _check(lib().palial_gpu_gen_spd(d_a, n, nb, seed, stream or None), None)


def residual_probe(alg: str, d_a0: int, d_f: int, n: int, nb: int, nprobe: int = 8, seed: int = 7,
                   d_s: int | None = None) -> float:
    out = ctypes.c_double()
    _check(lib().palial_gpu_residual_probe(ALG[alg], d_a0, d_f, d_s or None, n, nb, nprobe, seed,
                                           ctypes.byref(out)), None)
    return out.value


def trace_dump(path: str | None = None, csv_path: str | None = None) -> None:
    _check(lib().palial_gpu_trace_dump(path.encode() if path else None, csv_path.encode() if csv_path else None), None)


def dag_info(alg: str, n: int, nb: int, block: int = 0, priority: int = 0, nworkers: int = 152) -> dict:
    counts = (ctypes.c_longlong * 16)()
    cp, ms = ctypes.c_double(), ctypes.c_double()
    nrec = lib().palial_dag_info(ALG[alg], n, nb, block, priority, nworkers, counts, ctypes.byref(cp),
                                 ctypes.byref(ms))
    if nrec < 0:
        raise PalialError(-1, "invalid DAG parameters")
    return {"records": nrec, "type_counts": list(counts), "critical_path_s": cp.value, "makespan_s": ms.value}


def dag_validate(alg: str, n: int, nb: int, block: int = 0, priority: int = 0, nworkers: int = 152,
                 seed: int = 1) -> str:
    buf = ctypes.create_string_buffer(256)
    rc = lib().palial_dag_validate(ALG[alg], n, nb, block, priority, nworkers, seed, buf, 256)
    return "" if rc == 0 else (buf.value.decode() or f"rc={rc}")


def row_groups(n: int, nb: int) -> list[tuple[int, int, int, int]]:
    """The tile-row groups (first row, end row, due step, join step) in which the host-buffer
    mixed-precision Cholesky sends the upper triangle (host logic, no GPU)."""
    arrs = [(ctypes.c_int * 64)() for _ in range(4)]
    ng = lib().palial_gpu_row_groups(n, nb, *arrs, 64)
    _check(0 if ng > 0 else ng, None)
    return [(arrs[0][g], arrs[1][g], arrs[2][g], arrs[3][g]) for g in range(ng)]


def check_solve_tasks(mt: int, nbl: int, kind: int) -> int:
    """0 when the refinement's triangular-solve task list is deadlock-free (host logic)."""
    return lib().palial_gpu_check_solve_tasks(mt, nbl, kind)


def check_arrival_plan(n: int, nb: int, mode: int) -> int:
    """0 when the host-buffer Cholesky's catch-up plan is consistent (host logic)."""
    return lib().palial_gpu_check_arrival_plan(n, nb, mode)
