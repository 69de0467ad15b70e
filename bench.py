"""Benchmark: tiled Cholesky at N = 32768, NB = 512 on one GB300 (per GPU).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--suite fp64|kappa|batched|batched_solve|costmodel|kernels|qr_mixed]

A step is one solve A X = B (16 right-hand sides, uniform [-1, 1)) of a device-resident
SPD matrix A = B B^T + N I (seed = rank; the reference's tile layout) by the mixed-precision
path: BF16x3 trailing updates on tcgen05 (operands split into BF16 hi + lo, three products,
FP32 accumulation; --precision bf16 / fp8 select one product), FP32 diagonal tiles and
panels (BF16x3 block products), the exact-digit tensor-core residual (48-bit digit expansions,
integer accumulation; once the correction is small, the update form r - A d with FP32
products) and refinement to the FP64-level normwise
backward error (<= 1e-14 * N), checked after the timed region with the FP64 residual.  value = FP64-equivalent algorithmic flops (N^3/3) / time to solution
(factorization + refinement), summed over ranks (replicas, no collective on the data path).
Inputs (8.6 GB) are far larger than L2 (129 MB): no flush is needed.

The JSON line also carries:
  fp64_tiled    the plain FP64 tiled factorization (persistent scheduler, FP64 DFMA) of the
                same matrix: its TFLOP/s and the mixed/FP64 speed-up;
  e2e           the same solve through the host-buffer C ABI (palial_gpu_solve_ir_host on
                pinned host memory: A's upper triangle (what Cholesky reads) and B copied in,
                X copied out, every step);
  e2e_pageable  the same from a pageable (malloc'd) host buffer, as the reference's caller has;
  kappa         config 3 at N = 32768: Cholesky at kappa = 1e6 and 1e10, LU at 1e6: the
                precision ladder's solve (rung used, refinement and GMRES steps, FP64-checked
                backward error, forward error against the FP64 solve) beside the FP64
                factorization's solve;
  lu, qr        no-pivot LU (kappa = 1e2 matrix) and QR (uniform [-1, 1), seed 1) at N = 32768:
                mixed-precision solve time beside the FP64 solve (--no-extra skips these three);
  roofline      the tcgen05 trailing-update kernel (the mixed path's tensor-core kernel),
                timed live on the largest step (k = 0); bound chosen by its arithmetic
                intensity against the measured ridge (BF16x3: tensor), achieved / measured
                peak from MEASURED_PEAKS.json, the HBM rate beside it;
  cpu_baseline  the oracle's OpenMP port of the reference's Cholesky (same task DAG, same
                OpenBLAS calls) on this host's cores, on a bounded sample (N = 16384);
  clocks        nvidia-smi samples taken during the timed region.
`--impl reference` times the reference's CPU implementation (the oracle port, OpenMP, all
host cores) on the same metric, one bounded sample (N = 16384) per step.
`--suite fp64` prints one line per FP64 factorization of configs N in {16384, 32768} for
Cholesky, LU and QR; `--suite kappa` one line per kappa in {1e2, 1e6, 1e10}, algorithm and
precision at N = 32768 (A = U diag(s) V^T, 64 Householder reflectors each side);
`--suite kernels [--n N]` times the dominant kernels alone (the small case ncu captures run).
`--suite batched` factors the uneven batch (2000 matrices, N log-uniform in [32, 2048)) in one
FP64 launch, then times batched solves of it: FP64 factorizations vs block size and precision
(FP32 + FP64 refinement, or FP64) autotuned per algorithm and size class; `--suite
batched_solve` runs the solves alone (FP64 with the FP64 autotuner's measured block sizes).
`--suite qr_mixed` times the mixed-precision QR solve beside the FP64 QR solve (N = 16384, 32768).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N, NB = 32768, 512
CPU_N = 16384
# block per size class that the FP64 batched autotuner picks on the synthetic batch (measured)
FP64_BATCH_BLOCKS = (64, 128, 64, 64, 64, 64)
METRIC = "TFLOP/s Cholesky/LU/QR N=32768: mixed-prec+IR vs FP64 tiled, both at FP64 acc"


def flops(n: int) -> float:
    return n ** 3 / 3.0


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        rows = []
        if self.path and os.path.exists(self.path):
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9:
                    rows.append(f)
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for name, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def fp64_peak_tflops(torch) -> float:
    """cuBLAS DGEMM 8192^3, best of 3 (CUDA events): the FP64 denominator of the roofline."""
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    c = a @ b
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        c = a @ b
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) * 1e-3)
    del a, b, c
    torch.cuda.empty_cache()
    return 2.0 * n ** 3 / best * 1e-12


def cpu_baseline_sample(nthreads: int, seed: int = 0, spd_host=None) -> tuple[float, float]:
    """Oracle OpenMP port (reference task DAG over OpenBLAS) on one N = CPU_N Cholesky."""
    import numpy as np  # first: numpy's own BLAS keeps every host thread for the generator
    from oracle import oracle as O

    a = spd_host if spd_host is not None else O.to_tiles(O.gen_spd(seed, CPU_N), NB)
    t = np.array(a, copy=True)
    sec = O.run("cholesky", t, CPU_N, NB, nthreads=nthreads)
    return flops(CPU_N) / sec * 1e-12, sec


def spd_host_from_gpu(P, torch, n: int, seed: int):
    """The SPD input generated on the GPU (identical bytes to the CPU generator)."""
    d = torch.empty(n * n, dtype=torch.float64, device="cuda")
    P.gen_spd(d.data_ptr(), n, NB, seed)
    h = d.cpu().numpy().copy()
    del d
    torch.cuda.empty_cache()
    return h


def headline_config(n: int, precision: str, world: int) -> dict:
    """The workload both arms report on (the reference arm times a bounded sample of it)."""
    return {"workload": f"mixed-precision Cholesky + IR, N={n}, NB={NB}, 16 RHS, {precision} "
                        "trailing updates on tcgen05 (FP32 accumulate), FP32 diagonal tiles, FP32 "
                        "panels with BF16x3 block products, exact-digit tensor-core and update-form "
                        "refinement residuals, FP64-checked backward error; SPD B*B^T+N*I seed=rank, "
                        "device-resident; inputs 8.6 GB >> L2 (no flush needed)",
            "n": n, "nb": NB, "nrhs": 16, "precision": precision, "parallelism": f"replicas x{world}"}


def run_reference(args, rank: int, world: int) -> None:
    """The reference's CPU implementation of the path (the oracle's OpenMP restatement of
    src/cholesky.h over OpenBLAS, bit-identical to the reference's own build) on every host
    core.  Input generated on the host by the oracle's generator; nothing of the GPU library is
    loaded.  Each step is one FP64 Cholesky at N = CPU_N (about 2.4 s on 16 Arm cores): a
    bounded sample of the N = 32768 workload, whose 8x larger run (about 20 s a step) would
    hold the whole --steps/--warmup run for many minutes."""
    if rank != 0:
        return
    nthreads = os.cpu_count() or 1
    import numpy as np  # noqa: F401  (before the oracle: numpy's BLAS keeps all host threads)
    from oracle import oracle as O

    spd = O.to_tiles(O.gen_spd(0, CPU_N), NB)
    times = []
    for i in range(args.warmup + args.steps):
        _, sec = cpu_baseline_sample(nthreads, spd_host=spd)
        if i >= args.warmup:
            times.append(sec)
    sec = sum(times) / len(times)
    value = flops(CPU_N) / sec * 1e-12
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": headline_config(N, args.precision, world),
        "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": nthreads, "kind": "port",
                         "sample": f"one FP64 Cholesky N={CPU_N} NB={NB} per step (bounded sample of the N={N} "
                                   "workload, same SPD generator, seed 0): the oracle's OpenMP restatement of "
                                   "reference src/cholesky.h over OpenBLAS, OMP_NUM_THREADS=all cores, "
                                   "OPENBLAS_NUM_THREADS=1; input generated on the host"},
        "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "native_libraries": in_tree_libraries(),
    }
    print(json.dumps(line), flush=True)


def in_tree_libraries() -> list[str]:
    """Shared objects of this repository mapped into the process (Linux /proc/self/maps)."""
    found = set()
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                path = line.split()[-1] if len(line.split()) >= 6 else ""
                if path.endswith(".so") and path.startswith(ROOT):
                    found.add(os.path.relpath(path, ROOT))
    except OSError:
        pass
    return sorted(found)


def fp64_backward_error(P, torch, a0, n: int, nb: int, x, b, nrhs: int) -> float:
    """max_j ||b_j - A x_j||_inf / (||A||_inf ||x_j||_inf + ||b_j||_inf) with the library's FP64
    residual (outside the timed region), for the solution the last timed step returned."""
    import ctypes
    lib = P.lib()
    lib.palial_gpu_residual.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    r = torch.empty_like(x)
    if lib.palial_gpu_residual(a0.data_ptr(), n, nb, x.data_ptr(), b.data_ptr(), r.data_ptr(), nrhs, 0, None):
        return float("nan")
    mt = n // nb
    anorm = float(a0.view(mt, mt, nb, nb).abs().sum(dim=(0, 2)).transpose(0, 1).reshape(n).max()) \
        if n <= 16384 else float(_rowsum_max(torch, a0, n, nb))
    rv, xv, bv = r.view(nrhs, n), x.view(nrhs, n), b.view(nrhs, n)
    eta = (rv.abs().amax(dim=1) / (anorm * xv.abs().amax(dim=1) + bv.abs().amax(dim=1))).max()
    return float(eta)


def _rowsum_max(torch, a0, n: int, nb: int):
    """||A||_inf of a tile-layout matrix, one tile column at a time (bounded extra memory)."""
    mt = n // nb
    t = a0.view(mt, mt, nb, nb)  # [tile col][tile row][col][row]
    rows = torch.zeros(mt, nb, dtype=torch.float64, device=a0.device)
    for tc in range(mt):
        rows += t[tc].abs().sum(dim=1)
    return rows.max()


def peaks() -> dict:
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def time_update_kernel(P, torch, n: int, precision: str = "bf16") -> dict:
    """Live CUDA-event timing of one tcgen05 trailing update (step k = 0, the bench's update
    precision) on an FP32 tile matrix, pack included: tensor flops and algorithmic bytes per
    launch (C read + write in FP32, panel read once in FP32, packed operands written and read)."""
    code = {"bf16": 1, "fp8": 2, "bf16x3": 3, "tf32x3": 6}.get(precision, 1)
    w = torch.randn(n * n, dtype=torch.float32, device="cuda")
    for _ in range(2):
        P.lib().palial_gpu_mp_update_step(0, code, w.data_ptr(), n, NB, 0)
    ts = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        P.lib().palial_gpu_mp_update_step(0, code, w.data_ptr(), n, NB, 0)
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1) * 1e-3)
    del w
    torch.cuda.empty_cache()
    r = n // NB - 1
    pairs = r * (r + 1) // 2
    products = 3 if code in (3, 6) else 1
    packed = {1: 2.0, 2: 1.0, 3: 4.0, 6: 8.0}[code]  # bytes per element of the packed panel(s)
    flop = pairs * 2.0 * NB ** 3 * products
    byts = pairs * NB * NB * 8.0 + r * NB * NB * (4.0 + 2.0 * packed)
    t = min(ts)
    return {"seconds": t, "flop": flop, "bytes": byts, "products": products}


def _solve(P, torch, alg: str, da, n: int, b, nrhs: int, precision: str, stream: int):
    x = torch.zeros_like(b)
    st = P.solve_ir(alg, da.data_ptr(), n, NB, b.data_ptr(), x.data_ptr(), nrhs, precision=precision,
                    ir_max_iter=30, stream=stream, raise_on_error=False)
    torch.cuda.synchronize()
    return st, x


def _fwd(torch, x, xref, nrhs: int) -> float:
    """max_j ||x_j - xref_j||_inf / ||xref_j||_inf."""
    xv, rv = x.view(nrhs, -1), xref.view(nrhs, -1)
    return float(((xv - rv).abs().amax(dim=1) / rv.abs().amax(dim=1)).max())


def config_keys(P, torch, n: int, b, nrhs: int, stream: int) -> dict:
    """One run each of the metric's other configurations at N = n (untimed by the step loop;
    each call's own wall time): config 3's kappa = 1e6 matrices (A = U diag(s) V^T, s geometric
    from 1 to 1/kappa, 64 Householder reflectors each side; U = V for Cholesky) solved by the
    precision ladder (AUTO) and by the FP64 factorization + FP64 refinement, with the backward
    error recomputed by the FP64 residual and the forward error of the ladder's X against the
    FP64 solve's; no-pivot LU at kappa = 1e2 (ladder vs FP64); the QR solve of the uniform
    [-1, 1) matrix (seed 1) by the FP32 tile QR (TSMQR's products with V as BF16x3 on the warp
    tensor cores) + FP64 refinement vs the FP64 QR solve."""
    out = {}
    da = torch.empty(n * n, dtype=torch.float64, device="cuda")
    flop = {"cholesky": n ** 3 / 3.0, "lu": 2.0 * n ** 3 / 3.0, "qr": 4.0 * n ** 3 / 3.0}

    def ladder_vs_fp64(alg: str, kappa: float) -> dict:
        P.gen_kappa(da.data_ptr(), n, NB, kappa, alg == "cholesky", seed=7)
        st, x = _solve(P, torch, alg, da, n, b, nrhs, "auto", stream)
        eta = fp64_backward_error(P, torch, da, n, NB, x, b, nrhs)
        st64, x64 = _solve(P, torch, alg, da, n, b, nrhs, "fp64", stream)
        rec = {"kappa": kappa, "converged": st.code in (0, 1), "precision_used": P.PREC_NAME.get(st.precision_used),
               "seconds": st.seconds, "tflops_fp64_equiv": flop[alg] / st.seconds * 1e-12,
               "ir_iters": st.ir_iters, "gmres_iters": st.gmres_iters, "backward_error_fp64_check": eta,
               "forward_error_vs_fp64_solve": _fwd(torch, x, x64, nrhs),
               "fp64_solve": {"seconds": st64.seconds, "tflops": flop[alg] / st64.seconds * 1e-12,
                              "converged": st64.code in (0, 1), "backward_error": st64.backward_error},
               "speedup_over_fp64": st64.seconds / st.seconds}
        del x, x64
        return rec

    out["kappa"] = {"n": n, "nb": NB, "nrhs": nrhs,
                    "cholesky": {"1e6": ladder_vs_fp64("cholesky", 1e6), "1e10": ladder_vs_fp64("cholesky", 1e10)},
                    "lu": {"1e6": ladder_vs_fp64("lu", 1e6)},
                    "note": "AUTO ladder BF16x3 -> TF32x3 -> FP64; the forward error a backward error eta "
                            "allows is about kappa * eta (target eta <= 1e-14 * N)"}
    out["lu"] = dict(ladder_vs_fp64("lu", 1e2), n=n, nb=NB, nrhs=nrhs, matrix="U diag(s) V^T, kappa 1e2")
    P.gen_uniform(da.data_ptr(), n, NB, 1)
    x = torch.zeros_like(b)
    st = P.qr_solve_ir(da.data_ptr(), n, NB, b.data_ptr(), x.data_ptr(), nrhs, allow_not_converged=True,
                       precision="bf16x3")
    eta = fp64_backward_error(P, torch, da, n, NB, x, b, nrhs)
    x64 = torch.zeros_like(b)
    s64 = P.qr_solve(da.data_ptr(), n, n, NB, b.data_ptr(), x64.data_ptr(), nrhs)
    out["qr"] = {"n": n, "nb": NB, "nrhs": nrhs, "matrix": "uniform [-1, 1), seed 1",
                 "converged": st.code == 0, "precision_used": P.PREC_NAME.get(st.precision_used),
                 "seconds": st.seconds, "factor_seconds": st.factor_seconds,
                 "tflops_fp64_equiv": flop["qr"] / st.seconds * 1e-12, "ir_iters": st.ir_iters,
                 "backward_error_fp64_check": eta, "forward_error_vs_fp64_solve": _fwd(torch, x, x64, nrhs),
                 "fp64_solve": {"seconds": s64.seconds, "tflops": flop["qr"] / s64.seconds * 1e-12},
                 "speedup_over_fp64": s64.seconds / st.seconds}
    del da, x, x64
    torch.cuda.empty_cache()
    return out


def run_batched(args, P, torch, rank: int = 0, world: int = 1) -> None:
    """The batched workload: 2000 matrices, N log-uniform in [32, 2048) (seed 2), half SPD Cholesky, half
    uniform LU, FP64, one persistent launch replayed from a CUDA graph; block size per size
    class chosen by the autotuner.  With N > 1 ranks every rank factors its share of a
    size-balanced partition (no collective on the data path; total work fixed: strong
    scaling); the batch time is the max over ranks."""
    from palial_gb300 import batched as B
    rep = B.synthetic(args.batch, seed=2, rank=rank, world=world, autotune=True, reps=max(3, args.steps))
    t = rep["seconds"]
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([t], dtype=torch.float64, device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t = float(tt.item())
    if rank != 0:
        return
    ns, algs = B.batch_sizes(args.batch, 2)
    total_flops = float(sum(n ** 3 / 3.0 if a == 0 else 2.0 * n ** 3 / 3.0 for n, a in zip(ns, algs)))
    per_class = {}
    for c in range(6):
        if rep["count_of_class"][c]:
            per_class[B.class_label(c)] = {"count": rep["count_of_class"][c], "block": rep["bs_of_class"][c],
                                           "p50_ms": rep["p50_ms"][c], "p99_ms": rep["p99_ms"][c]}
    print(json.dumps({"suite": "batched", "matrices": int(len(ns)), "precision": "fp64", "n_gpus": world,
                      "scaling": "strong", "matrices_per_s": len(ns) / t, "batch_seconds": t,
                      "tflops": total_flops / t * 1e-12, "launches_per_batch_per_rank": 1, "cuda_graph": True,
                      "autotune_seconds": rep["autotune_seconds"],
                      "autotune": {f"{B.class_label(c)} bs={bs}": rep["autotune_s"][c * 3 + j]
                                   for c in range(6) for j, bs in enumerate(B.CANDIDATE_BS)
                                   if rep["autotune_s"][c * 3 + j] >= 0},
                      "per_size_class_rank0": per_class}), flush=True)
    run_batched_solve(args, rep["bs_of_class"], len(ns), world)


def run_batched_solve(args, bs_fp64, count: int, world: int) -> None:
    """Batched solves of the same synthetic batch (one right-hand side per matrix, uniform
    [-1, 1)) to FP64-level backward error (1e-14 * N): (a) every matrix factored in FP64 with the
    FP64 autotuner's block sizes, one FP64 refinement check; (b) block size and precision per
    (algorithm, size class) from the solve autotuner: FP32 factorizations in one persistent
    launch + FP64 refinement, FP64 where FP32 does not pay or does not converge; an LU matrix
    whose FP32 attempt fails gets a second FP32 attempt on its random-butterfly transform, and
    any matrix still failing an FP64 fallback.  Both timed as whole calls (copies,
    factorizations, refinement loop).  Rank 0's share when run under torchrun."""
    from palial_gb300 import batched as B
    reps = max(3, args.steps)
    fp64 = B.solve_synthetic(args.batch, seed=2, rank=0, world=world, autotune=False,
                             bs12=list(bs_fp64) * 2, prec12=[0] * 12, reps=reps)
    mixed = B.solve_synthetic(args.batch, seed=2, rank=0, world=world, autotune=True, reps=reps)
    prec_name = {0: "fp64", 1: "fp32+ir", 2: "bf16x3-update+ir"}
    phases = ("factor", "refine", "fp64_fallback")
    choice = {f"{('cholesky', 'lu')[k // 6]} {B.class_label(k % 6)}":
              {"block": mixed["bs_of_class"][k], "precision": prec_name[mixed["prec_of_class"][k]]}
              for k in range(12)}
    print(json.dumps({"suite": "batched_solve", "matrices": count, "n_gpus": world, "rank0_matrices": mixed["count"],
                      "fp64": {"seconds": fp64["seconds"], "matrices_per_s": fp64["matrices_per_s"],
                               "tflops": fp64["tflops"], "max_backward_error": fp64["max_backward_error"],
                               "converged": fp64["rc"] == 0, "phases_s": dict(zip(phases, fp64["phase_seconds"]))},
                      "mixed": {"seconds": mixed["seconds"], "matrices_per_s": mixed["matrices_per_s"],
                                "tflops": mixed["tflops"], "max_backward_error": mixed["max_backward_error"],
                                "max_refinement_steps": mixed["max_iters"], "fp64_fallbacks": mixed["fallbacks"],
                                "butterfly_solves": mixed["butterflies"],
                                "converged": mixed["rc"] == 0, "autotune_seconds": mixed["autotune_seconds"],
                                "phases_s": dict(zip(phases, mixed["phase_seconds"])), "choice": choice},
                      "speedup_mixed_vs_fp64": fp64["seconds"] / mixed["seconds"]}), flush=True)


def run_costmodel(args, P, torch) -> None:
    """The learned cost model: train the task-cost MLP on device traces of FP64 Cholesky / LU / QR
    sweeps (sweep_plan), report its per-task and per-run (makespan) prediction error on held-out
    runs, then plan FP64 Cholesky at N = 49152: (a) the learned plan -- (NB, block) with the
    smallest makespan predicted under the learned costs among plan_space, run with the learned
    critical-path priorities; (b) the fallback -- the exhaustive autotuner over NB (default
    block) timed at N = 49152 itself, static flop-model priorities.  Both makespans, the time
    each method spent choosing, and whether the learned-priority factors equal the static ones
    bit for bit (same plan, both orders)."""
    import numpy as np
    from palial_gb300.costmodel import COST_NBS, CostModel, exhaustive_nb, learned_run, plan_space, sweep_plan, trace_records
    runs = [(alg, n, nb, bs) for alg in ("cholesky", "lu", "qr") for (n, nb, bs) in sweep_plan(alg)]
    rng = np.random.default_rng(0)
    xs, ys, tags, measured = [], [], [], []
    t0 = time.perf_counter()
    for alg, n, nb, bs in runs:
        x, y, sec = trace_records(torch, alg, n, nb, bs, with_time=True)
        if len(y) > 60000:  # bound the host memory of the largest runs
            keep = np.sort(rng.choice(len(y), 60000, replace=False))
            x, y = x[keep], y[keep]
        xs.append(x)
        ys.append(y)
        tags.append(np.full(len(y), len(tags)))
        measured.append(sec)
    trace_s = time.perf_counter() - t0
    X, Y, T = np.concatenate(xs), np.concatenate(ys), np.concatenate(tags)
    held = sorted(rng.choice(len(runs), 4, replace=False).tolist())   # whole runs held out
    test = np.isin(T, held)
    train_idx = np.flatnonzero(~test)
    if len(train_idx) > 400000:
        train_idx = rng.choice(train_idx, 400000, replace=False)
    m = CostModel(seed=0)
    t1 = time.perf_counter()
    loss = m.fit(X[train_idx], Y[train_idx], epochs=40, batch=1024, lr=2e-3)
    train_s = time.perf_counter() - t1
    rel = np.abs(np.exp(m.predict_log_us(X[test]) - Y[test]) - 1.0)
    workers = P.lib().palial_gpu_sm_count()
    held_runs = []
    for i in held:
        alg, n, nb, bs = runs[i]
        pred = m.predicted_makespan(["cholesky", "lu", "qr"].index(alg), n, nb, bs, workers)
        held_runs.append({"alg": alg, "n": n, "nb": nb, "block": bs, "measured_s": measured[i], "predicted_s": pred,
                          "rel_error": abs(pred / measured[i] - 1.0)})
    # planning at the target size
    nbig = args.costmodel_n
    t2 = time.perf_counter()
    preds = {(nb, bs): m.predicted_makespan(0, nbig, nb, bs, workers) for nb, bs in plan_space(nbig)}
    plan = min(preds, key=preds.get)
    plan_s = time.perf_counter() - t2
    fb_nb, fb_times, fb_sums, fb_search_s = exhaustive_nb(torch, "cholesky", nbig, COST_NBS)
    learned_s, learned_sum = learned_run(torch, m, "cholesky", nbig, plan[0], workers, block=plan[1])
    static_s, static_sum = learned_run(torch, None, "cholesky", nbig, plan[0], workers, block=plan[1])
    print(json.dumps({
        "suite": "costmodel", "runs": len(runs), "records_total": int(len(Y)), "records_train": int(len(train_idx)),
        "records_heldout": int(test.sum()), "trace_seconds": trace_s, "train_seconds": train_s,
        "train_loss": loss, "heldout_median_rel_error": float(np.median(rel)),
        "heldout_p90_rel_error": float(np.percentile(rel, 90)), "heldout_runs_makespan": held_runs,
        "n": nbig, "plans": {f"nb{nb}/bs{bs}": v for (nb, bs), v in preds.items()},
        "learned": {"nb": plan[0], "block": plan[1], "predicted_makespan_s": preds[plan], "choice_seconds": plan_s,
                    "measured_makespan_s": learned_s, "static_priority_makespan_s": static_s},
        "fallback": {"nb": fb_nb, "block": "default", "measured_s_by_nb": fb_times, "search_seconds": fb_search_s,
                     "measured_makespan_s": fb_times[fb_nb]},
        "gain_over_fallback_makespan": fb_times[fb_nb] / learned_s,
        "gain_learned_over_static_priorities": static_s / learned_s,
        "factors_bitwise_identical_across_priorities": learned_sum == static_sum}), flush=True)


def run_kernels(args, P, torch) -> None:
    """The path's dominant kernels alone at N = --n (small captures for ncu): the tcgen05
    trailing update of step 0 (pack included), the compensated-FP32 residual and the
    update-form residual with 16 right-hand sides, and the two-level FP32 factorization of one
    NB x NB diagonal tile; CUDA-event times (best of 3 after 2 warm-ups) per call."""
    import ctypes
    n = args.n
    upd = time_update_kernel(P, torch, n, args.precision)
    a = torch.empty(n * n, dtype=torch.float64, device="cuda")
    P.gen_spd(a.data_ptr(), n, NB, 0)
    g = torch.Generator("cuda").manual_seed(1)
    x = torch.rand(16, n, dtype=torch.float64, device="cuda", generator=g) - 0.5
    b = torch.rand(16, n, dtype=torch.float64, device="cuda", generator=g)
    r = torch.empty_like(b)
    lib = P.lib()
    lib.palial_gpu_residual.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]

    def best(fn):
        for _ in range(2):
            fn()
        ts = []
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
        return min(ts)

    t_df = best(lambda: lib.palial_gpu_residual(a.data_ptr(), n, NB, x.data_ptr(), b.data_ptr(), r.data_ptr(), 16,
                                                1, None))
    t_up = best(lambda: lib.palial_gpu_residual(a.data_ptr(), n, NB, x.data_ptr(), None, r.data_ptr(), 16, 2,
                                                None))
    t_dig = best(lambda: lib.palial_gpu_residual(a.data_ptr(), n, NB, x.data_ptr(), b.data_ptr(), r.data_ptr(), 16,
                                                 3, None))
    t1 = torch.empty(NB * NB, dtype=torch.float64, device="cuda")
    P.gen_spd(t1.data_ptr(), NB, NB, 0)
    w1 = torch.empty(NB * NB, dtype=torch.float32, device="cuda")
    t_diag = best(lambda: P.mp_factor("cholesky", t1.data_ptr(), w1.data_ptr(), NB, NB, precision=args.precision))
    line = {"suite": "kernels", "n": n, "nb": NB, "precision": args.precision,
            "update_step0_s": upd["seconds"], "update_tflops": upd["flop"] / upd["seconds"] * 1e-12,
            "update_gbs": upd["bytes"] / upd["seconds"] * 1e-9,
            "residual_compensated_call_s": t_df, "residual_digits_call_s": t_dig,
            "residual_update_form_call_s": t_up,
            "residual_update_form_gbs": 8.0 * n * n / t_up * 1e-9,
            "diag_tile_call_s": t_diag}
    if args.all_kernels:
        line.update(every_kernel_once(P, torch, n))
    print(json.dumps(line), flush=True)


def every_kernel_once(P, torch, n: int) -> dict:
    """One call of each remaining path of the library at size n (the small case the per-kernel
    ncu captures select from): mixed-precision Cholesky and LU solves (diagonal tiles, panel
    solves, block inverses, refinement solves and residuals), FP64 Cholesky / LU / QR on the
    persistent scheduler, the FP32 QR solve (FP32 task scheduler; also with the tensor-core
    TSMQR), the host-buffer Cholesky solve, a batched FP32 solve of four matrices (FP32
    scheduler, batched residual and correction kernels, one LU on its butterfly transform) and a
    few MLP training steps; wall seconds per call."""
    import numpy as np
    out = {}
    nrhs = 16
    b = torch.empty(n * nrhs, dtype=torch.float64, device="cuda")
    P.gen_dense(b.data_ptr(), n, nrhs, 5, P.STREAM_RHS)
    x = torch.zeros_like(b)
    a = torch.empty(n * n, dtype=torch.float64, device="cuda")
    for alg, prec in (("cholesky", "bf16x3"), ("lu", "tf32x3")):
        P.gen_kappa(a.data_ptr(), n, NB, 1e2, alg == "cholesky", seed=7)
        st = P.solve_ir(alg, a.data_ptr(), n, NB, b.data_ptr(), x.data_ptr(), nrhs, precision=prec, raise_on_error=False)
        out[f"{alg}_{prec}_solve_s"] = st.seconds
    for alg in ("cholesky", "lu", "qr"):
        if alg == "cholesky":
            P.gen_spd(a.data_ptr(), n, NB, 0)
        else:
            P.gen_uniform(a.data_ptr(), n, NB, 1)
        s = torch.zeros_like(a) if alg == "qr" else None
        st = P.factor_dev(alg, a.data_ptr(), s.data_ptr() if s is not None else None, n, NB)
        out[f"{alg}_fp64_factor_s"] = st.seconds
        del s
    P.gen_uniform(a.data_ptr(), n, NB, 1)
    x.zero_()
    st = P.qr_solve_ir(a.data_ptr(), n, NB, b.data_ptr(), x.data_ptr(), nrhs, allow_not_converged=True)
    out["qr_fp32_solve_s"] = st.seconds
    x.zero_()
    st = P.qr_solve_ir(a.data_ptr(), n, NB, b.data_ptr(), x.data_ptr(), nrhs, allow_not_converged=True,
                       precision="bf16x3")
    out["qr_fp32_tensor_core_solve_s"] = st.seconds
    # the host-buffer Cholesky solve (upper triangle copied, lower written on the device)
    P.gen_spd(a.data_ptr(), n, NB, 0)
    host = torch.empty(n * n, dtype=torch.float64, pin_memory=True)
    host.copy_(a)
    bh = b.cpu().numpy().reshape(nrhs, n).copy()
    xh = np.zeros((nrhs, n))
    st = P.solve_ir_host("cholesky", host.numpy(), n, NB, bh, xh, nrhs, precision="bf16x3", raise_on_error=False)
    out["cholesky_host_solve_s"] = st.seconds
    del a, host
    torch.cuda.empty_cache()
    from palial_gb300 import batched as B
    rng = np.random.default_rng(0)
    sizes, nbs, algs = [512, 384, 256, 256], [128, 128, 64, 64], [0, 1, 0, 1]
    mats = []
    for k, m in enumerate(sizes):
        q = rng.uniform(-1, 1, (m, m))
        mats.append(q @ q.T + m * np.eye(m) if algs[k] == 0 else q + m * np.eye(m))
    mats[3] = rng.uniform(-1, 1, (256, 256))
    mats[3][0, 0] = 1e-9  # FP32 no-pivot LU fails: the butterfly stage solves it
    tiles = [torch.from_numpy(np.ascontiguousarray(
        mm.reshape(m // nb, nb, m // nb, nb).transpose(2, 0, 3, 1)).ravel()).cuda() for mm, m, nb in zip(mats, sizes, nbs)]
    rhs = [torch.from_numpy(rng.uniform(-1, 1, m)).cuda() for m in sizes]
    xs = [torch.zeros_like(r) for r in rhs]
    t0 = time.perf_counter()
    B.solve(algs, sizes, nbs, [t.data_ptr() for t in tiles], [r.data_ptr() for r in rhs], [v.data_ptr() for v in xs])
    out["batched_solve_s"] = time.perf_counter() - t0
    from palial_gb300.costmodel import CostModel
    m = CostModel(seed=0)
    xf = rng.uniform(-1, 1, (4096, m.nin)).astype(np.float32)
    t0 = time.perf_counter()
    m.train(xf, xf[:, 0].copy(), epochs=2, batch=512)
    out["mlp_train_s"] = time.perf_counter() - t0
    return out


def run_qr_mixed(args, P, torch) -> None:
    """QR solves of A X = B (A uniform [-1, 1), seed 1; 16 right-hand sides) at N = 16384 and
    32768: the mixed-precision QR (FP32 tile QR + FP64 refinement) with NB = 512 and 256 (its
    single-CTA TSQRT chain shortens with the tile), the same with its TSMQR products on the
    tensor cores (precision bf16x3), against the FP64 QR solve of the same system at NB = 512;
    whole calls on device buffers, TFLOP/s from 4N^3/3."""
    nrhs = 16
    for n in (16384, 32768):
        b = torch.empty(n * nrhs, dtype=torch.float64, device="cuda")
        P.gen_dense(b.data_ptr(), n, nrhs, 5, P.STREAM_RHS)
        x = torch.zeros_like(b)
        for nb in (NB, 256):
            da = torch.empty(n * n, dtype=torch.float64, device="cuda")
            P.gen_uniform(da.data_ptr(), n, nb, 1)
            x.zero_()
            st = P.qr_solve_ir(da.data_ptr(), n, nb, b.data_ptr(), x.data_ptr(), nrhs, allow_not_converged=True)
            line = {"suite": "qr_mixed", "n": n, "nb": nb, "nrhs": nrhs, "converged": st.code == 0,
                    "seconds": st.seconds, "factor_seconds": st.factor_seconds, "ir_iters": st.ir_iters,
                    "backward_error": st.backward_error,
                    "tflops_fp64_equiv": 4.0 * n ** 3 / 3.0 / st.seconds * 1e-12,
                    "precision_used": "fp32" if st.precision_used == 5 else "fp64", "message": st.message.decode()}
            x.zero_()
            tc = P.qr_solve_ir(da.data_ptr(), n, nb, b.data_ptr(), x.data_ptr(), nrhs, allow_not_converged=True,
                               precision="bf16x3")
            line["tensor_core_tsmqr"] = {"converged": tc.code == 0, "seconds": tc.seconds,
                                         "factor_seconds": tc.factor_seconds, "ir_iters": tc.ir_iters,
                                         "backward_error": tc.backward_error,
                                         "precision_used": {3: "bf16x3", 5: "fp32"}.get(tc.precision_used, "fp64")}
            if nb == NB:
                x.zero_()
                s64 = P.qr_solve(da.data_ptr(), n, n, NB, b.data_ptr(), x.data_ptr(), nrhs)
                line["fp64_qr_solve"] = {"seconds": s64.seconds, "tflops": 4.0 * n ** 3 / 3.0 / s64.seconds * 1e-12}
                line["speedup_over_fp64"] = s64.seconds / st.seconds
            print(json.dumps(line), flush=True)
            del da
            torch.cuda.empty_cache()
        del b, x


def run_suite(args, P, torch) -> None:
    import numpy as np
    if args.suite == "kernels":
        run_kernels(args, P, torch)
        return
    if args.suite == "costmodel":
        run_costmodel(args, P, torch)
        return
    if args.suite == "batched":
        run_batched(args, P, torch)
        return
    if args.suite == "batched_solve":
        run_batched_solve(args, FP64_BATCH_BLOCKS, args.batch, 1)
        return
    if args.suite == "qr_mixed":
        run_qr_mixed(args, P, torch)
        return
    if args.suite == "fp64":
        for alg in ((args.alg,) if args.alg else ("cholesky", "lu", "qr")):
            for n in ((4096, 16384, 32768) if alg == "cholesky" else (16384, 32768)):
                d0 = torch.empty(n * n, dtype=torch.float64, device="cuda")
                if alg == "cholesky":
                    P.gen_spd(d0.data_ptr(), n, NB, 0)
                else:
                    P.gen_uniform(d0.data_ptr(), n, NB, 1)
                s = torch.zeros_like(d0) if alg == "qr" else None
                d = d0.clone()
                st = P.factor_dev(alg, d.data_ptr(), s.data_ptr() if s is not None else None, n, NB)
                probe = P.residual_probe(alg, d0.data_ptr(), d.data_ptr(), n, NB, 8)
                print(json.dumps({"suite": "fp64", "alg": alg, "n": n, "nb": NB, "seconds": st.seconds,
                                  "tflops": st.tflops, "residual_probe": probe,
                                  "note": "TFLOP/s from N^3/3, 2N^3/3, 4N^3/3"}), flush=True)
                del d, d0, s
                torch.cuda.empty_cache()
        return
    n, nrhs = args.n, 16
    b = torch.empty(n * nrhs, dtype=torch.float64, device="cuda")
    P.gen_dense(b.data_ptr(), n, nrhs, 5, P.STREAM_RHS)
    import ctypes
    for alg in ("cholesky", "lu"):
        for kappa in (1e2, 1e6, 1e10):
            da = torch.empty(n * n, dtype=torch.float64, device="cuda")
            P.gen_kappa(da.data_ptr(), n, NB, kappa, alg == "cholesky", seed=7)
            precs = ("bf16", "fp8", "bf16x3", "tf32x3", "auto") + (("bf16x3-rbt",) if alg == "lu" else ())
            for prec in precs:
                dx = torch.zeros_like(b)
                o = P.make_opts(precision=prec.split("-")[0], ir_max_iter=30)
                o.reserved[6] = 1 if prec.endswith("-rbt") else 0  # LU of the random-butterfly transform
                st = P.Status()
                st.code = P.lib().palial_gpu_solve_ir(P.ALG[alg], da.data_ptr(), n, NB, b.data_ptr(), dx.data_ptr(),
                                                      nrhs, ctypes.byref(o), ctypes.byref(st), None)
                print(json.dumps({"suite": "kappa", "alg": alg, "n": n, "kappa": kappa, "precision": prec,
                                  "converged": st.code in (0, 1), "code": st.code, "ir_iters": st.ir_iters,
                                  "gmres_iters": st.gmres_iters, "backward_error": st.backward_error,
                                  "seconds": st.seconds, "factor_seconds": st.factor_seconds, "shift": st.shift,
                                  "tflops_fp64_equiv": st.tflops,
                                  "precision_used": (P.PREC_NAME.get(st.precision_used, prec)
                                                     if prec == "auto" else prec)}), flush=True)
            del da
            torch.cuda.empty_cache()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=10, help="host-buffer steps (the pageable leg runs half)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--n", type=int, default=N)
    ap.add_argument("--precision", default="bf16x3")
    ap.add_argument("--suite", default=None, choices=[None, "fp64", "kappa", "batched", "batched_solve", "costmodel",
                                                      "kernels", "qr_mixed"])
    ap.add_argument("--batch", type=int, default=2000)
    ap.add_argument("--costmodel-n", type=int, default=49152, help="target size of the cost-model suite")
    ap.add_argument("--all-kernels", action="store_true", help="kernels suite: also run every other path once")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the kappa / lu / qr keys")
    ap.add_argument("--alg", default=None, choices=[None, "cholesky", "lu", "qr"], help="fp64 suite: one algorithm")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    rank, world, local = dist_info()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import numpy as np
    import torch

    import palial_gb300 as P

    n, nrhs = args.n, 16
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    P.init(local)
    if args.suite == "batched":
        run_batched(args, P, torch, rank, world)
        return
    if args.suite == "batched_solve":
        if rank == 0:
            run_batched_solve(args, FP64_BATCH_BLOCKS, args.batch, world)
        return
    if args.suite:
        if rank == 0:
            run_suite(args, P, torch)
        return
    stream = torch.cuda.current_stream()
    a0 = torch.empty(n * n, dtype=torch.float64, device="cuda")
    P.gen_spd(a0.data_ptr(), n, NB, seed=rank)
    b = torch.empty(n * nrhs, dtype=torch.float64, device="cuda")
    P.gen_dense(b.data_ptr(), n, nrhs, 5, P.STREAM_RHS)  # uniform [-1, 1), column-major
    x = torch.zeros_like(b)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def step() -> P.Status:
        return P.solve_ir("cholesky", a0.data_ptr(), n, NB, b.data_ptr(), x.data_ptr(), nrhs,
                          precision=args.precision, stream=stream.cuda_stream, raise_on_error=False)

    for _ in range(args.warmup):
        step()
    sts = []
    barrier()
    launches0 = P.lib().palial_gpu_kernel_launches()
    with ClockSampler(local) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        torch.cuda.nvtx.range_push("timed_steps")  # profilers can select this region by name
        for _ in range(args.steps):
            sts.append(step())
        torch.cuda.nvtx.range_pop()
        e1.record(stream)
        barrier()
    total = e0.elapsed_time(e1) * 1e-3
    gpu_launches = P.lib().palial_gpu_kernel_launches() - launches0
    if world > 1:
        t = torch.tensor([total], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total = float(t.item())
    per_step = total / args.steps
    value = world * flops(n) / per_step * 1e-12
    converged = all(st.code in (0, 1) for st in sts)
    eta = max(st.backward_error for st in sts)
    launches = sts[-1].ir_iters  # informational
    eta_fp64 = fp64_backward_error(P, torch, a0, n, NB, x, b, nrhs)  # untimed check of the last X

    # plain FP64 tiled factorization of the same matrix (one timed run after the DAG is built)
    fp64 = None
    if not args.no_fp64:
        a = torch.empty_like(a0)
        a.copy_(a0)
        P.factor_dev("cholesky", a.data_ptr(), None, n, NB, stream=stream.cuda_stream, allow_warn=False)
        a.copy_(a0)
        st64 = P.factor_dev("cholesky", a.data_ptr(), None, n, NB, stream=stream.cuda_stream, allow_warn=False)
        fp64 = {"tflops": st64.tflops, "seconds": st64.seconds,
                "residual_probe": P.residual_probe("cholesky", a0.data_ptr(), a.data_ptr(), n, NB, 8),
                "speedup_mixed_over_fp64": (flops(n) / per_step * 1e-12) / st64.tflops}
        del a
        torch.cuda.empty_cache()

    # the metric's other configurations (kappa = 1e6 Cholesky / LU, LU, QR) at N = n, once each
    extra = {} if args.no_extra else config_keys(P, torch, n, b, nrhs, stream.cuda_stream)

    # roofline: live timing of the tcgen05 update kernel at its largest step
    pk = peaks()
    upd = time_update_kernel(P, torch, n, args.precision)
    gbs = upd["bytes"] / upd["seconds"] * 1e-9
    # bound from the arithmetic intensity against the measured ridge (BF16 burst / HBM copy)
    tfs = upd["flop"] / upd["seconds"] * 1e-12
    ridge = pk.get("bf16_tflops", 1900.0) * 1e12 / (pk.get("hbm_gbs", 6800.0) * 1e9)
    if upd["flop"] / upd["bytes"] > ridge:
        bound, achieved, peak, unit = "tensor", tfs, pk.get("bf16_tflops", 1900.0), "TFLOP/s"
    else:
        bound, achieved, peak, unit = "hbm", gbs, pk.get("hbm_gbs", 6800.0), "GB/s"

    # e2e: host buffers through the C ABI
    host = torch.empty(n * n, dtype=torch.float64, pin_memory=True)
    host.copy_(a0)  # device -> pinned directly (no 8.6 GB pageable temporary on the host)
    torch.cuda.synchronize()
    host_np = host.numpy()
    xh = np.zeros((nrhs, n))
    bhc = b.cpu().numpy().reshape(nrhs, n).copy()  # column-major n x nrhs == row-major nrhs x n
    e2e_times = []
    for i in range(1 + args.e2e_steps):
        barrier()
        t0 = time.perf_counter()
        P.solve_ir_host("cholesky", host_np, n, NB, bhc, xh, nrhs, precision=args.precision, raise_on_error=False)
        barrier()
        if i >= 1:
            e2e_times.append(time.perf_counter() - t0)
    e2e_sec = sum(e2e_times) / len(e2e_times) if e2e_times else float("nan")
    e2e_value = world * flops(n) / e2e_sec * 1e-12
    # the host link itself: a plain copy of A from the same pinned buffer, a few times
    link = []
    for _ in range(4):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        a0.copy_(host, non_blocking=True)
        torch.cuda.synchronize()
        link.append(round(8.0 * n * n / (time.perf_counter() - t0) * 1e-9, 1))
    # the same from pageable host memory, as the reference's own caller allocates it
    # (posix_memalign, palial_src/main.c:110): numpy's buffer is ordinary malloc'd memory
    page = np.empty(n * n)
    page[:] = host_np
    del host, host_np
    page_times = []
    for i in range(1 + max(1, args.e2e_steps // 2)):
        barrier()
        t0 = time.perf_counter()
        P.solve_ir_host("cholesky", page, n, NB, bhc, xh, nrhs, precision=args.precision, raise_on_error=False)
        barrier()
        if i >= 1:
            page_times.append(time.perf_counter() - t0)
    page_sec = sum(page_times) / len(page_times)
    del page

    # the host-buffer Cholesky copies the upper triangle's tiles of A (the triangle the
    # factorization reads; the lower one is written on the device from it) and B
    mt = n // NB
    h2d_bytes = 8 * NB * NB * mt * (mt + 1) // 2 + 8 * n * nrhs
    if rank == 0:
        cpu = None
        if not args.no_cpu:
            nthreads = os.cpu_count() or 1
            spd = spd_host_from_gpu(P, torch, CPU_N, 0)
            v, sec = cpu_baseline_sample(nthreads, spd_host=spd)
            cpu = {"value": v, "unit": "TFLOP/s", "cores": nthreads, "kind": "port",
                   "sample": f"one Cholesky N={CPU_N} NB={NB} ({sec:.1f} s): the oracle's OpenMP restatement of "
                             "reference src/cholesky.h over OpenBLAS on all host cores"}
        line = {
            "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": headline_config(n, args.precision, world),
            "converged": converged, "backward_error": eta, "backward_error_fp64_check": eta_fp64,
            "ir_iters": launches,
            "fp64_tiled": fp64,
            "e2e": {"value": e2e_value, "unit": "TFLOP/s", "h2d_bytes_per_step": h2d_bytes,
                    "d2h_bytes_per_step": 8 * n * nrhs, "step_seconds": [round(t, 5) for t in e2e_times],
                    "host_buffer": "pinned (page-locked) A",
                    "host_link_gbs_samples": link},
            "e2e_pageable": {"value": world * flops(n) / page_sec * 1e-12, "unit": "TFLOP/s",
                             "h2d_bytes_per_step": h2d_bytes, "d2h_bytes_per_step": 8 * n * nrhs,
                             "step_seconds": [round(t, 5) for t in page_times],
                             "host_buffer": "pageable A (numpy / malloc), as the reference's caller"},
            **extra,
            "roofline": {"bound": bound, "achieved": achieved, "peak": peak, "unit": unit,
                         "frac": achieved / peak,
                         "hbm_gbs": gbs, "hbm_frac": gbs / pk.get("hbm_gbs", 6800.0),
                         # DRAM read + write of one launch: ncu (dram__bytes_read.sum +
                         # dram__bytes_write.sum) on the BF16x3 tile-run update at N=16384, k=0 (496
                         # tile pairs, 576.8 + 469.0 MB, profiles/mp_update_run_n16384.md), scaled by tile pairs
                         "traffic": 1045.8e6 / 496 * ((n // NB - 1) * (n // NB) // 2),
                         "traffic_note": "ncu capture of the BF16x3 update at N=16384 step 0 (bench.py --suite "
                                         "kernels --n 16384), scaled by tile pairs; algorithmic C bytes are 2 MB per pair",
                         "kernel": "mp_update_run_kernel<%s> (tcgen05, step k=0 of N=%d, pack included)" % (args.precision, n),
                         "tensor_tflops": upd["flop"] / upd["seconds"] * 1e-12,
                         "tensor_frac_of_bf16_peak": upd["flop"] / upd["seconds"] * 1e-12 / pk.get("bf16_tflops", 1900.0),
                         # the factorization's own flops (one product per tile pair): the BF16x3 split
                         # spends two thirds of the tensor work on precision
                         "algorithmic_tflops": upd["flop"] / upd["products"] / upd["seconds"] * 1e-12,
                         "algorithmic_frac": upd["flop"] / upd["products"] / upd["seconds"] * 1e-12 / pk.get("bf16_tflops", 1900.0),
                         "peak_source": "MEASURED_PEAKS.json (of measured)" if "source" not in pk else "fallback"},
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "gpu_launches": gpu_launches,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
