"""Benchmark: tiled Cholesky at N = 32768, NB = 512 on one GB300 (per GPU).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one factorization of a device-resident N x N SPD matrix (B B^T + N I, B on a
2^-7 grid in [-1, 1), seed 0; the reference's tile layout) through the library's
device-pointer entry point, including the restore of the input from a pristine copy
(8.6 GB device-to-device).  Inputs (8.6 GB) are far larger than L2 (129 MB), so no flush
is needed.  value = algorithmic FP64 flops (N^3/3) per step / step time, whole job (sum
over ranks; replicas: each rank factors its own matrix, no collective on the data path).

The JSON line also carries:
  e2e           the same metric through the host-buffer C ABI entry point
                (palial_gpu_cholesky on pinned host memory: H2D + factor + D2H per step);
  roofline      the scheduler kernel's FP64 rate against the FP64 peak measured in this
                run with cuBLAS DGEMM (no FP64 figure exists in MEASURED_PEAKS.json);
  cpu_baseline  the oracle's OpenMP port of the reference (same task DAG, same OpenBLAS
                calls) on this host's cores, on a bounded sample (N = 16384);
  clocks        nvidia-smi samples taken during the timed region.
`--impl reference` times the reference's CPU implementation (the oracle port, OpenMP, all
host cores) on the same metric, one bounded sample (N = 16384) per step.
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
    from oracle import oracle as O
    import numpy as np

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


def run_reference(args, rank: int, world: int) -> None:
    if rank != 0:
        return
    nthreads = os.cpu_count() or 1
    times = []
    spd = None
    try:
        import torch  # noqa: F401
        if torch.cuda.is_available():
            import palial_gb300 as P
            P.init(0)
            spd = spd_host_from_gpu(P, torch, CPU_N, 0)
    except Exception:  # the CPU arm does not need a GPU: generate on the host instead
        spd = None
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
        "config": {"workload": f"tiled Cholesky FP64, N={CPU_N} (bounded sample of N={N}), NB={NB}, "
                               f"SPD B*B^T+N*I seed 0", "n": CPU_N, "nb": NB},
        "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": nthreads, "kind": "port",
                         "sample": f"one Cholesky N={CPU_N} NB={NB} per step: the oracle's OpenMP restatement "
                                   "of reference src/cholesky.h over OpenBLAS, OMP_NUM_THREADS=all cores"},
        "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--n", type=int, default=N)
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    rank, world, local = dist_info()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import numpy as np
    import torch

    import palial_gb300 as P

    n = args.n
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    P.init(local)
    stream = torch.cuda.current_stream()
    peak = fp64_peak_tflops(torch)

    a0 = torch.empty(n * n, dtype=torch.float64, device="cuda")
    a = torch.empty_like(a0)
    P.gen_spd(a0.data_ptr(), n, NB, seed=rank)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def step() -> float:
        a.copy_(a0)
        st = P.factor_dev("cholesky", a.data_ptr(), None, n, NB, stream=stream.cuda_stream, allow_warn=False)
        return st.seconds

    for _ in range(args.warmup):
        step()
    kern = []
    barrier()
    with ClockSampler(local) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            kern.append(step())
        e1.record(stream)
        barrier()
    total = e0.elapsed_time(e1) * 1e-3
    if world > 1:
        t = torch.tensor([total], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total = float(t.item())
    per_step = total / args.steps
    value = world * flops(n) / per_step * 1e-12
    resid = P.residual_probe("cholesky", a0.data_ptr(), a.data_ptr(), n, NB, 8)

    # e2e: host buffers through the C ABI (H2D + factor + D2H inside each timed step)
    host = torch.empty(n * n, dtype=torch.float64, pin_memory=True)
    host_np = host.numpy()
    a0_host = a0.cpu()
    del a
    torch.cuda.empty_cache()
    e2e_times = []
    for i in range(1 + args.e2e_steps):
        host.copy_(a0_host)
        barrier()
        t0 = time.perf_counter()
        P.cholesky(host_np, n, NB)
        barrier()
        if i >= 1:
            e2e_times.append(time.perf_counter() - t0)
    e2e_sec = sum(e2e_times) / max(1, len(e2e_times)) if e2e_times else float("nan")
    e2e_value = world * flops(n) / e2e_sec * 1e-12
    del host, a0_host

    line = None
    if rank == 0:
        cpu = None
        if not args.no_cpu:
            nthreads = os.cpu_count() or 1
            spd = spd_host_from_gpu(P, torch, CPU_N, 0)
            v, sec = cpu_baseline_sample(nthreads, spd_host=spd)
            cpu = {"value": v, "unit": "TFLOP/s", "cores": nthreads, "kind": "port",
                   "sample": f"one Cholesky N={CPU_N} NB={NB} ({sec:.1f} s): the oracle's OpenMP restatement of "
                             "reference src/cholesky.h over OpenBLAS on all host cores"}
        kern_avg = sum(kern) / len(kern)
        achieved = flops(n) / kern_avg * 1e-12
        line = {
            "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"tiled Cholesky FP64 (plain path), N={n}, NB={NB}, scheduler block 256, "
                                   "SPD B*B^T+N*I seed=rank, device-resident; inputs 8.6 GB >> L2 (no flush needed)",
                       "n": n, "nb": NB, "precision": "fp64", "parallelism": f"replicas x{world}"},
            "e2e": {"value": e2e_value, "unit": "TFLOP/s", "h2d_bytes_per_step": 8 * n * n,
                    "d2h_bytes_per_step": 8 * n * n},
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": None,
                         "kernel": "sched_f64_kernel (persistent scheduler, 1 launch per step)",
                         "peak_source": "FP64 cuBLAS DGEMM 8192^3 measured in this run (no FP64 peak in "
                                        "MEASURED_PEAKS.json)"},
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "gpu_launches": args.steps,
            "residual_probe": resid,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
