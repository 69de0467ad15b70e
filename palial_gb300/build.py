"""Build libpalial_gpu.so (sm_103a) and the `palial` command-line program, in tree.

Translation units are compiled in parallel with nvcc (one -gencode, sm_103a only) and
linked with the static CUDA runtime.  Outputs: palial_gb300/lib/libpalial_gpu.so and
palial_gb300/bin/palial.  Both are git-ignored build products.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lib", "libpalial_gpu.so")
BIN = os.path.join(HERE, "bin", "palial")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
           "-Xcompiler", "-Wall", "-Xcompiler", "-Wno-unused-function"]

SOURCES = ["sched_f64.cu", "gen_check.cu", "runtime.cu", "dag.cpp", "noalloc.cu", "mp_gemm.cu", "mp_solve.cu", "mp_driver.cu", "mlp.cu", "nvml_clock.cpp", "qr_solve.cu", "batch_driver.cu", "mp_diag.cu", "mp_rhs.cu", "layout.cu", "rbt.cu", "sched_f32.cu", "batch_solve.cu", "mp_qr.cu", "mp_resid_digits.cu"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _deps(src: str) -> list[str]:
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    return [src] + hdrs + [os.path.join(ROOT, "include", "palial_gpu.h")]


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd: list[str]) -> None:
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + p.stdout + p.stderr)
        raise RuntimeError(f"build step failed: {cmd[-1]}")
    if p.stderr.strip() and os.environ.get("PALIAL_BUILD_VERBOSE"):
        sys.stderr.write(p.stderr)


def _compile(src: str, force: bool, extra: list[str]) -> str:
    path = os.path.join(CSRC, src)
    out = os.path.join(OBJ, src + ".o")
    if force or _stale(out, _deps(path)):
        lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
        _run([nvcc(), *ARCH, *NVFLAGS, *extra, f"-I{os.path.join(ROOT, 'include')}", *lang, "-c", path, "-o", out])
    return out


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    os.makedirs(os.path.dirname(BIN), exist_ok=True)
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, force, extra), SOURCES))
    if force or _stale(LIB, objs):
        _run([nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs, "-lpthread", "-ldl", "-lrt"])
    cli = os.path.join(HOST, "palial_main.c")
    if os.path.exists(cli) and (force or _stale(BIN, [cli, LIB, os.path.join(ROOT, "include", "palial_entry.h"),
                                                     os.path.join(ROOT, "include", "palial_descriptor.h")])):
        _run(["gcc", "-O2", "-std=gnu11", f"-I{os.path.join(ROOT, 'include')}", cli, "-o", BIN,
              f"-L{os.path.dirname(LIB)}", "-lpalial_gpu", f"-Wl,-rpath,{os.path.dirname(LIB)}", "-lm"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="--ptxas" in sys.argv))
