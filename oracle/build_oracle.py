"""Build recipe for the CPU oracle (test infrastructure only).

* ``oracle/liboracle.so``: the C restatement (palial_oracle.c), built with -fopenmp so
  that it can run serially (parity oracle) or as OpenMP tasks (timed CPU baseline).
* ``oracle/_ref/libpalial_ref_serial.so`` and ``oracle/_ref/libpalial_ref_omp.so``: the
  reference's own hot-path headers compiled unmodified through ref_harness.c, only when a
  reference checkout is available (this container).  They are git-ignored build outputs.

Both link SciPy's bundled OpenBLAS (the reference links OpenBLAS through pkg-config,
palial_src/Makefile:18, unpinned; here it is the OpenBLAS that ships inside SciPy).
Flags follow the reference's needs: -ftrivial-auto-var-init=zero because src/lu.h:13 and
src/qr.h:17 print uninitialised loop variables into fixed-size buffers.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference checkout: $PALIAL_REFERENCE, else a "reference" directory beside this
# repository (absent on machines without a checkout; the reference build is then skipped).
REF_DEFAULT = os.environ.get("PALIAL_REFERENCE") or os.path.join(
    os.path.dirname(os.path.dirname(os.path.realpath(HERE))), "reference")


def find_openblas() -> str:
    """Return the path of SciPy's bundled OpenBLAS shared library."""
    import scipy  # noqa: WPS433 (import inside: scipy is only needed to locate the file)

    base = os.path.dirname(os.path.dirname(os.path.abspath(scipy.__file__)))
    hits = sorted(glob.glob(os.path.join(base, "scipy.libs", "libscipy_openblas*.so*")))
    hits = [h for h in hits if "openblas64" not in os.path.basename(h)]
    if not hits:
        raise RuntimeError("SciPy's bundled OpenBLAS (scipy.libs/libscipy_openblas*.so) not found")
    return hits[0]


def _cc(args: list[str]) -> None:
    proc = subprocess.run(args, capture_output=True, text=True)
    if proc.returncode != 0:
        sys.stderr.write(" ".join(args) + "\n" + proc.stdout + proc.stderr)
        raise RuntimeError(f"oracle build failed: {args[-1]}")


def _link_args(blas: str) -> list[str]:
    d = os.path.dirname(blas)
    return [blas, f"-Wl,-rpath,{d}", "-lm"]


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(p) > t for p in deps if os.path.exists(p))


def build_oracle(force: bool = False) -> str:
    blas = find_openblas()
    src = os.path.join(HERE, "palial_oracle.c")
    out = os.path.join(HERE, "liboracle.so")
    shim = os.path.join(HERE, "blas_shim")
    deps = [src, os.path.join(shim, "cblas.h"), os.path.join(shim, "lapacke.h")]
    if force or _stale(out, deps):
        _cc(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-std=gnu11", f"-I{shim}", src, "-o", out]
            + _link_args(blas))
    return out


def build_reference(ref_root: str = REF_DEFAULT, force: bool = False) -> list[str]:
    """Compile the reference's hot path (serial and OpenMP) into oracle/_ref/.

    Returns the list of built libraries, or [] when no reference checkout is present.
    """
    if not os.path.isdir(os.path.join(ref_root, "src")):
        return []
    blas = find_openblas()
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    harness = os.path.join(HERE, "ref_harness.c")
    shim = os.path.join(HERE, "blas_shim")
    inc = [f"-I{shim}", f"-I{os.path.join(ref_root, 'include')}", f"-I{os.path.join(ref_root, 'src')}"]
    deps = [harness] + glob.glob(os.path.join(ref_root, "src", "**", "*.h"), recursive=True)
    built = []
    for name, omp in (("libpalial_ref_serial.so", []), ("libpalial_ref_omp.so", ["-fopenmp"])):
        out = os.path.join(outdir, name)
        if force or _stale(out, deps):
            _cc(["gcc", "-O2", "-fPIC", "-shared", "-std=gnu99", "-ftrivial-auto-var-init=zero",
                 "-w", *omp, *inc, harness, "-o", out] + _link_args(blas))
        built.append(out)
    return built


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    for p in build_reference(force="--force" in sys.argv):
        print(p)
