"""Generate the golden fixtures in this directory from the REFERENCE itself.

Runs the reference's own hot-path sources (compiled unmodified into oracle/_ref/ by
oracle/build_oracle.py, serial program order) on seeded inputs and stores inputs'
checksums and outputs as small .npz files:

* ``special4x4.npz``  the reference's compile-time 4x4 fixture (include/populate.h:13-33,
  NB = 2) and the reference's Cholesky / LU / QR of it;
* ``chol_192_64.npz``, ``lu_192_64.npz``, ``lu_dom_128_32.npz``, ``qr_192_64.npz``: factors
  of the seeded generators (SPD B B^T + N I with seed 0; uniform [-1, 1) with seed 1; the
  reference's own diagonally dominant pattern 0.5 + diag in [173, 346) from seed 3);
* ``sha256.json``: SHA-256 of reference outputs at N = 1024, NB = 256 (bit-exact check of
  the restatement wherever the same OpenBLAS build is loaded);
* ``trace_names_cholesky_8192_512.txt``: the task names, in creation order, of the
  reference's own published trace of Cholesky N = 8192, NB = 512
  (exp/data/tasks_times_8192_512_31_ondemand, first column).

Usage: ``python tests/golden/make_golden.py`` (needs the reference checkout).
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import build_oracle, oracle as O  # noqa: E402

REF = build_oracle.REF_DEFAULT


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def dominant(seed: int, n: int) -> np.ndarray:
    """The reference generator's pattern (include/populate.h:36-67) with a seeded diagonal:
    0.5 everywhere, diagonal 173 * (1 + u) with u uniform in [0, 1)."""
    a = np.full((n, n), 0.5)
    u = (O.gen_uniform(seed, n, 1)[:, 0] + 1.0) * 0.5
    a[np.diag_indices(n)] = 173.0 * u + 173.0
    return a


def ref_factor(alg: str, a: np.ndarray, nb: int):
    n = a.shape[0]
    t = O.to_tiles(a, nb)
    s = np.zeros_like(t) if alg == "qr" else None
    O.run_reference(alg, t, n, nb, s)
    return t, s


def main() -> None:
    built = build_oracle.build_reference()
    if not built:
        raise SystemExit("reference checkout not found; fixtures can only be made where it exists")
    blas = os.path.basename(build_oracle.find_openblas())

    # 1. the reference's own 4x4 fixture
    special = np.zeros(16)
    O.ref_lib().ref_populate_special4x4(special.ctypes.data_as(O._dp()))  # noqa: SLF001
    out = {"a_tiles": special.copy()}
    for alg in ("cholesky", "lu", "qr"):
        t = special.copy()
        s = np.zeros_like(t) if alg == "qr" else None
        O.run_reference(alg, t, 4, 2, s)
        out[f"{alg}_tiles"] = t
        if s is not None:
            out["qr_s_tiles"] = s
    np.savez(os.path.join(HERE, "special4x4.npz"), **out)

    meta = {"openblas": blas}
    cases = [
        ("chol_192_64", "cholesky", lambda: O.gen_spd(0, 192), 64),
        ("lu_192_64", "lu", lambda: O.gen_uniform(1, 192), 64),
        ("lu_dom_128_32", "lu", lambda: dominant(3, 128), 32),
        ("qr_192_64", "qr", lambda: O.gen_uniform(1, 192), 64),
    ]
    for name, alg, gen, nb in cases:
        a = gen()
        t, s = ref_factor(alg, a, nb)
        rec = {"input_sha256": sha(O.to_tiles(a, nb)), "n": a.shape[0], "nb": nb, "alg": alg}
        arrays = {"out_tiles": t}
        if s is not None:
            arrays["s_tiles"] = s
        np.savez(os.path.join(HERE, f"{name}.npz"), **arrays)
        meta[name] = rec

    big = {}
    for alg, gen in (("cholesky", lambda: O.gen_spd(0, 1024)), ("lu", lambda: O.gen_uniform(1, 1024)),
                     ("qr", lambda: O.gen_uniform(1, 1024))):
        t, s = ref_factor(alg, gen(), 256)
        big[alg] = {"out": sha(t)}
        if s is not None:
            # only the upper triangles of S tiles are defined by the reference
            mt = 4
            st = s.reshape(mt, mt, 256, 256).copy()
            for i in range(mt):
                for j in range(mt):
                    st[i, j] = np.triu(st[i, j].T).T  # tile stored column-major: [col][row]
            big[alg]["s_upper"] = sha(st)
    meta["sha256_1024_256"] = big
    published = os.path.join(REF, "exp", "data", "tasks_times_8192_512_31_ondemand")
    with open(published) as src, open(os.path.join(HERE, "trace_names_cholesky_8192_512.txt"), "w") as dst:
        for line in src:
            dst.write(line.split(",")[0].strip() + "\n")
    with open(os.path.join(HERE, "sha256.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print("wrote fixtures for", blas)


if __name__ == "__main__":
    main()
