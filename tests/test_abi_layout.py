"""The Python (ctypes) mirrors of the C-ABI structs agree with the header: every field's offset
and every struct's size, compiled from include/palial_gpu.h with the host C compiler (no GPU)."""
import ctypes
import os
import shutil
import subprocess
import tempfile

import pytest

from palial_gb300 import Desc, Opts, Status
from palial_gb300.batched import BatchReport, SolveReport

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MIRRORS = {"palial_desc": Desc, "palial_opts": Opts, "palial_status": Status,
           "palial_batch_report": BatchReport, "palial_batch_solve_report": SolveReport}


def _c_layout():
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "palial_gpu.h"', "int main(void) {"]
    for cname, py in MIRRORS.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "layout.c"), os.path.join(d, "layout")
        with open(src, "w") as fh:
            fh.write("\n".join(lines))
        subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    return {tuple(l.split()[:2]): int(l.split()[2]) for l in out.splitlines()}


def test_ctypes_mirrors_match_the_header():
    c = _c_layout()
    for cname, py in MIRRORS.items():
        assert ctypes.sizeof(py) == c[(cname, "size")], cname
        for f, _ in py._fields_:
            assert getattr(py, f).offset == c[(cname, f)], (cname, f)
