"""GPU-clock reporting against a fake NVML, and the reference trace-hook bridge of
palial_entry.h (compiles with and without hooks; on a GPU the hooks receive every task).

The clock code only queries NVML (the reference's palial_power/server.c sets CPU frequencies;
nothing here sets a GPU clock): the test also checks that every NVML symbol it resolves is
a query (nvmlInit or nvmlDeviceGet*)."""
import ctypes
import json
import os
import re
import subprocess
import sys
import textwrap

import pytest

import palial_gb300 as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")

FAKE_NVML = r"""
int nvmlInit_v2(void) { return 0; }
int nvmlDeviceGetHandleByPciBusId_v2(const char *bus, void **dev) { (void)bus; (void)dev; return 6; }
int nvmlDeviceGetHandleByIndex_v2(unsigned i, void **dev) { *dev = (void *)(unsigned long)(i + 1); return 0; }
int nvmlDeviceGetClockInfo(void *dev, int type, unsigned *mhz) { *mhz = type == 1 ? 1965u : 3996u; return dev ? 0 : 1; }
int nvmlDeviceGetMaxClockInfo(void *dev, int type, unsigned *mhz) { *mhz = type == 1 ? 2070u : 3996u; return dev ? 0 : 1; }
int nvmlDeviceGetCurrentClocksEventReasons(void *dev, unsigned long long *r) { *r = 0x4ull; return dev ? 0 : 1; }
"""


def test_nvml_symbols_are_queries_only():
    src = open(os.path.join(ROOT, "palial_gb300", "csrc", "nvml_clock.cpp")).read()
    syms = re.findall(r'dlsym\(h, "(\w+)"\)', src)
    assert syms and all(s == "nvmlInit_v2" or s.startswith("nvmlDeviceGet") for s in syms), syms


def test_clock_sample_with_fake_nvml(tmp_path):
    so = tmp_path / "libfakenvml.so"
    c = tmp_path / "fake.c"
    c.write_text(FAKE_NVML)
    subprocess.run(["gcc", "-shared", "-fPIC", "-O1", str(c), "-o", str(so)], check=True)
    code = textwrap.dedent(f"""
        import ctypes, json
        lib = ctypes.CDLL({P.LIB_PATH!r})
        a, b, r = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        rc = lib.palial_gpu_clock_sample(ctypes.byref(a), ctypes.byref(b), ctypes.byref(r))
        class Rep(ctypes.Structure):
            _fields_ = [("s", ctypes.c_double), ("e", ctypes.c_double), ("m", ctypes.c_double),
                        ("d", ctypes.c_double), ("r", ctypes.c_int)]
        rep = Rep()
        rc2 = lib.palial_gpu_clock_report(ctypes.byref(rep))
        print(json.dumps([rc, a.value, b.value, r.value, rc2, rep.e, rep.m, rep.r, rep.s, rep.d]))
    """)
    env = dict(os.environ, PALIAL_NVML_LIBRARY=str(so), CUDA_VISIBLE_DEVICES="")
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, check=True)
    rc, sm, mx, reasons, rc2, e, m, r2, s, d = json.loads(out.stdout.strip().splitlines()[-1])
    assert (rc, sm, mx, reasons) == (0, 1965.0, 2070.0, 4)
    # no traced run: the report carries the current sample, start and device estimate unknown
    assert (rc2, e, m, r2, s, d) == (0, 1965.0, 2070.0, 4, -1.0, -1.0)


def test_clock_sample_without_nvml_reports_unavailable():
    code = textwrap.dedent(f"""
        import ctypes
        lib = ctypes.CDLL({P.LIB_PATH!r})
        a, b, r = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        print(lib.palial_gpu_clock_sample(ctypes.byref(a), ctypes.byref(b), ctypes.byref(r)), a.value, r.value)
    """)
    env = dict(os.environ, PALIAL_NVML_LIBRARY="/nonexistent/libnvidia-ml.so.1")
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, check=True)
    rc, a, r = out.stdout.split()
    assert int(rc) == -5 and float(a) == -1.0 and int(r) == -1


HOOK_PROG = r"""
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "palial_descriptor.h"
#include "palial_entry.h"
#ifdef WITH_HOOKS
static FILE *out;
static int nnames, ncpu, ntime;
void palial_set_task_name(const char *name) { fprintf(out, "N %s\n", name); nnames++; }
void palial_set_task_cpu_node(int cpu, int node, char *name) { fprintf(out, "C %d %d %s\n", cpu, node, name); ncpu++; }
void palial_get_task_time(struct timeval s, struct timeval e, char *name)
{
    long long a = (long long)s.tv_sec * 1000000 + s.tv_usec, b = (long long)e.tv_sec * 1000000 + e.tv_usec;
    fprintf(out, "T %lld %lld %s\n", a, b, name);
    ntime++;
}
#endif
int main(int argc, char **argv)
{
    int n = 2048, nb = 512;
    MATRIX_desc A = palial_matrix_desc_init(nb, (long)n * n, (long)nb * nb, n);
    A.matrix = malloc(sizeof(double) * n * n);
    palial_opts_default(&palial_entry_opts);
    palial_entry_opts.trace = 1;
    palial_entry_opts.block = nb;
    if (palial_gpu_generate(1, 0, (const palial_desc *)&A)) return 2;
#ifdef WITH_HOOKS
    out = fopen(argv[1], "w");
#endif
    cholesky(A);
#ifdef WITH_HOOKS
    fclose(out);
    printf("%d %d %d %d\n", palial_entry_status.code, nnames, ncpu, ntime);
#else
    printf("%d\n", palial_entry_status.code);
#endif
    free(A.matrix);
    (void)argc; (void)argv;
    return 0;
}
"""


def _compile_hook_prog(tmp_path, with_hooks):
    src = tmp_path / "hooks.c"
    src.write_text(HOOK_PROG)
    exe = tmp_path / ("with_hooks" if with_hooks else "no_hooks")
    libdir = os.path.dirname(P.LIB_PATH)
    cmd = ["gcc", "-O1", "-std=gnu11", "-Wall", "-Werror", f"-I{INC}", str(src), "-o", str(exe), f"-L{libdir}",
           "-lpalial_gpu", f"-Wl,-rpath,{libdir}"] + (["-DWITH_HOOKS"] if with_hooks else [])
    subprocess.run(cmd, check=True)
    return exe


@pytest.mark.parametrize("with_hooks", [False, True])
def test_entry_header_compiles_with_and_without_hooks(tmp_path, with_hooks):
    assert _compile_hook_prog(tmp_path, with_hooks).exists()


@pytest.mark.gpu
def test_entry_hooks_receive_every_task(tmp_path):
    exe = _compile_hook_prog(tmp_path, True)
    log = tmp_path / "hooks.log"
    out = subprocess.run([str(exe), str(log)], capture_output=True, text=True, check=True, timeout=300)
    code, nn, nc, nt = map(int, out.stdout.split())
    mt = 4
    ntasks = mt + 2 * (mt * (mt - 1) // 2) + mt * (mt - 1) * (mt - 2) // 6
    assert code == 0 and nn == nc == nt == ntasks
    lines = log.read_text().splitlines()
    names = [ln.split()[1] for ln in lines if ln.startswith("N ")]
    need = P.lib().palial_dag_names
    need.restype = ctypes.c_longlong
    need.argtypes = [ctypes.c_int] * 4 + [ctypes.c_char_p, ctypes.c_longlong]
    buf = ctypes.create_string_buffer(4096)
    need(0, 2048, 512, 512, buf, 4096)
    assert names == buf.value.decode().split()
    sms = {int(ln.split()[1]) for ln in lines if ln.startswith("C ")}
    assert all(0 <= s < 1024 for s in sms) and {int(ln.split()[2]) for ln in lines if ln.startswith("C ")} == {0}
    for ln in lines:
        if ln.startswith("T "):
            _, a, b, _ = ln.split()
            assert int(b) >= int(a) > 1_600_000_000_000_000  # microseconds since the epoch
