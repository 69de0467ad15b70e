"""The allocation-free TSMQR entry point against the allocating one.

palial_gpu_tile_dtsmqr_noalloc serves callers that may not allocate device memory (an
application that owns all device memory, or code that must avoid cudaMalloc/cudaFree and
their device-wide synchronization): it keeps its scratch in a fixed array inside the
library.  Two calls in a row, on different tiles and tile sizes, must each give what
palial_gpu_tile_dtsmqr gives on the same inputs (normwise 1e-12, the tolerance of the other
tile-kernel tests).  The file is named to be collected last.
"""
import numpy as np
import pytest

import palial_gb300 as P
from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _dev(x):
    return torch.from_numpy(np.asfortranarray(x).ravel(order="F").copy()).cuda()


def _inputs(nb, seed):
    v = O.gen_uniform(seed, nb)
    t = np.triu(O.gen_uniform(seed + 1, nb)) / nb
    a1 = O.gen_uniform(seed + 2, nb)
    a2 = O.gen_uniform(seed + 3, nb)
    return v, t, a1, a2


def _rel(a, b):
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


def test_noalloc_tsmqr_matches_allocating_entry_point():
    lib = P.lib()
    for nb, seed in ((512, 100), (256, 200)):
        v, t, a1, a2 = _inputs(nb, seed)
        dv, dt = _dev(v), _dev(t)
        r1, r2 = _dev(a1), _dev(a2)
        assert lib.palial_gpu_tile_dtsmqr(nb, r1.data_ptr(), r2.data_ptr(), dv.data_ptr(), dt.data_ptr(), nb) == 0
        n1, n2 = _dev(a1), _dev(a2)
        stream = torch.cuda.current_stream().cuda_stream
        rc = lib.palial_gpu_tile_dtsmqr_noalloc(nb, n1.data_ptr(), n2.data_ptr(), dv.data_ptr(), dt.data_ptr(),
                                                nb, stream)
        assert rc == 0
        torch.cuda.synchronize()
        assert _rel(n1, r1) <= 1e-12 and _rel(n2, r2) <= 1e-12, nb


def test_noalloc_call_allocates_no_device_memory():
    """After a warm-up call, further calls leave the device's free memory unchanged."""
    lib = P.lib()
    nb = 512
    v, t, a1, a2 = _inputs(nb, 300)
    dv, dt, n1, n2 = _dev(v), _dev(t), _dev(a1), _dev(a2)
    args = (nb, n1.data_ptr(), n2.data_ptr(), dv.data_ptr(), dt.data_ptr(), nb, None)
    assert lib.palial_gpu_tile_dtsmqr_noalloc(*args) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert lib.palial_gpu_tile_dtsmqr_noalloc(*args) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_rejects_tiles_beyond_its_scratch():
    d = torch.zeros(1024 * 1024, dtype=torch.float64, device="cuda")
    p = d.data_ptr()
    assert P.lib().palial_gpu_tile_dtsmqr_noalloc(1024, p, p, p, p, 1024, None) == -1
