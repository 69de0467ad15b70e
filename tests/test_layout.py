"""Layout bridges (column-major <-> the reference's tile layout), any-N solves by padding,
and the tiled-matrix file format.  The file format and sizes need no GPU; the conversions and
solves run on the GPU (checked against the oracle's layout helpers and numpy)."""
import os
import struct

import numpy as np
import pytest

import palial_gb300 as P
from oracle import oracle as O


def test_padded_size():
    lib = P.lib()
    assert [lib.palial_gpu_padded_size(n, 256) for n in (1, 255, 256, 257, 1000, 1024)] == [256, 256, 256, 512, 1024,
                                                                                         1024]
    assert lib.palial_gpu_padded_size(0, 256) == 0


def test_tiles_file_roundtrip(tmp_path):
    n, nb = 384, 128
    a = O.gen_uniform(7, n)
    t = O.to_tiles(a, nb)
    f = tmp_path / "a.palt"
    P.tiles_write(str(f), t, n, nb)
    raw = f.read_bytes()
    assert raw[:8] == b"PALTILE1" and struct.unpack("<3q", raw[8:32]) == (n, nb, 0)
    assert len(raw) == 32 + 8 * n * n
    t2, n2, nb2 = P.tiles_read(str(f))
    assert (n2, nb2) == (n, nb) and np.array_equal(t2, t)
    assert np.array_equal(O.from_tiles(t2, n, nb), a)


@pytest.mark.parametrize("payload", [b"", b"PALTILE0" + struct.pack("<3q", 4, 2, 0),
                                     b"PALTILE1" + struct.pack("<3q", 5, 2, 0),
                                     b"PALTILE1" + struct.pack("<3q", 4, 2, 0) + b"\0" * 16])
def test_tiles_file_rejects_bad_files(tmp_path, payload):
    f = tmp_path / "bad.palt"
    f.write_bytes(payload)
    with pytest.raises(P.PalialError):
        P.tiles_read(str(f))


@pytest.mark.gpu
@pytest.mark.parametrize("n,nb", [(512, 128), (1000, 256), (257, 256), (64, 512)])
def test_colmajor_tiles_roundtrip(n, nb):
    import torch
    npad = P.lib().palial_gpu_padded_size(n, nb)
    a = O.gen_uniform(3, n)
    lda = n + 5
    ca = np.zeros((n, lda))  # row-major storage of the column-major lda x n buffer: ca[c, r]
    ca[:, :n] = a.T
    dc = torch.from_numpy(ca.ravel()).cuda()
    dt = torch.zeros(npad * npad, dtype=torch.float64, device="cuda")
    assert P.lib().palial_gpu_colmajor_to_tiles(dc.data_ptr(), lda, n, dt.data_ptr(), npad, nb, 2.5, None) == 0
    ref = np.diag(np.full(npad, 2.5))
    ref[:n, :n] = a
    assert np.array_equal(dt.cpu().numpy(), O.to_tiles(ref, nb))
    back = torch.zeros(n * lda, dtype=torch.float64, device="cuda")
    assert P.lib().palial_gpu_tiles_to_colmajor(dt.data_ptr(), npad, nb, back.data_ptr(), lda, n, None) == 0
    torch.cuda.synchronize()
    assert np.array_equal(back.cpu().numpy().reshape(n, lda)[:, :n].T, a)


@pytest.mark.gpu
@pytest.mark.parametrize("alg,n", [("cholesky", 1000), ("lu", 1000), ("cholesky", 777), ("lu", 1280)])
@pytest.mark.parametrize("precision", ["bf16", "fp64"])
def test_solve_colmajor_any_n(alg, n, precision):
    """Any N through the column-major front end: backward error at the FP64 target."""
    import torch
    nrhs, nb = 3, 256
    if alg == "cholesky":
        k = O.gen_uniform(4, n)
        a = k @ k.T / n + np.eye(n) * 2.0
    else:
        a = O.gen_uniform(5, n) + np.eye(n) * n  # diagonally dominant: no-pivot LU is stable
    b = O.gen_uniform(6, n, nrhs)
    da = torch.from_numpy(np.asfortranarray(a).ravel(order="F")).cuda()
    db = torch.from_numpy(np.asfortranarray(b).ravel(order="F")).cuda()
    dx = torch.zeros(n * nrhs, dtype=torch.float64, device="cuda")
    st = P.solve_colmajor(alg, n, da.data_ptr(), n, db.data_ptr(), n, dx.data_ptr(), n, nrhs, nb=nb,
                          precision=precision)
    assert st.code in (0, 1)
    x = dx.cpu().numpy().reshape(nrhs, n).T
    r = b - a @ x
    eta = (np.abs(r).max(axis=0) / (np.abs(a).sum(axis=1).max() * np.abs(x).max(axis=0) + np.abs(b).max(axis=0))).max()
    assert eta <= 1e-14 * n, eta
    assert np.allclose(x, np.linalg.solve(a, b), rtol=1e-9, atol=1e-12)
