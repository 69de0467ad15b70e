"""The blocked Householder algorithm of the mixed-precision QR's tile kernels (tile_qr.cuh:
64-column panels factored column by column, the trailing columns updated by the panel's block
reflector, the full compact-WY T assembled from the panel T's) restated in numpy (FP64) and
checked against the oracle's unblocked GEQRT / TSQRT (the reference's dgeqr2 + dlarft and
TS kernel): the same R, V and T up to rounding."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O

def larfg(alpha, x):
    xn = np.linalg.norm(x)
    if xn == 0: return 0.0, alpha, x
    beta = -np.copysign(np.hypot(alpha, xn), alpha)
    tau = (beta - alpha) / beta
    return tau, beta, x / (alpha - beta)

def larft(tau, dot, nbp):
    T = np.zeros((nbp, nbp))
    for i in range(nbp):
        z = np.array([-tau[i] * dot(j, i) for j in range(i)])
        for r in range(i):
            T[r, i] = sum(T[r, p] * z[p] for p in range(r, i))
        T[i, i] = tau[i]
    return T

def assemble(T, nb, ytq):
    for q0 in range(64, nb, 64):
        Y = ytq(q0)
        Y2 = Y @ np.triu(T[q0:q0+64, q0:q0+64])
        T[:q0, q0:q0+64] = -np.triu(T[:q0, :q0]) @ Y2
    return T

def geqrt_blocked(A):
    A = A.copy(); nb = A.shape[0]; tau = np.zeros(nb); T = np.zeros((nb, nb))
    for p0 in range(0, nb, 64):
        for i in range(p0, p0 + 64):
            t, beta, v = larfg(A[i, i], A[i+1:, i])
            A[i, i] = beta; A[i+1:, i] = v; tau[i] = t
            if t != 0:
                for j in range(i + 1, p0 + 64):
                    s = A[i, j] + A[i+1:, i] @ A[i+1:, j]
                    f = -t * s
                    A[i, j] += f; A[i+1:, j] += f * A[i+1:, i]
        def dot(j, i):
            cj, ci = A[:, p0+j], A[:, p0+i]
            return cj[p0+i] + cj[p0+i+1:] @ ci[p0+i+1:]
        T[p0:p0+64, p0:p0+64] = larft(tau[p0:p0+64], dot, 64)
        nc = nb - p0 - 64
        if nc > 0:
            V = np.tril(A[p0:, p0:p0+64], -1); V[np.arange(64), np.arange(64)] = 1.0
            C = A[p0:, p0+64:]
            W = V.T @ C
            W2 = np.triu(T[p0:p0+64, p0:p0+64]).T @ W
            A[p0:, p0+64:] = C - V @ W2
    def ytq(q0):
        Va = A[q0:, :q0]
        VQ = np.tril(A[q0:, q0:q0+64], -1); VQ[np.arange(64), np.arange(64)] = 1.0
        return Va.T @ VQ
    return A, assemble(T, nb, ytq)

def tsqrt_blocked(A1, A2):
    A1 = A1.copy(); A2 = A2.copy(); nb = A1.shape[0]; tau = np.zeros(nb); T = np.zeros((nb, nb))
    for p0 in range(0, nb, 64):
        for i in range(p0, p0 + 64):
            t, beta, v = larfg(A1[i, i], A2[:, i])
            A1[i, i] = beta; A2[:, i] = v; tau[i] = t
            if t != 0:
                for j in range(i + 1, p0 + 64):
                    s = A1[i, j] + A2[:, i] @ A2[:, j]
                    f = -t * s
                    A1[i, j] += f; A2[:, j] += f * A2[:, i]
        T[p0:p0+64, p0:p0+64] = larft(tau[p0:p0+64], lambda j, i: A2[:, p0+j] @ A2[:, p0+i], 64)
        nc = nb - p0 - 64
        if nc > 0:
            V = A2[:, p0:p0+64]
            W = A1[p0:p0+64, p0+64:] + V.T @ A2[:, p0+64:]
            W2 = np.triu(T[p0:p0+64, p0:p0+64]).T @ W
            A1[p0:p0+64, p0+64:] -= W2
            A2[:, p0+64:] -= V @ W2
    return A1, A2, assemble(T, nb, lambda q0: A2[:, :q0].T @ A2[:, q0:q0+64])



@pytest.mark.parametrize("nb", [64, 192, 256])
def test_blocked_tile_qr_equals_unblocked_oracle(nb):
    dp = ctypes.POINTER(ctypes.c_double)
    L = O.lib()
    a = O.gen_uniform(9, nb)
    ra, rt, tau, work = np.asfortranarray(a.copy()), np.zeros((nb, nb), order="F"), np.zeros(nb), np.zeros(nb * nb)
    L.orc_dgeqrt(nb, ra.ctypes.data_as(dp), nb, rt.ctypes.data_as(dp), nb, tau.ctypes.data_as(dp),
                 work.ctypes.data_as(dp))
    ga, gt = geqrt_blocked(a)
    assert np.abs(ga - ra).max() <= 1e-12 and np.abs(np.triu(gt) - np.triu(rt)).max() <= 1e-12
    a2 = O.gen_uniform(11, nb)
    r1, r2, t2 = np.asfortranarray(ra.copy()), np.asfortranarray(a2.copy()), np.zeros((nb, nb), order="F")
    L.orc_dtsqrt(nb, r1.ctypes.data_as(dp), nb, r2.ctypes.data_as(dp), nb, t2.ctypes.data_as(dp), nb,
                 tau.ctypes.data_as(dp), work.ctypes.data_as(dp))
    b1, b2, bt = tsqrt_blocked(ra, a2)
    assert np.abs(np.triu(b1) - np.triu(r1)).max() <= 1e-12 and np.abs(b2 - r2).max() <= 1e-12
    assert np.abs(np.triu(bt) - np.triu(t2)).max() <= 1e-12
