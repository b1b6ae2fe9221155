"""LU with partial pivoting and Cholesky at n = 8192 (FP64, blocksize 128,
16 right-hand sides) against the oracle at full size.  This is the size where
the device factorization runs its look-ahead schedule and several recursion
levels per panel block, which the smaller parity cases do not reach.

Bar: the pivot sequence equal to the oracle's except at steps whose
candidates are tied within a few ulps; when the pivots are equal, the factors
within a relative 1e-8 of the largest entry (two backward-stable orders of
the same elimination); the normwise backward error within 4 n eps64 of the
oracle's.  Cholesky has no pivots: its factor must match to 1e-10 relative
(the matrix G^T G / n + I has condition number below 10).  Measured between
two CPU orders of the same elimination (the oracle's blocked nb = 128 LU and
LAPACK's getrf over OpenBLAS) on this LU input: equal pivots, factors 2.7e-12
apart; Cholesky factors 7.8e-16 apart.

This file is collected last on purpose: the oracle's side takes tens of
seconds on the host, and a failure here leaves every other test already run."""
import os

import numpy as np
import pytest

from elemental_gb300 import matrices as mats
from oracle import oracle as O

pytestmark = pytest.mark.gpu
EPS = np.finfo(np.float64).eps
N, Q, NB = 8192, 16, 128


@pytest.fixture(scope="module")
def ctx():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from elemental_gb300 import device as D

    O.set_threads(os.cpu_count() or 1)
    return D.context(0)


def dev(a):
    import torch

    from elemental_gb300 import device as D

    a = np.asarray(a, dtype=np.float64)
    T = D.colmajor(a.shape[0], a.shape[1])
    T.copy_(torch.from_numpy(np.ascontiguousarray(a)))
    return T


def test_lu_n8192_matches_oracle(ctx):
    A = mats.gaussian(N, N, 88192)
    B = mats.gaussian(N, Q, 88193)
    LUr, pivr = O.lu(A, nb=NB)
    Xr = O.lu_solve_after(LUr, pivr, B)
    dA = dev(A)
    piv = ctx.lu(dA, nb=NB)
    dB = dev(B)
    ctx.lu_solve_after(dA, piv, dB)
    assert ctx.status() == (0, 0)
    p = piv.cpu().numpy()
    bad = np.nonzero(p != pivr)[0]
    if bad.size:
        ties = set(O.tied_pivot_steps(A, pivr, nb=NB, ulps=8))
        assert set(bad.tolist()) <= ties, f"pivot mismatch at {bad[:10]}"
    else:
        LU = dA.cpu().numpy()
        assert np.abs(LU - LUr).max() <= 1e-8 * np.abs(LUr).max()
    X = dB.cpu().numpy()
    assert O.backward_error(A, X, B) <= O.backward_error(A, Xr, B) + 4 * N * EPS


@pytest.mark.parametrize("uplo", [0, 1])
def test_cholesky_n8192_matches_oracle(ctx, uplo):
    A = mats.spd(N, 98192 + uplo)
    B = mats.gaussian(N, Q, 98194)
    u = "U" if uplo else "L"
    Cr = O.cholesky(A, u, nb=NB)
    Xr = O.cholesky_solve_after(Cr, B, u)
    dA = dev(A)
    ctx.cholesky(dA, uplo=uplo, nb=NB)
    dB = dev(B)
    ctx.cholesky_solve_after(dA, dB, uplo=uplo)
    assert ctx.status() == (0, 0)
    tri = np.triu if uplo else np.tril
    C = dA.cpu().numpy()
    assert np.abs(tri(C) - tri(Cr)).max() <= 1e-10 * np.abs(Cr).max()
    X = dB.cpu().numpy()
    assert O.backward_error(A, X, B) <= O.backward_error(A, Xr, B) + 4 * N * EPS
