"""GPU parity of the FP64 / FP32 factor-and-solve path against the oracle and
the reference's golden fixtures.

Bar: pivot sequences identical to the reference's (swap destinations,
0-based) except at steps where the reference's candidates are tied within a
few ulps; factors and solutions within RTOL of the reference's; normwise
backward error within 4 n eps64 of the reference's."""
import glob
import os

import numpy as np
import pytest
import torch

from elemental_gb300 import device as D
from elemental_gb300 import matrices as mats
from oracle import oracle as O

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps
RTOL64 = 1e-10
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def dev(a, dtype=torch.float64):
    return D.to_colmajor(torch.from_numpy(np.ascontiguousarray(np.asfortranarray(a).T)).t()
                         .to(dtype).cuda())


def host(t):
    return t.double().cpu().numpy()


def assert_pivots(piv_gpu, piv_ref, A, nb):
    piv_gpu = np.asarray(piv_gpu).ravel()
    piv_ref = np.asarray(piv_ref).ravel()
    bad = np.nonzero(piv_gpu != piv_ref)[0]
    if bad.size:
        ties = set(O.tied_pivot_steps(A, piv_ref, nb=nb, ulps=8))
        assert set(bad.tolist()) <= ties, f"pivot mismatch at {bad[:10]} (ties {sorted(ties)[:10]})"


def gpu_lu(ctx, A, nb, dtype=torch.float64):
    dA = dev(A, dtype)
    piv = ctx.lu(dA, nb=nb)
    info, err = ctx.status()
    assert err == 0
    return host(dA), piv.cpu().numpy(), info


@pytest.mark.parametrize("m,n,nb", [(1, 1, 128), (2, 2, 128), (31, 31, 32), (32, 32, 32),
                                    (33, 33, 32), (100, 100, 96), (129, 129, 32),
                                    (150, 100, 32), (100, 150, 32), (257, 257, 64),
                                    (300, 300, 128), (520, 520, 128), (1000, 700, 128),
                                    (1002, 517, 64), (2100, 2100, 1024)])
def test_lu_matches_oracle(ctx, m, n, nb):
    A = mats.gaussian(m, n, 7 * m + n)
    LU, piv, info = gpu_lu(ctx, A, nb)
    assert info == 0
    LUr, pivr = O.lu(A, nb=nb)
    assert_pivots(piv, pivr, A, nb)
    assert np.abs(LU - LUr).max() <= RTOL64 * max(1.0, np.abs(LUr).max())


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "lu_*.npz"))),
                         ids=lambda p: os.path.basename(p)[:-4])
def test_lu_matches_reference_fixture(ctx, path):
    g = np.load(path)
    nb = int(g["nb"])
    dt = torch.float32 if str(g["dtype"]) == "float32" else torch.float64
    LU, piv, info = gpu_lu(ctx, g["A"], nb, dt)
    if int(g["status"]) != 0:
        assert info > 0  # SingularMatrixException in the reference
        return
    assert info == 0
    assert_pivots(piv, g["piv"], g["A"], nb)
    tol = 2e-4 if dt == torch.float32 else RTOL64
    assert np.abs(LU - g["LU"]).max() <= tol * max(1.0, np.abs(g["LU"]).max())


def test_lu_singular_reports_first_zero_pivot(ctx):
    A = mats.gaussian(64, 64, 3)
    A[:, 40] = 0.0
    _, _, info = gpu_lu(ctx, A, 32)
    assert info == 41


def test_config1_parity_and_backward_error(ctx):
    """Config 1: n = 1024, 1 RHS, iid N(0,1), default blocksize 128."""
    g = np.load(os.path.join(GOLD, "cfg1_lusolve_1024_nb128.npz"))
    n = int(g["n"])
    A = mats.gaussian(n, n, int(g["seed_A"]))
    b = mats.gaussian(n, 1, int(g["seed_b"]))
    dA, db = dev(A), dev(b)
    piv = ctx.lu(dA, nb=128)
    ctx.lu_solve_after(dA, piv, db)
    ctx.check()
    assert_pivots(piv.cpu().numpy(), g["piv"], A, 128)
    X = host(db)
    berr = O.backward_error(A, X, b)
    assert berr <= float(g["berr"]) + 4 * n * EPS
    # the device-side metric agrees with the host one
    dA0 = dev(A)
    berr_dev = ctx.backward_error(dA0, db, dev(b))
    assert abs(berr_dev - berr) <= 1e-3 * berr + 1e-18


@pytest.mark.parametrize("orient", [0, 1])
@pytest.mark.parametrize("n,q,nb", [(120, 3, 32), (300, 1, 128), (513, 16, 128), (200, 17, 64)])
def test_lu_solve_after(ctx, orient, n, q, nb):
    A = mats.gaussian(n, n, n + q)
    B = mats.gaussian(n, q, n + q + 1)
    dA = dev(A)
    piv = ctx.lu(dA, nb=nb)
    dB = dev(B)
    ctx.lu_solve_after(dA, piv, dB, orient)
    ctx.check()
    LUr, pivr = O.lu(A, nb=nb)
    Xr = O.lu_solve_after(LUr, pivr, B, orient)
    X = host(dB)
    Aop = A if orient == 0 else A.T
    assert O.backward_error(Aop, X, B) <= O.backward_error(Aop, Xr, B) + 4 * n * EPS
    assert np.abs(X - Xr).max() <= 1e-8 * max(1.0, np.abs(Xr).max())


@pytest.mark.parametrize("uplo", [0, 1])
@pytest.mark.parametrize("n,nb", [(1, 128), (100, 96), (257, 64), (400, 128)])
def test_cholesky_matches_oracle(ctx, uplo, n, nb):
    A = mats.spd(n, 11 * n)
    dA = dev(A)
    ctx.cholesky(dA, uplo=uplo, nb=nb)
    ctx.check(cholesky=True)
    C = host(dA)
    Cr = O.cholesky(A, "U" if uplo else "L", nb=nb)
    tri = np.triu if uplo else np.tril
    assert np.abs(tri(C) - tri(Cr)).max() <= RTOL64 * np.abs(Cr).max()
    # the other triangle is untouched
    other = np.tril(A, -1) if uplo else np.triu(A, 1)
    assert np.array_equal(np.tril(C, -1) if uplo else np.triu(C, 1), other)


@pytest.mark.parametrize("path", sorted(p for p in glob.glob(os.path.join(GOLD, "chol*.npz"))
                                        if not os.path.basename(p).startswith("cholpiv")) +
                         glob.glob(os.path.join(GOLD, "hpdsolve*.npz")),
                         ids=lambda p: os.path.basename(p)[:-4])
def test_cholesky_fixtures(ctx, path):
    g = np.load(path)
    uplo = 1 if str(g["uplo"]) == "U" else 0
    nb = int(g["nb"])
    op = str(g["op"])
    dA = dev(g["A"])
    if op == "hpdsolve":
        dB = dev(g["B"])
        ctx.hpd_solve(dA, dB, uplo=uplo, nb=nb)
        ctx.check(cholesky=True)
        assert np.abs(host(dB) - g["X"]).max() <= 1e-9 * max(1, np.abs(g["X"]).max())
        return
    ctx.cholesky(dA, uplo=uplo, nb=nb)
    info, err = ctx.status()
    if int(g["status"]) != 0:
        assert info > 0  # NonHPDMatrixException in the reference
        return
    assert info == 0 and err == 0
    tri = np.triu if uplo else np.tril
    C = host(dA)
    assert np.abs(tri(C) - tri(g["C"])).max() <= RTOL64 * np.abs(g["C"]).max()
    if op == "cholsolve":
        dB = dev(g["B"])
        ctx.cholesky_solve_after(dA, dB, uplo=uplo)
        ctx.check()
        assert np.abs(host(dB) - g["X"]).max() <= 1e-9 * max(1, np.abs(g["X"]).max())


@pytest.mark.parametrize("n,q,nb", [(120, 5, 32), (333, 16, 128), (700, 2, 128)])
def test_linear_solve(ctx, n, q, nb):
    A = mats.gaussian(n, n, 5 * n)
    B = mats.gaussian(n, q, 5 * n + 1)
    dA = dev(A)
    dB = dev(B)
    ctx.linear_solve(dA, dB, nb=nb)
    ctx.check()
    assert np.array_equal(host(dA), A)  # A is left untouched (the reference copies it)
    Xr = O.linear_solve(A, B, nb=nb)
    X = host(dB)
    assert np.abs(X - Xr).max() <= 1e-8 * max(1.0, np.abs(Xr).max())
    assert O.backward_error(A, X, B) <= O.backward_error(A, Xr, B) + 4 * n * EPS


def test_linear_solve_fixture(ctx):
    g = np.load(os.path.join(GOLD, "linsolve_120_nb32.npz"))
    dB = dev(g["B"])
    ctx.linear_solve(dev(g["A"]), dB, nb=int(g["nb"]))
    ctx.check()
    assert np.abs(host(dB) - g["X"]).max() <= 1e-9 * max(1, np.abs(g["X"]).max())


@pytest.mark.parametrize("n", [1, 1024])
def test_float32_path(ctx, n):
    A = mats.gaussian(n, n, 99 + n)
    B = mats.gaussian(n, 2, 98 + n)
    dA = dev(A, torch.float32)
    piv = ctx.lu(dA)
    dB = dev(B, torch.float32)
    ctx.lu_solve_after(dA, piv, dB)
    ctx.check()
    LUr, pivr = O.lu(A.astype(np.float32), dtype=np.float32)
    mism = int(np.sum(piv.cpu().numpy() != pivr))
    assert mism <= max(2, n // 100)
    assert O.backward_error(A, host(dB), B) < 1e-5


def test_edge_empty_and_zero_rhs(ctx):
    dA = D.colmajor(0, 0)
    piv = ctx.lu(dA)
    assert piv.numel() == 0
    A = mats.gaussian(50, 50, 1)
    dA = dev(A)
    piv = ctx.lu(dA)
    dB = D.colmajor(50, 0)
    ctx.lu_solve_after(dA, piv, dB)
    ctx.check()


def test_nan_input_does_not_hang(ctx):
    A = mats.gaussian(80, 80, 2)
    A[5, 3] = np.nan
    dA = dev(A)
    ctx.lu(dA, nb=32)
    info, err = ctx.status()
    assert err == 0
