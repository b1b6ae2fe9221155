"""Tournament pivoting (CALU) in the FP32 preconditioner LU (calu.cu): a
valid pivoted factorization of the same quality as partial pivoting, and
refinement to the FP64 target with it."""
import numpy as np
import pytest
import torch

from elemental_gb300 import device as D
from elemental_gb300 import matrices as mats

pytestmark = pytest.mark.gpu


def cm(a):
    return D.to_colmajor(torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.float32).T)).t()
                         .cuda())


def factor(ctx, A, tournament, nb=128, kind=2):
    ctx.set_option("tournament", 1 if tournament else 0)
    try:
        dA = cm(A)
        piv = ctx.lu_mixed(dA, gemm_kind=kind, nb=nb).cpu().numpy()
        info, err = ctx.status()
    finally:
        ctx.set_option("tournament", 0)
    assert err == 0 and info == 0
    return dA.cpu().double().numpy(), piv


def residual(A, LU, piv):
    n = A.shape[0]
    L = np.tril(LU, -1) + np.eye(n)
    U = np.triu(LU)
    PA = A.astype(np.float64).copy()
    for i, p in enumerate(piv):
        assert i <= p < n
        PA[[i, p]] = PA[[p, i]]
    return np.linalg.norm(PA - L @ U) / np.linalg.norm(A), np.abs(np.tril(LU, -1)).max()


@pytest.mark.parametrize("n,nb", [(100, 32), (1000, 128), (2500, 256), (4096, 512)])
def test_tournament_lu_is_a_valid_pivoted_factorization(ctx, n, nb):
    A = mats.gaussian(n, n, 300 + n).astype(np.float32)
    LU_t, piv_t = factor(ctx, A, True, nb)
    LU_p, piv_p = factor(ctx, A, False, nb)
    rt, lt = residual(A, LU_t, piv_t)
    rp, lp = residual(A, LU_p, piv_p)
    assert lp <= 1.0 + 1e-6
    # tournament multipliers are not bounded by 1 (a model of the same
    # per-panel tournament in FP64 numpy reaches |l| ~ 70 at n = 1000 too);
    # what matters is the factorization's residual
    assert lt < 1e3, lt
    assert rt < 50 * rp + 1e-6, (rt, rp)
    assert np.all(np.isfinite(LU_t))


def test_tournament_singular_column_reports_info(ctx):
    n = 200
    A = mats.gaussian(n, n, 7).astype(np.float32)
    A[:, 50] = 0.0
    ctx.set_option("tournament", 1)
    try:
        dA = cm(A)
        ctx.lu_mixed(dA, gemm_kind=2, nb=64)
        info, err = ctx.status()
    finally:
        ctx.set_option("tournament", 0)
    assert err == 0 and info == 51


@pytest.mark.parametrize("method", ["lu-ir", "gmres-ir"])
def test_refined_solve_with_tournament_pivoting(ctx, method):
    n = 3000
    A = mats.gaussian(n, n, 11)
    B = mats.gaussian(n, 4, 12)
    dA = D.to_colmajor(torch.from_numpy(A).cuda())
    dB = D.to_colmajor(torch.from_numpy(B).cuda())
    X, info = ctx.refined_solve(dA, dB, precision="fp32", method=method, pivoting="tournament")
    assert info["converged"] and not info["fell_back"], info
    Xh = X.cpu().numpy()
    for c in range(4):
        be = np.linalg.norm(B[:, c] - A @ Xh[:, c]) / (
            np.linalg.norm(A) * np.linalg.norm(Xh[:, c]) + np.linalg.norm(B[:, c]))
        assert be <= n * 2.0 ** -53
