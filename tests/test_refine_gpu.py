"""Mixed-precision LU-IR / GMRES-IR (ir.cu): FP64-level backward error from
tensor-core low-precision factors, the FP64 fallback, and agreement with the
FP64 oracle solution."""
import numpy as np
import pytest
import torch

from elemental_gb300 import device as D
from elemental_gb300 import matrices as mats
from oracle import oracle as O

pytestmark = pytest.mark.gpu
EPS = np.finfo(np.float64).eps


def dev(a):
    return D.to_colmajor(torch.from_numpy(np.ascontiguousarray(np.asfortranarray(a).T)).t().cuda())


@pytest.mark.parametrize("precision", ["fp32", "tf32", "bf16"])
@pytest.mark.parametrize("method", ["lu-ir", "gmres-ir"])
@pytest.mark.parametrize("n,q", [(1024, 1), (1500, 16), (700, 17)])
def test_refined_solve_gaussian(ctx, precision, method, n, q):
    A = mats.gaussian(n, n, 31 * n + q)
    B = mats.gaussian(n, q, 31 * n + q + 1)
    dA, dB = dev(A), dev(B)
    X, info = ctx.refined_solve(dA, dB, precision=precision, method=method)
    Xh = X.cpu().numpy()
    berr = O.backward_error(A, Xh, B)
    assert berr <= n * EPS, (berr, info)
    assert abs(info["backward_error"] - berr) <= 0.05 * berr + 1e-18
    assert np.array_equal(dA.cpu().numpy(), A)  # inputs untouched
    if precision == "fp32":
        assert info["converged"] and not info["fell_back"] and info["iterations"] <= 6
    # the FP64 oracle solution agrees to the conditioning-limited accuracy
    LU, piv = O.lu(A)
    Xr = O.lu_solve_after(LU, piv, B)
    assert np.abs(Xh - Xr).max() <= 1e-8 * max(1.0, np.abs(Xr).max())


@pytest.mark.parametrize("kappa", [1e2, 1e6, 1e10])
@pytest.mark.parametrize("precision,method", [("fp32", "lu-ir"), ("bf16", "gmres-ir"),
                                              ("tf32", "gmres-ir")])
def test_refined_solve_conditioned(ctx, kappa, precision, method):
    n = 512
    A = mats.conditioned(n, kappa, 7)
    B = mats.gaussian(n, 2, 8)
    X, info = ctx.refined_solve(dev(A), dev(B), precision=precision, method=method)
    berr = O.backward_error(A, X.cpu().numpy(), B)
    assert berr <= n * EPS, (kappa, info)


def test_fallback_on_stall(ctx):
    n = 400
    A = mats.conditioned(n, 1e12, 3)
    B = mats.gaussian(n, 1, 4)
    X, info = ctx.refined_solve(dev(A), dev(B), precision="bf16", method="lu-ir", max_iters=3)
    assert info["fell_back"] and info["precision"] == "fp64"
    assert O.backward_error(A, X.cpu().numpy(), B) <= n * EPS


def test_no_fallback_reports_not_converged(ctx):
    n = 400
    A = mats.conditioned(n, 1e12, 3)
    B = mats.gaussian(n, 1, 4)
    X, info = ctx.refined_solve(dev(A), dev(B), precision="bf16", method="lu-ir", max_iters=3,
                                fallback=False)
    assert not info["fell_back"] and not info["converged"]


def test_fp64_precision_is_plain_lu(ctx):
    n = 300
    A = mats.gaussian(n, n, 5)
    B = mats.gaussian(n, 3, 6)
    X, info = ctx.refined_solve(dev(A), dev(B), precision="fp64")
    assert info["iterations"] == 0 and not info["fell_back"]
    LU, piv = O.lu(A)
    assert np.abs(X.cpu().numpy() - O.lu_solve_after(LU, piv, B)).max() < 1e-10


def test_singular_low_precision_factor_falls_back(ctx):
    n = 200
    A = mats.gaussian(n, n, 9)
    A[:, 50] = A[:, 49] * (1 + 1e-12)  # FP32 copy is exactly singular-ish
    B = mats.gaussian(n, 1, 10)
    X, info = ctx.refined_solve(dev(A), dev(B), precision="bf16")
    assert np.isfinite(X.cpu().numpy()).all() or info["fell_back"]
