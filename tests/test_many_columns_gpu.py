"""More than 65535 columns in one call: the element-wise kernels that take
one column per grid.y index loop over the columns, so a SolveAfter or a
refined solve with 70000 right-hand sides and a tensor-core update with
70000 columns of B run and give the oracle's results.  (The reference's
lu::SolveAfter, src/lapack_like/factor/LU/SolveAfter.hpp:66-92, takes any
number of right-hand sides.)"""
import numpy as np
import pytest
import torch

from elemental_gb300 import device as D
from elemental_gb300 import matrices as mats
from oracle import oracle as O

pytestmark = pytest.mark.gpu

NRHS = 70000
EPS = np.finfo(np.float64).eps


def dev(a, dtype=torch.float64):
    return D.to_colmajor(torch.from_numpy(np.ascontiguousarray(np.asfortranarray(a).T)).t()
                         .to(dtype).cuda())


def host(t):
    return t.double().cpu().numpy()


@pytest.mark.parametrize("orientation", [0, 1])
def test_solve_after_with_70000_rhs_matches_oracle(ctx, orientation):
    n = 64
    A = mats.gaussian(n, n, 4101)
    B = mats.gaussian(n, NRHS, 4102)
    dA = dev(A)
    piv = ctx.lu(dA, nb=32)
    dB = dev(B)
    ctx.lu_solve_after(dA, piv, dB, orientation=orientation)
    ctx.check()
    LUr, pivr = O.lu(A, nb=32)
    assert np.array_equal(piv.cpu().numpy(), pivr)
    Xr = O.lu_solve_after(LUr, pivr, B, orientation)
    X = host(dB)
    assert np.all(np.isfinite(X))
    # same factors (to rounding), same substitutions: the solutions agree to
    # a small multiple of the conditioning times eps
    scale = np.abs(Xr).max(axis=0)
    assert np.max(np.abs(X - Xr).max(axis=0) / scale) < 1e-10
    Aop = A if orientation == 0 else A.T
    assert O.backward_error(Aop, X, B) <= 4 * n * EPS


def test_refined_solve_with_70000_rhs(ctx):
    n = 64
    A = mats.gaussian(n, n, 4201)
    B = mats.gaussian(n, NRHS, 4202)
    dA, dB = dev(A), dev(B)
    X, info = ctx.refined_solve(dA, dB, precision="fp32")
    ctx.check()
    assert info["converged"]
    Xh = host(X)
    assert O.backward_error(A, Xh, B) <= n * EPS
    # the inputs are untouched
    assert np.array_equal(host(dA), A) and np.array_equal(host(dB), B)


@pytest.mark.parametrize("kind", [1, 2])
def test_tensor_core_update_with_70000_columns(ctx, kind):
    """C -= A B with B 32 x 70000 (its packing kernel takes one column of B
    per grid.y index), checked against an FP64 product of the same
    TF32-rounded (kind 1) or TF32x3 (kind 2, ~FP32-exact) operands."""
    m, k = 128, 32
    rng = np.random.default_rng(4301)
    A = rng.standard_normal((m, k)).astype(np.float32)
    Bm = rng.standard_normal((k, NRHS)).astype(np.float32)
    C = rng.standard_normal((m, NRHS)).astype(np.float32)
    dA, dBm, dC = dev(A, torch.float32), dev(Bm, torch.float32), dev(C, torch.float32)
    ctx.gemm_sub_tc(dA, dBm, dC, gemm_kind=kind)
    ctx.check()
    ref = C.astype(np.float64) - A.astype(np.float64) @ Bm.astype(np.float64)
    err = np.abs(host(dC) - ref).max() / (np.abs(A).max() * np.abs(Bm).max() * k)
    assert err < (2e-3 if kind == 1 else 1e-5), err
