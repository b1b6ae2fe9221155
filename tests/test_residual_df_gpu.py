"""The double-float residual (ElGBResidualDF_d, residual_df.cu): R = B - A X
to FP64 accuracy on the FP32 pipe, against a correctly rounded host
residual (exact products by Dekker's split, then math.fsum per row), and the
mixed-precision solve that uses it by default, against the same solve with
FP64 residuals.  The residual is the one of the refinement loop of the
reference's refined_solve (include/El/lapack_like/solve/Refined.hpp:70-73)."""
import math

import numpy as np
import pytest
import torch

from elemental_gb300 import device as D
from elemental_gb300 import matrices as mats
from oracle import oracle as O

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps


def dev(a):
    return D.to_colmajor(torch.from_numpy(np.ascontiguousarray(np.asfortranarray(a).T)).t()
                         .cuda())


def _veltkamp(a):
    c = 134217729.0 * a  # 2^27 + 1
    hi = c - (c - a)
    return hi, a - hi


def exact_residual_rows(A, X, B, rows):
    """Correctly rounded b_i - sum_j a_ij x_jc for the given rows: every
    product a_ij x_jc = p + e exactly (Dekker), then math.fsum."""
    out = np.empty((len(rows), X.shape[1]))
    for k, i in enumerate(rows):
        a = A[i]
        ah, al = _veltkamp(a)
        for c in range(X.shape[1]):
            x = X[:, c]
            xh, xl = _veltkamp(x)
            p = a * x
            e = ((ah * xh - p) + ah * xl + al * xh) + al * xl
            out[k, c] = math.fsum(np.concatenate(([B[i, c]], -p, -e)))
    return out


@pytest.mark.parametrize("n,q", [(1024, 1), (1024, 16), (4096, 16), (4097, 3), (8192, 1),
                                 (8192, 16), (100, 20)])
def test_df_residual_is_correctly_rounded_to_a_few_ulps(ctx, n, q):
    rng = np.random.default_rng(n + 7 * q)
    A = rng.standard_normal((n, n))
    # a near-solution, so that the residual cancels as in refinement
    Xt = rng.standard_normal((n, q))
    B = A @ Xt
    X = Xt + 1e-9 * rng.standard_normal((n, q))
    R = ctx.residual_df(dev(A), dev(X), dev(B))
    ctx.check()
    Rg = R.cpu().numpy()
    rows = np.unique(np.concatenate([np.arange(min(n, 8)), rng.integers(0, n, 56)]))
    Rex = exact_residual_rows(A, X, B, rows)
    scale = np.abs(A[rows]) @ np.abs(X) + np.abs(B[rows])
    err = np.abs(Rg[rows] - Rex) / scale
    # the scheme's bound: its low word's FP32 rounding, ~2^-48 sqrt(128 / n)
    # of the row's scale (measured at most 6 ulps by a bit-faithful CPU
    # emulation of the same arithmetic at n <= 4096)
    bound = (16 if n >= 1024 else 32) * EPS
    assert err.max() <= bound, err.max()
    # normwise, in the units of the backward error ||r|| / (||A||_F ||x|| +
    # ||b||), the row bound carries over (||(|A||x| + |b|)|| <= ||A||_F ||x||
    # + ||b||)
    den = np.linalg.norm(A[rows]) * np.linalg.norm(X) + np.linalg.norm(B[rows])
    nw = np.linalg.norm(Rg[rows] - Rex) / den
    assert nw <= bound, nw


def test_df_product_without_b_and_extreme_scaling(ctx):
    """R = A X (no B) with X scaled by 2^+-200 per column: the per-column
    power-of-two scaling keeps every product in FP32 range."""
    n = 2048
    rng = np.random.default_rng(5)
    A = rng.standard_normal((n, n)) * 1e3
    X = rng.standard_normal((n, 4)) * np.array([2.0 ** 200, 2.0 ** -200, 1.0, 1e-30])
    R = ctx.residual_df(dev(A), dev(X)).cpu().numpy()
    assert np.all(np.isfinite(R))
    rows = np.arange(0, n, 97)
    Rex = -exact_residual_rows(A, X, np.zeros((n, 4)), rows)
    scale = np.abs(A[rows]) @ np.abs(X)
    assert np.all(np.abs(R[rows] - Rex) <= 16 * EPS * scale)


def test_df_split_of_entries_across_exponents(ctx):
    """Entries from 2^-90 to 2^40 (with exact zeros): the split of A takes
    its integer path for |a| in [2^-74, 2^127) and FP64 conversions for the
    rest; both must give the words of cvt.rn.f32.f64."""
    n = 1536
    rng = np.random.default_rng(8)
    A = rng.standard_normal((n, n)) * np.exp2(rng.integers(-90, 41, (n, n)))
    A[rng.random((n, n)) < 0.01] = 0.0
    X = rng.standard_normal((n, 3))
    B = A @ X
    R = ctx.residual_df(dev(A), dev(X), dev(B)).cpu().numpy()
    rows = np.arange(0, n, 61)
    Rex = exact_residual_rows(A, X, B, rows)
    scale = np.abs(A[rows]) @ np.abs(X) + np.abs(B[rows])
    assert np.all(np.abs(R[rows] - Rex) <= 16 * EPS * scale)


def test_df_residual_falls_back_for_entries_outside_fp32_range(ctx):
    n = 512
    rng = np.random.default_rng(6)
    A = rng.standard_normal((n, n)) * 1e200
    X = rng.standard_normal((n, 2))
    B = rng.standard_normal((n, 2)) * 1e200
    R = ctx.residual_df(dev(A), dev(X), dev(B)).cpu().numpy()
    ref = B - A @ X
    scale = np.abs(A) @ np.abs(X) + np.abs(B)
    assert np.all(np.abs(R - ref) <= 4 * n * EPS * scale)


@pytest.mark.parametrize("method", ["lu-ir", "gmres-ir"])
@pytest.mark.parametrize("n,q,kappa", [(2048, 16, 0.0), (3000, 1, 0.0), (2048, 4, 1e6)])
def test_refined_solve_with_df_residual_matches_fp64_residual(ctx, method, n, q, kappa):
    if kappa:
        A = mats.conditioned(n, kappa, 91)
    else:
        A = mats.gaussian(n, n, 91)
    B = mats.gaussian(n, q, 92)
    dA, dB = dev(A), dev(B)
    out = {}
    for df in (1, 0):
        ctx.set_option("residual_df", df)
        try:
            X, info = ctx.refined_solve(dA, dB, precision="fp32", method=method)
        finally:
            ctx.set_option("residual_df", 1)
        ctx.check()
        out[df] = (X.cpu().numpy(), info)
    for df, (X, info) in out.items():
        assert info["converged"], (df, info)
        assert O.backward_error(A, X, B) <= n * EPS, (df, info)
    # the two residuals agree to FP64 level, so refinement takes the same path
    assert abs(out[1][1]["iterations"] - out[0][1]["iterations"]) <= 1
