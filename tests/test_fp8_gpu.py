"""FP8 (E4M3) tensor-core updates with per-panel power-of-two scales
(tc_gemm.cu kind kTcFP8) and the FP8 factorization under refinement.

The reference's own arithmetic has no FP8; the contract checked here is the
one the path states: operands scaled by 2^e with max|x| 2^e <= 448, rounded
to E4M3 (round to nearest even, saturating), products accumulated in FP32,
the scales divided out -- against an FP64 model of exactly that."""
import numpy as np
import pytest
import torch

from elemental_gb300 import device as D
from elemental_gb300 import matrices as mats

pytestmark = pytest.mark.gpu


def e4m3(x):
    """Round to E4M3: 3 explicit mantissa bits, exponent bias 7, normals down
    to 2^-6, subnormal step 2^-9, finite maximum 448 (saturating)."""
    x = np.asarray(x, dtype=np.float64)
    a = np.abs(x)
    e = np.floor(np.log2(np.where(a > 0, a, 1.0)))
    e = np.maximum(e, -6.0)
    step = np.exp2(e - 3.0)
    q = np.round(a / step) * step  # numpy rounds halves to even
    q = np.minimum(q, 448.0)
    return np.sign(x) * np.where(a > 0, q, 0.0)


def pow2_scale(amax):
    if amax <= 0:
        return 1.0
    return float(np.exp2(np.floor(np.log2(448.0 / amax))))


def cm(a):
    return D.to_colmajor(torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.float32).T)).t()
                         .cuda())


def test_e4m3_model():
    assert e4m3(448.0) == 448.0 and e4m3(1000.0) == 448.0
    assert e4m3(1.0625) == 1.0 and e4m3(1.1875) == 1.25   # ties to even
    assert e4m3(2.0 ** -9) == 2.0 ** -9 and e4m3(2.0 ** -11) == 0.0


@pytest.mark.parametrize("m,n,k", [(128, 256, 64), (300, 500, 200), (1000, 777, 512)])
def test_fp8_gemm_matches_scaled_e4m3_model(ctx, m, n, k):
    rng = np.random.default_rng(m + n + k)
    A = (rng.standard_normal((m, k)) * 3.0).astype(np.float32)
    B = (rng.standard_normal((k, n)) * 0.01).astype(np.float32)
    C = rng.standard_normal((m, n)).astype(np.float32)
    dC = cm(C)
    ctx.gemm_sub_tc(cm(A), cm(B), dC, gemm_kind=3)
    assert ctx.status()[1] == 0
    got = dC.cpu().double().numpy()
    sa, sb = pow2_scale(np.abs(A).max()), pow2_scale(np.abs(B).max())
    Aq = e4m3(A.astype(np.float64) * sa)
    Bq = e4m3(B.astype(np.float64) * sb)
    ref = C.astype(np.float64) - (Aq @ Bq) / (sa * sb)
    prod_scale = np.abs(A).max() * np.abs(B).max() * np.sqrt(k)
    assert np.abs(got - ref).max() <= 2e-5 * prod_scale, np.abs(got - ref).max()
    # and it is really 8-bit: far from the FP32 product
    exact = C.astype(np.float64) - A.astype(np.float64) @ B.astype(np.float64)
    assert np.abs(got - exact).max() > 1e-3 * prod_scale


def test_fp8_solve_meets_the_target_through_the_fallback(ctx):
    """E4M3's 3-bit mantissa leaves the FP8 factorization too coarse for
    refinement to converge on these systems (see the factor residual below);
    the solve then falls back to the FP64 LU and still meets n eps64."""
    n = 1024
    A = mats.conditioned(n, 1e2, 31)
    B = mats.gaussian(n, 4, 32)
    dA = D.to_colmajor(torch.from_numpy(A).cuda())
    dB = D.to_colmajor(torch.from_numpy(B).cuda())
    X, info = ctx.refined_solve(dA, dB, precision="fp8", method="gmres-ir", nb=128,
                                max_iters=60)
    assert info["converged"], info
    assert info["backward_error"] <= n * 2.0 ** -53
    Xh = X.cpu().numpy()
    be = max(np.linalg.norm(B[:, c] - A @ Xh[:, c]) /
             (np.linalg.norm(A) * np.linalg.norm(Xh[:, c]) + np.linalg.norm(B[:, c]))
             for c in range(4))
    assert be <= n * 2.0 ** -53
    X2, info2 = ctx.refined_solve(dA, dB, precision="fp8", method="gmres-ir", nb=128,
                                  max_iters=60, fallback=False)
    assert not info2["fell_back"] and info2["precision"] == "fp8"


def test_fp8_lu_factor_is_coarse_but_pivoted(ctx):
    """The FP8 factorization keeps the pivot structure (|L| <= 1) and stays
    finite, at a residual orders above TF32x3's (E4M3 carries 3 mantissa
    bits; one power-of-two scale per panel operand)."""
    n = 512
    A = mats.gaussian(n, n, 41).astype(np.float32)
    res = {}
    for kind in (2, 3):
        dA = cm(A)
        piv = ctx.lu_mixed(dA, gemm_kind=kind, nb=64).cpu().numpy()
        LU = dA.cpu().double().numpy()
        assert np.isfinite(LU).all()
        L = np.tril(LU, -1) + np.eye(n)
        U = np.triu(LU)
        assert np.abs(np.tril(LU, -1)).max() <= 1.0 + 1e-6
        PA = A.astype(np.float64).copy()
        for i, p in enumerate(piv):
            PA[[i, p]] = PA[[p, i]]
        res[kind] = np.linalg.norm(PA - L @ U) / np.linalg.norm(A)
    assert res[2] < 1e-5
    assert res[3] > 1e3 * res[2] and res[3] < 2.0, res
