"""The tcgen05 tensor-core update C -= A B (tc_gemm.cu) against an FP64
product of the same rounded operands (the arithmetic the tensor core is
asked to do), and the tensor-core LU against the FP32 oracle."""
import numpy as np
import pytest
import torch

from elemental_gb300 import device as D
from elemental_gb300 import matrices as mats
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def tf32_rna(x):
    """Round FP32 to TF32 (10 explicit mantissa bits), nearest, ties away."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x1000) & 0xFFFFE000
    return b.astype(np.uint32).view(np.float32)


def rounded(x, kind):
    x = np.asarray(x, dtype=np.float32)
    if kind == 0:
        return torch.from_numpy(x).bfloat16().float().numpy().astype(np.float64)
    hi = tf32_rna(x)
    if kind == 1:
        return hi.astype(np.float64)
    return hi.astype(np.float64), tf32_rna(x - hi).astype(np.float64)


def cm(a):
    return D.to_colmajor(torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.float32).T)).t()
                         .cuda())


@pytest.mark.parametrize("kind", [0, 1, 2])
@pytest.mark.parametrize("m,n,k", [(128, 256, 64), (64, 64, 16), (300, 500, 200),
                                   (1000, 777, 512), (257, 1030, 96)])
def test_tc_gemm_sub_matches_rounded_product(ctx, kind, m, n, k):
    rng = np.random.default_rng(m * 7 + n * 3 + k + kind)
    A = rng.standard_normal((m, k)).astype(np.float32)
    B = rng.standard_normal((k, n)).astype(np.float32)
    C = rng.standard_normal((m, n)).astype(np.float32)
    dC = cm(C)
    ctx.gemm_sub_tc(cm(A), cm(B), dC, gemm_kind=kind)
    info, err = ctx.status()
    assert err == 0
    got = dC.cpu().double().numpy()
    if kind == 2:
        Ah, Al = rounded(A, 2)
        Bh, Bl = rounded(B, 2)
        ref = C.astype(np.float64) - (Ah @ Bh + Ah @ Bl + Al @ Bh)
        exact = C.astype(np.float64) - A.astype(np.float64) @ B.astype(np.float64)
        # FP32 accumulation of ~FP32-accurate products
        assert np.abs(got - exact).max() <= 2e-5 * np.sqrt(k) * 4
    else:
        ref = C.astype(np.float64) - rounded(A, kind) @ rounded(B, kind)
    scale = np.sqrt(k) * 4
    assert np.abs(got - ref).max() <= 1e-5 * scale, np.abs(got - ref).max()


@pytest.mark.parametrize("kind,tol", [(2, 4e-5), (1, 5e-2), (0, 3e-1), (-1, 4e-5)])
@pytest.mark.parametrize("n,nb", [(1024, 256), (1500, 512)])
def test_tc_lu_backward_error(ctx, kind, tol, n, nb):
    A = mats.gaussian(n, n, n + kind)
    dA = cm(A)
    piv = ctx.lu_mixed(dA, gemm_kind=kind, nb=nb)
    ctx.check()
    LU = dA.cpu().double().numpy()
    L = np.tril(LU, -1) + np.eye(n)
    U = np.triu(LU)
    PA = O.permute_rows(piv.cpu().numpy(), A.astype(np.float64))
    rel = np.linalg.norm(PA - L @ U) / np.linalg.norm(A)
    assert rel <= tol, rel
    # pivots of a partially pivoted LU only agree with the oracle's up to the
    # first near-tie that the different rounding breaks the other way, so
    # only the first steps are compared (exact-FP32 SIMT path only)
    if kind == -1:
        LUr, pivr = O.lu(A.astype(np.float32), nb=nb, dtype=np.float32)
        assert np.array_equal(piv.cpu().numpy()[:8], pivr[:8])
