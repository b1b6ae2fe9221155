"""Edge cases and FP32 variants of the next rows (LU without pivoting, full
pivoting, diagonal-pivoted Cholesky) on the GPU against the oracle, whose FP64
restatements are pinned to the reference's fixtures
(tests/test_oracle_golden.py): 1 x 1 and vector-shaped matrices, and the _s
entry points."""
import numpy as np
import pytest

from elemental_gb300 import matrices as mats
from oracle import oracle as O

pytestmark = pytest.mark.gpu
EPS32 = float(np.finfo(np.float32).eps)


@pytest.fixture(scope="module")
def ctx():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from elemental_gb300 import device as D

    return D.context(0)


def dev(A, dtype="f64"):
    import torch

    from elemental_gb300 import device as D

    dt = torch.float64 if dtype == "f64" else torch.float32
    A = np.asarray(A)
    T = D.colmajor(A.shape[0], A.shape[1], dtype=dt)
    T.copy_(torch.from_numpy(np.ascontiguousarray(A)).to(dt))
    return T


@pytest.mark.parametrize("shape", [(1, 1), (1, 5), (5, 1), (2, 7), (7, 2)])
def test_lu_full_small_shapes(ctx, shape):
    A0 = mats.gaussian(*shape, seed=31 + shape[0] * 10 + shape[1])
    A = dev(A0)
    p, q = ctx.lu_full(A)
    assert ctx.status() == (0, 0)
    LUo, po, qo = O.lu_full(A0)
    assert np.array_equal(p.cpu().numpy(), po) and np.array_equal(q.cpu().numpy(), qo)
    assert np.abs(A.cpu().numpy() - LUo).max() <= 1e-14 * max(1.0, np.abs(LUo).max())


def test_lu_full_fp32_matches_oracle(ctx):
    A0 = mats.gaussian(48, 40, 77).astype(np.float32)
    A = dev(A0, "f32")
    p, q = ctx.lu_full(A)
    assert ctx.status() == (0, 0)
    LUo, po, qo = O.lu_full(A0, dtype=np.float32)
    assert np.array_equal(p.cpu().numpy(), po) and np.array_equal(q.cpu().numpy(), qo)
    assert np.abs(A.cpu().numpy() - LUo).max() <= 50 * EPS32 * np.abs(LUo).max()


@pytest.mark.parametrize("uplo", [0, 1])
def test_cholesky_piv_one_by_one_and_fp32(ctx, uplo):
    A = dev(np.array([[4.0]]))
    piv = ctx.cholesky_piv(A, uplo)
    assert int(piv.cpu().numpy()[0]) == 0 and float(A.cpu().numpy()[0, 0]) == 2.0
    S0 = mats.spd(64, 9 + uplo).astype(np.float32)
    S = dev(S0, "f32")
    piv = ctx.cholesky_piv(S, uplo)
    Co, po = O.cholesky_piv(S0, "L" if uplo == 0 else "U", nb=128, dtype=np.float32)
    assert np.array_equal(piv.cpu().numpy(), po)
    tri = np.tril if uplo == 0 else np.triu
    assert np.abs(tri(S.cpu().numpy()) - tri(Co)).max() <= 50 * EPS32 * np.abs(Co).max()


def test_lu_nopiv_fp32_and_wide(ctx):
    D0 = (mats.gaussian(40, 70, 5) + np.hstack([40.0 * np.eye(40), np.zeros((40, 30))]))
    A = dev(D0.astype(np.float32), "f32")
    ctx.lu_nopiv(A)
    assert ctx.status() == (0, 0)
    Wo = O.lu_nopiv(D0.astype(np.float32), nb=128, dtype=np.float32)
    assert np.abs(A.cpu().numpy() - Wo).max() <= 50 * EPS32 * np.abs(Wo).max()
