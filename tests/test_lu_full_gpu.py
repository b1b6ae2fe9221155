"""El::LU(A, P, Q) with full pivoting and lu::SolveAfter(orientation, A, P,
Q, B) on the GPU, through the device ABI and Elemental's C ABI on host
matrices, against the reference's own outputs (tests/golden/lufull*.npz, made
by tests/golden/gen_golden.py from the compiled reference) and the oracle.

The row and column swap destinations are integer results and must match the
reference exactly (including an exact tie for a pivot, which MaxAbsLoc gives
to the first entry in column-major order).  The factors are compared to
rounding: the update is one fused multiply-add per entry, as the reference's
BLAS ger computes it."""
import os

import numpy as np
import pytest

import elemental_gb300 as El
from elemental_gb300 import matrices as mats
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
EPS64 = np.finfo(np.float64).eps


def load(name):
    return np.load(os.path.join(GOLD, name + ".npz"))


@pytest.fixture(scope="module")
def ctx():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from elemental_gb300 import device as D

    return D.context(0)


def dev(A):
    import torch

    from elemental_gb300 import device as D

    A = np.asarray(A, dtype=np.float64)
    T = D.colmajor(A.shape[0], A.shape[1])
    T.copy_(torch.from_numpy(np.ascontiguousarray(A)))
    return T


@pytest.mark.parametrize("name", ["lufull_60", "lufull_70x45", "lufull_45x70", "lufull_tie_16"])
def test_lu_full_matches_reference(ctx, name):
    g = load(name)
    A = dev(g["A"])
    p, q = ctx.lu_full(A)
    assert ctx.status() == (0, 0)
    assert np.array_equal(p.cpu().numpy(), g["p"])
    assert np.array_equal(q.cpu().numpy(), g["q"])
    assert np.abs(A.cpu().numpy() - g["LU"]).max() <= 1e-12 * np.abs(g["LU"]).max()


def test_lu_full_zero_matrix_sets_info(ctx):
    g = load("lufull_zero_30")
    assert int(g["status"]) == 3  # SingularMatrixException at the first step
    A = dev(g["A"])
    ctx.lu_full(A)
    assert ctx.status() == (1, 0)


@pytest.mark.parametrize("o", ["N", "T"])
def test_lu_full_solve_matches_reference(ctx, o):
    import torch

    g = load(f"lufullsolve_{o}_64")
    A = dev(g["A"])
    p, q = ctx.lu_full(A)
    assert np.array_equal(p.cpu().numpy(), g["p"]) and np.array_equal(q.cpu().numpy(), g["q"])
    B = dev(g["B"])
    ctx.lu_full_solve_after(A, p, q, B, 0 if o == "N" else 1)
    assert ctx.status() == (0, 0)
    X = B.cpu().numpy()
    assert np.abs(X - g["X"]).max() <= 1e-11 * np.abs(g["X"]).max()
    del torch


def test_lu_full_matches_oracle_and_reconstructs(ctx):
    # 400 x 300: pivots equal to the oracle (which is bit-identical to the
    # reference), P A Q^T = L U
    A0 = mats.gaussian(400, 300, 2024)
    A = dev(A0)
    p, q = ctx.lu_full(A)
    assert ctx.status() == (0, 0)
    LUo, po, qo = O.lu_full(A0)
    assert np.array_equal(p.cpu().numpy(), po) and np.array_equal(q.cpu().numpy(), qo)
    W = A.cpu().numpy()
    assert np.abs(W - LUo).max() <= 1e-11 * np.abs(LUo).max()
    L = np.tril(W, -1)[:, :300] + np.eye(400, 300)
    U = np.triu(W[:300, :])
    PA = O.permute_rows(po, A0)
    PAQ = O.permute_rows(qo, np.asfortranarray(PA.T)).T
    assert np.linalg.norm(L @ U - PAQ) <= 50 * 400 * EPS64 * np.linalg.norm(A0)


def test_lu_full_through_el_c_abi():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    g = load("lufullsolve_N_64")
    A = El.Matrix(g["A"].copy(order="F"))
    P, Q = El.LU(A, El.LU_FULL)
    assert np.array_equal(P.SwapDestinations(), g["p"])
    assert np.array_equal(Q.SwapDestinations(), g["q"])
    B = El.Matrix(g["B"].copy(order="F"))
    El.SolveAfterLUFullPiv(El.NORMAL, A, P, Q, B)
    assert np.abs(B.array - g["X"]).max() <= 1e-11 * np.abs(g["X"]).max()
    with pytest.raises(El.SingularMatrixException):
        El.LU(El.Matrix(np.zeros((30, 30))), El.LU_FULL)
