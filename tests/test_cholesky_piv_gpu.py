"""El::Cholesky(uplo, A, P) with diagonal pivoting and its
cholesky::SolveAfter on the GPU, through the device ABI and Elemental's C ABI
on host matrices, against the reference's own outputs
(tests/golden/cholpiv*.npz, made by tests/golden/gen_golden.py from the
compiled reference) and the oracle.

The device factors right-looking (eager updates); the reference's lazy panels
compute the same updated diagonals up to rounding, so the swap destinations
must match exactly (on these inputs no two candidates are within rounding of
each other -- the correlation matrix's first step, where every diagonal entry
is exactly 1, checks the first-index rule) and the factors to rounding."""
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


@pytest.mark.parametrize("name", ["cholpiv_L_spd90_nb32", "cholpiv_U_spd90_nb32",
                                  "cholpiv_L_corr70_nb32", "cholpiv_U_corr70_nb32"])
def test_cholesky_piv_matches_reference(ctx, name):
    g = load(name)
    u = str(g["uplo"])
    A = dev(g["A"])
    before = A.clone()
    piv = ctx.cholesky_piv(A, 0 if u == "L" else 1)
    assert ctx.status() == (0, 0)
    assert np.array_equal(piv.cpu().numpy(), g["piv"])
    tri = np.tril if u == "L" else np.triu
    C = A.cpu().numpy()
    assert np.abs(tri(C) - tri(g["C"])).max() <= 1e-12 * np.abs(g["C"]).max()
    # the other strict triangle is not touched
    other = np.triu if u == "L" else np.tril
    k = 1 if u == "L" else -1
    assert np.array_equal(other(C, k), other(before.cpu().numpy(), k))


@pytest.mark.parametrize("u", ["L", "U"])
def test_cholesky_piv_solve_matches_reference(ctx, u):
    g = load(f"cholpivsolve_{u}_spd90_nb32")
    A = dev(g["A"])
    up = 0 if u == "L" else 1
    piv = ctx.cholesky_piv(A, up)
    assert np.array_equal(piv.cpu().numpy(), g["piv"])
    B = dev(g["B"])
    ctx.cholesky_piv_solve_after(A, piv, B, up)
    assert ctx.status() == (0, 0)
    assert np.abs(B.cpu().numpy() - g["X"]).max() <= 1e-11 * np.abs(g["X"]).max()


def test_cholesky_piv_matches_oracle_and_reconstructs(ctx):
    n = 600
    A0 = mats.spd(n, 4242)
    A = dev(A0)
    piv = ctx.cholesky_piv(A, 0)
    assert ctx.status() == (0, 0)
    Co, po = O.cholesky_piv(A0, "L", nb=128)
    assert np.array_equal(piv.cpu().numpy(), po)
    L = np.tril(A.cpu().numpy())
    assert np.abs(L - np.tril(Co)).max() <= 1e-12 * np.abs(Co).max()
    PA = O.permute_rows(po, A0)
    PAP = O.permute_rows(po, np.asfortranarray(PA.T)).T
    assert np.linalg.norm(L @ L.T - PAP) <= 20 * n * EPS64 * np.linalg.norm(A0)


def test_cholesky_piv_through_el_c_abi():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    g = load("cholpivsolve_U_spd90_nb32")
    A = El.Matrix(g["A"].copy(order="F"))
    P = El.Cholesky(El.UPPER, A, piv=True)
    assert np.array_equal(P.SwapDestinations(), g["piv"])
    B = El.Matrix(g["B"].copy(order="F"))
    El.SolveAfterCholeskyPiv(El.UPPER, El.NORMAL, A, P, B)
    assert np.abs(B.array - g["X"]).max() <= 1e-11 * np.abs(g["X"]).max()
