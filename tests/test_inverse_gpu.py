"""El::LU without pivoting, El::Inverse and El::OneCondition on the GPU,
through the device ABI (elemental_gb300.device) and Elemental's C ABI on host
matrices (elemental_gb300.El mirror), against the reference's own outputs
(tests/golden, made by tests/golden/gen_golden.py from the compiled
reference) and the oracle.

Tolerances: LU without pivoting is compared elementwise relative to the
factors' size (different but backward-stable operation orders); the inverse
is unique, and two backward-stable inverses differ by up to ~kappa_1 * n *
eps relative, so that is the bound used; OneCondition inherits the inverse's
relative error."""
import os

import numpy as np
import pytest

import elemental_gb300 as El
from elemental_gb300 import matrices as mats
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
EPS64 = np.finfo(np.float64).eps
EPS32 = float(np.finfo(np.float32).eps)


def load(name):
    return np.load(os.path.join(GOLD, name + ".npz"))


@pytest.fixture(scope="module")
def ctx():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from elemental_gb300 import device as D

    return D.context(0)


def dev(A, dtype=None):
    import torch

    from elemental_gb300 import device as D

    A = np.asarray(A)
    dt = dtype or (torch.float32 if A.dtype == np.float32 else torch.float64)
    T = D.colmajor(A.shape[0], A.shape[1], dtype=dt)
    T.copy_(torch.from_numpy(np.ascontiguousarray(A)).to(dt))
    return T


def kappa1(A):
    return np.linalg.cond(np.asarray(A, dtype=np.float64), 1)


@pytest.mark.parametrize("name", ["lunopiv_100_nb32", "lunopiv_90x130_nb32",
                                  "lunopiv_130x90_nb32"])
def test_lu_nopiv_matches_reference(ctx, name):
    g = load(name)
    A = dev(g["A"])
    ctx.lu_nopiv(A, nb=int(g["nb"]))
    assert ctx.status() == (0, 0)
    ref = g["LU"]
    assert np.abs(A.cpu().numpy() - ref).max() <= 1e-12 * np.abs(ref).max()


def test_lu_nopiv_exact_zero_pivot_sets_info(ctx):
    # row 40 is zero, so pivot 40 stays exactly 0: the reference throws
    # SingularMatrixException (status 3 in the fixture); the device reports
    # the 1-based column
    g = load("lunopiv_singular_100_nb32")
    assert int(g["status"]) == 3
    A = dev(g["A"])
    ctx.lu_nopiv(A, nb=32)
    assert ctx.status() == (41, 0)


def test_lu_nopiv_large_reconstructs(ctx):
    # n = 3000 (several panel blocks and recursion levels): L U = A
    n = 3000
    A0 = mats.gaussian(n, n, 77) + n * np.eye(n)
    A = dev(A0)
    ctx.lu_nopiv(A)
    assert ctx.status() == (0, 0)
    W = A.cpu().numpy()
    L = np.tril(W, -1) + np.eye(n)
    U = np.triu(W)
    assert np.linalg.norm(L @ U - A0) <= 20 * n * EPS64 * np.linalg.norm(A0)


@pytest.mark.parametrize("name", ["inverse_100_nb32", "inverse_129_nb96",
                                  "inverse_haar_k1e6_80_nb16"])
def test_inverse_matches_reference(ctx, name):
    g = load(name)
    A = dev(g["A"])
    ctx.inverse(A, nb=int(g["nb"]))
    assert ctx.status() == (0, 0)
    X, ref = A.cpu().numpy(), g["Ainv"]
    n = len(ref)
    assert np.linalg.norm(X - ref) <= 10 * n * EPS64 * kappa1(g["A"]) * np.linalg.norm(ref)


def test_inverse_fp32_matches_reference(ctx):
    g = load("inverse_s_64_nb32")
    A = dev(g["A"])
    ctx.inverse(A, nb=32)
    assert ctx.status() == (0, 0)
    X, ref = A.cpu().numpy(), g["Ainv"].astype(np.float64)
    assert np.linalg.norm(X - ref) <= 10 * 64 * EPS32 * kappa1(g["A"]) * np.linalg.norm(ref)


def test_inverse_singular_sets_info(ctx):
    g = load("inverse_singular_50_nb16")
    assert int(g["status"]) == 3
    A = dev(g["A"])
    ctx.inverse(A, nb=16)
    assert ctx.status() == (8, 0)  # column 7 is zero


def test_inverse_large_is_an_inverse(ctx):
    n = 2048
    A0 = mats.gaussian(n, n, 91)
    A = dev(A0)
    ctx.inverse(A)
    assert ctx.status() == (0, 0)
    X = A.cpu().numpy()
    R = A0 @ X - np.eye(n)
    assert np.linalg.norm(R) <= 10 * n * EPS64 * np.linalg.norm(A0) * np.linalg.norm(X)


@pytest.mark.parametrize("name", ["onecond_haar_k1e4_80", "onecond_gauss_120",
                                  "onecond_singular_50"])
def test_one_condition_matches_reference(ctx, name):
    g = load(name)
    A = dev(g["A"])
    A_before = A.clone()
    c, ref = ctx.one_condition(A, nb=32), float(g["cond"])
    assert ctx.status() == (0, 0)  # a singular A is not an error: +inf
    assert bool((A == A_before).all())  # A is not modified
    if np.isinf(ref):
        assert np.isinf(c)
    else:
        assert abs(c - ref) <= 10 * len(g["A"]) * EPS64 * kappa1(g["A"]) * ref


def test_empty_matrices(ctx):
    import torch

    from elemental_gb300 import device as D

    A = D.colmajor(0, 0, dtype=torch.float64)
    ctx.inverse(A)
    ctx.lu_nopiv(A)
    assert ctx.one_condition(A) == 0.0


def test_el_c_abi_lu_nopiv_inverse_onecond():
    g = load("inverse_129_nb96")
    El.PushBlocksizeStack(96)
    try:
        A = El.Matrix(g["A"].copy(order="F"))
        El.Inverse(A)
        ref = g["Ainv"]
        assert np.linalg.norm(A.array - ref) <= (10 * 129 * EPS64 * kappa1(g["A"])
                                                 * np.linalg.norm(ref))
        gc = load("onecond_haar_k1e4_80")
        c = El.OneCondition(El.Matrix(gc["A"].copy(order="F")))
        assert abs(c - float(gc["cond"])) <= 1e-9 * float(gc["cond"])
        assert np.isinf(El.OneCondition(El.Matrix(load("onecond_singular_50")["A"]
                                                  .copy(order="F"))))
        gl = load("lunopiv_100_nb32")
        El.PushBlocksizeStack(32)
        try:
            L = El.Matrix(gl["A"].copy(order="F"))
            assert El.LU(L, El.LU_WITHOUT_PIVOTING) is None
            assert np.abs(L.array - gl["LU"]).max() <= 1e-12 * np.abs(gl["LU"]).max()
            with pytest.raises(El.SingularMatrixException):
                El.LU(El.Matrix(load("lunopiv_singular_100_nb32")["A"].copy(order="F")),
                      El.LU_WITHOUT_PIVOTING)
        finally:
            El.PopBlocksizeStack()
        with pytest.raises(El.SingularMatrixException):
            El.Inverse(El.Matrix(load("inverse_singular_50_nb16")["A"].copy(order="F")))
        with pytest.raises(El.ElError):
            El.Inverse(El.Matrix(mats.gaussian(5, 7, 3)))  # non-square: logic error
    finally:
        El.PopBlocksizeStack()


def test_oracle_agrees_with_device_inverse(ctx):
    # the oracle restatement and the device on a fresh case the fixtures do
    # not hold (kappa = 1e8 Haar, n = 300)
    A0 = mats.conditioned(300, 1e8, 5)
    A = dev(A0)
    ctx.inverse(A, nb=64)
    X = A.cpu().numpy()
    Xo = O.inverse(A0, nb=64)
    assert np.linalg.norm(X - Xo) <= 10 * 300 * EPS64 * kappa1(A0) * np.linalg.norm(Xo)
