"""The Elemental-compatible C ABI (include/El_gb300.h) on host matrices, as
the reference's ctypes layer drives it (python/lapack_like/factor.py)."""
import numpy as np
import pytest

import elemental_gb300 as El
from elemental_gb300 import matrices as mats
from oracle import oracle as O

pytestmark = pytest.mark.gpu
EPS = np.finfo(np.float64).eps


@pytest.fixture(autouse=True)
def _gpu():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def test_lu_and_solve_after_through_el_c_abi():
    n = 300
    A0 = mats.gaussian(n, n, 42)
    B0 = mats.gaussian(n, 4, 43)
    A = El.Matrix(A0.copy(order="F"))
    P = El.LU(A)
    LUr, pivr = O.lu(A0, nb=El.Blocksize())
    assert np.array_equal(P.SwapDestinations(), pivr)
    assert np.abs(A.array - LUr).max() <= 1e-10 * np.abs(LUr).max()
    B = El.Matrix(B0.copy(order="F"))
    El.SolveAfterLUPartialPiv(El.NORMAL, A, P, B)
    assert O.backward_error(A0, B.array, B0) <= 4 * n * EPS


def test_singular_raises_runtime_error_code():
    A0 = mats.gaussian(40, 40, 1)
    A0[:, 7] = 0
    with pytest.raises(El.SingularMatrixException) as e:
        El.LU(El.Matrix(A0))
    assert e.value.code == 5  # EL_RUNTIME_ERROR, as EL_TRY maps SingularMatrixException


def test_cholesky_hpd_linear_solve_through_el_c_abi():
    n = 200
    S0 = mats.spd(n, 5)
    B0 = mats.gaussian(n, 3, 6)
    B = El.Matrix(B0.copy(order="F"))
    El.HPDSolve(El.Matrix(S0), B, El.LOWER, El.NORMAL)
    assert np.abs(B.array - O.hpd_solve(S0, B0, "L")).max() < 1e-9
    A0 = mats.gaussian(n, n, 7)
    B = El.Matrix(B0.copy(order="F"))
    El.LinearSolve(El.Matrix(A0), B)
    assert np.abs(B.array - O.linear_solve(A0, B0)).max() < 1e-8
    C = El.Matrix(S0.copy(order="F"))
    El.Cholesky(El.UPPER, C)
    assert np.abs(np.triu(C.array) - np.triu(O.cholesky(S0, "U"))).max() < 1e-10
    X = El.Matrix(B0.copy(order="F"))
    El.SolveAfterCholesky(El.UPPER, El.NORMAL, C, X)
    assert O.backward_error(S0, X.array, B0) <= 4 * n * EPS
    G = El.Matrix(mats.gaussian(30, 30, 9))
    with pytest.raises(El.SingularMatrixException):
        El.Cholesky(El.LOWER, G)


def test_linear_solve_mixed_on_library_host_memory():
    """El.host_empty (ElGBHostAlloc: registered anonymous pages) holds the
    matrices of a host-matrix call; results equal those on ordinary host
    memory, and the memory round-trips through device copies."""
    import torch

    n, q = 2048, 3
    A0 = mats.gaussian(n, n, 21)
    B0 = mats.gaussian(n, q, 22)
    Ah = El.host_empty((n, n))
    Ah[...] = A0
    Bh = El.host_empty((n, q))
    Bh[...] = B0
    assert Ah.flags.f_contiguous and Bh.flags.f_contiguous
    A = El.Matrix(Ah)
    B = El.Matrix(Bh)
    assert A.array.ctypes.data == Ah.ctypes.data
    El.LinearSolveMixed(A, B)
    B2 = El.Matrix(B0.copy(order="F"))
    El.LinearSolveMixed(El.Matrix(A0.copy(order="F")), B2)
    assert np.array_equal(Bh, B2.array)
    assert O.backward_error(A0, Bh, B0) <= n * EPS
    t = torch.from_numpy(Ah)
    d = t.cuda(non_blocking=True)
    back = El.host_empty((n, n))
    torch.from_numpy(back).copy_(d)
    assert np.array_equal(back, A0)


def test_host_memory_blocks_are_reusable():
    """Blocks of ElGBHostAlloc memory allocated, written, used for device
    copies and freed in turn (the mapping of a freed block may come back)."""
    import torch

    for k in range(4):
        a = El.host_empty((1024, 1024 + 7 * k))
        a[...] = k + 0.5
        d = torch.from_numpy(a).cuda()
        assert float(d.sum()) == (k + 0.5) * a.size
        del a, d
