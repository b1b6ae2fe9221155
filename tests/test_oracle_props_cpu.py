"""Properties of the oracle restatements beyond the reference's fixtures
(tests/test_oracle_golden.py pins them to the reference itself): invariants
each algorithm guarantees, on seeded inputs of shapes the fixtures do not
hold."""
import numpy as np
import pytest

from elemental_gb300 import matrices as mats
from oracle import oracle as O

EPS = np.finfo(np.float64).eps


def perm_rows(dests, A):
    return O.permute_rows(np.asarray(dests, dtype=np.int32), np.asfortranarray(A))


@pytest.mark.parametrize("shape", [(30, 20), (20, 30), (25, 25)])
def test_lu_full_invariants(shape):
    m, n = shape
    A = mats.gaussian(m, n, 900 + m + n)
    W, p, q = O.lu_full(A)
    k = min(m, n)
    L = np.tril(W, -1)[:, :k] + np.eye(m, k)
    U = np.triu(W[:k, :])
    assert np.abs(np.tril(W, -1)).max() <= 1.0  # full pivoting: |l_ij| <= 1
    assert all(p[i] >= i for i in range(k)) and all(q[i] >= i for i in range(k))
    PAQ = perm_rows(q, perm_rows(p, A).T).T
    assert np.linalg.norm(L @ U - PAQ) <= 20 * max(m, n) * EPS * np.linalg.norm(A)


def test_cholesky_piv_invariants():
    n = 50
    A = mats.spd(n, 901)
    for uplo in ("L", "U"):
        C, p = O.cholesky_piv(A, uplo, nb=16)
        L = np.tril(C) if uplo == "L" else np.triu(C).T
        d = np.diag(L)
        assert np.all(d[:-1] >= d[1:] - 1e-14)  # the largest remaining pivot first
        PAP = perm_rows(p, perm_rows(p, A).T).T
        assert np.linalg.norm(L @ L.T - PAP) <= 20 * n * EPS * np.linalg.norm(A)


def test_inverse_and_one_condition():
    A = mats.conditioned(60, 1e5, 902)
    X = O.inverse(A, nb=16)
    assert np.linalg.norm(A @ X - np.eye(60)) <= 60 * EPS * np.linalg.cond(A) * 10
    k1 = np.linalg.cond(A, 1)
    assert abs(O.one_condition(A, nb=16) - k1) <= 1e-8 * k1


def test_lu_nopiv_reconstructs():
    A = mats.gaussian(40, 40, 903) + 40 * np.eye(40)
    W = O.lu_nopiv(A, nb=16)
    L = np.tril(W, -1) + np.eye(40)
    assert np.linalg.norm(L @ np.triu(W) - A) <= 40 * EPS * np.linalg.norm(A) * 10
