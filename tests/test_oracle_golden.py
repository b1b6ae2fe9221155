"""The CPU oracle (oracle/el_oracle.c, and the numpy restatements of LU
without pivoting, Inverse and OneCondition in oracle/oracle.py) against
golden fixtures produced by the reference itself (tests/golden/gen_golden.py).
Pivots must match exactly; values of the C restatement match bit-for-bit on
the BLAS the fixtures were made with and to rounding on any other BLAS build;
the numpy restatements match to rounding."""
import glob
import hashlib
import os

import numpy as np
import pytest

from elemental_gb300 import matrices as mats
from oracle import oracle as O

GOLD = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
RTOL = 1e-11


def close(a, b, scale=1.0):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    tol = RTOL * max(scale, np.abs(b).max() if b.size else 0.0, 1.0)
    assert np.abs(a - b).max(initial=0.0) <= tol, np.abs(a - b).max()


def _name(p):
    return os.path.basename(p)[:-4]


@pytest.mark.parametrize("path", [p for p in GOLD if not _name(p).startswith("cfg1")],
                         ids=[_name(p) for p in GOLD if not _name(p).startswith("cfg1")])
def test_oracle_matches_reference_fixture(path):
    g = np.load(path)
    op = str(g["op"])
    st = int(g["status"])
    nb = int(g["nb"]) if "nb" in g else 128
    if op == "lu":
        dt = np.float32 if str(g["dtype"]) == "float32" else np.float64
        if st != 0:
            with pytest.raises(O.OracleError) as e:
                O.lu(g["A"], nb=nb, dtype=dt)
            assert e.value.status == st
            return
        LU, piv = O.lu(g["A"], nb=nb, dtype=dt)
        assert np.array_equal(piv, g["piv"])
        if dt == np.float32:
            assert np.abs(LU - g["LU"]).max() <= 1e-4 * max(1.0, np.abs(g["LU"]).max())
        else:
            close(LU, g["LU"])
    elif op == "lusolve":
        LU, piv = O.lu(g["A"], nb=nb)
        assert np.array_equal(piv, g["piv"])
        X = O.lu_solve_after(LU, piv, g["B"], 0 if str(g["orient"]) == "N" else 1)
        close(X, g["X"])
    elif op == "chol":
        if st != 0:
            with pytest.raises(O.OracleError) as e:
                O.cholesky(g["A"], str(g["uplo"]), nb=nb)
            assert e.value.status == st
            return
        C = O.cholesky(g["A"], str(g["uplo"]), nb=nb)
        close(C, g["C"])
    elif op == "cholsolve":
        C = O.cholesky(g["A"], str(g["uplo"]), nb=nb)
        close(C, g["C"])
        close(O.cholesky_solve_after(C, g["B"], str(g["uplo"])), g["X"])
    elif op == "hpdsolve":
        close(O.hpd_solve(g["A"], g["B"], str(g["uplo"]), nb=nb), g["X"])
    elif op == "linsolve":
        close(O.linear_solve(g["A"], g["B"], nb=nb), g["X"])
    elif op in ("lunopiv", "inverse"):
        dt = np.float32 if str(g.get("dtype", "float64")) == "float32" else np.float64
        fn = O.lu_nopiv if op == "lunopiv" else O.inverse
        if st != 0:  # SingularMatrixException in the reference
            with pytest.raises(O.OracleError) as e:
                fn(g["A"], nb=nb, dtype=dt)
            assert e.value.status == st
            return
        X = fn(g["A"], nb=nb, dtype=dt)
        ref = g["LU"] if op == "lunopiv" else g["Ainv"]
        # a block-level numpy restatement: equal to rounding, relative to
        # the result's size (the inverse of a kappa = 1e6 matrix included)
        tol = (1e-5 if dt == np.float32 else 1e-13) * np.abs(ref).max()
        assert np.abs(X - ref).max() <= tol, np.abs(X - ref).max()
    elif op == "write":  # the oracle's reader of Elemental's binary layout
        raw = bytes(g["raw"])
        A = g["A"]
        if str(g["fmt"]) == "bin":
            import tempfile

            with tempfile.TemporaryDirectory() as d:
                path = os.path.join(d, "m.bin")
                with open(path, "wb") as f:
                    f.write(raw)
                assert np.array_equal(O.read_el_binary(path, A.dtype), A)
        else:
            assert np.array_equal(np.frombuffer(raw, A.dtype).reshape(A.shape[::-1]).T, A)
    elif op in ("lufull", "lufullsolve"):
        if st != 0:
            with pytest.raises(O.OracleError) as e:
                O.lu_full(g["A"])
            assert e.value.status == st
            return
        LU, p, q = O.lu_full(g["A"])
        assert np.array_equal(p, g["p"]) and np.array_equal(q, g["q"])
        close(LU, g["LU"])
        if op == "lufullsolve":
            X = O.lu_full_solve_after(LU, p, q, g["B"], 0 if str(g["orient"]) == "N" else 1)
            close(X, g["X"])
    elif op in ("cholpiv", "cholpivsolve"):
        u = str(g["uplo"])
        C, piv = O.cholesky_piv(g["A"], u, nb=nb)
        assert np.array_equal(piv, g["piv"])
        tri = np.tril if u == "L" else np.triu
        close(tri(C), tri(g["C"]))
        if op == "cholpivsolve":
            close(O.cholesky_piv_solve_after(C, piv, g["B"], u), g["X"])
    elif op == "onecond":
        c, ref = O.one_condition(g["A"], nb=nb), float(g["cond"])
        if np.isinf(ref):
            assert np.isinf(c)
        else:
            assert abs(c - ref) <= 1e-12 * ref, (c, ref)
    else:
        pytest.fail(op)


def test_oracle_config1_against_reference():
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "cfg1_lusolve_1024_nb128.npz"))
    n = int(g["n"])
    A = mats.gaussian(n, n, int(g["seed_A"]))
    b = mats.gaussian(n, 1, int(g["seed_b"]))
    assert hashlib.sha256(A.tobytes(order="F")).hexdigest() == str(g["sha_A"]), \
        "input generator is not reproducible on this platform"
    assert hashlib.sha256(b.tobytes(order="F")).hexdigest() == str(g["sha_b"])
    LU, piv = O.lu(A, nb=128)
    assert np.array_equal(piv, g["piv"])
    X = O.lu_solve_after(LU, piv, b)
    close(X, g["X"], scale=1e3)
    berr = O.backward_error(A, X, b)
    assert berr <= 4 * n * np.finfo(np.float64).eps
    assert abs(berr - float(g["berr"])) <= 4 * n * np.finfo(np.float64).eps


def test_backward_error_metric():
    A = np.eye(3)
    X = np.ones((3, 1))
    assert O.backward_error(A, X, A @ X) == 0.0
    B = A @ X + np.array([[1e-3], [0], [0]])
    be = O.backward_error(A, X, B)
    assert abs(be - 1e-3 / (np.sqrt(3) * np.sqrt(3) + np.linalg.norm(B))) < 1e-15
