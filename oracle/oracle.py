"""ORACLE — test infrastructure only.

Python access to the CPU checker for the dense factor-and-solve path:

* ``el_oracle.c`` — a C restatement of Elemental's sequential El::LU,
  lu::SolveAfter, El::Cholesky, cholesky::SolveAfter, El::LinearSolve and
  El::HPDSolve that calls external BLAS exactly where the reference does
  (built here by :func:`build`, loaded by :func:`lib`);
* ``_ref/elref`` — the reference's own code compiled from its sources by
  ``build_ref.sh`` (only where the reference tree is present);
* numpy restatements of El::LU without pivoting, El::Inverse and
  El::OneCondition (block-level, the same steps as the reference; pinned to
  the reference's outputs within rounding by tests/test_oracle_golden.py)
  and of the added forms' semantics (refinement loop of
  include/El/lapack_like/solve/Refined.hpp:44-119 and the MLP).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this module, and only as the checker / the timed CPU baseline.  The
product path never routes through it.
"""
from __future__ import annotations

import ctypes
import glob
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libel_oracle.so")
REF_EXE = os.path.join(HERE, "_ref", "elref")

_lib = None
_blas = None


def blas_library():
    """Path and symbol prefix of an LP64 BLAS with the reference's routines.

    SciPy's bundled OpenBLAS (``scipy_<name>_`` symbols) is the one the
    reference oracle was built against; any system ``libopenblas`` /
    ``libblas`` with plain ``<name>_`` symbols also works.
    """
    try:
        import scipy

        d = os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs")
        hits = sorted(glob.glob(os.path.join(d, "libscipy_openblas-*.so")))
        if hits:
            return os.path.realpath(hits[0]), "scipy_"
    except ImportError:
        pass
    for cand in ("libopenblas.so.0", "libopenblas.so", "libblas.so.3"):
        for d in ("/usr/lib/x86_64-linux-gnu", "/usr/lib/aarch64-linux-gnu",
                  "/usr/lib64", "/usr/lib"):
            p = os.path.join(d, cand)
            if os.path.exists(p):
                return p, ""
    raise RuntimeError("oracle: no LP64 BLAS library found")


def build(force: bool = False) -> str:
    """Compiles el_oracle.c into oracle/lib/libel_oracle.so (gcc, seconds)."""
    src = os.path.join(HERE, "el_oracle.c")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)):
        return LIB_PATH
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-O2", "-shared", "-fPIC", "-std=gnu11",
                           src, "-o", tmp, "-ldl", "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib(threads: int = 1):
    """Loads the C oracle (building it if needed) and binds BLAS."""
    global _lib, _blas
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        path, prefix = blas_library()
        if L.elo_init(path.encode(), prefix.encode(), int(threads)) != 0:
            raise RuntimeError(f"oracle: could not bind BLAS from {path}")
        _lib, _blas = L, path
    else:
        _lib.elo_set_threads(int(threads))
    return _lib


def set_threads(n: int) -> None:
    lib().elo_set_threads(int(n))


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------
_SUF = {np.float64: "d", np.float32: "s"}


def _f(a, dtype):
    return np.asfortranarray(np.array(a, dtype=dtype, copy=True))


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _suffix(dtype):
    return _SUF[np.dtype(dtype).type]


class OracleError(RuntimeError):
    def __init__(self, status):
        super().__init__({3: "singular matrix", 4: "matrix not HPD",
                          2: "bad arguments", 1: "BLAS not loaded"}.get(
                              status, f"status {status}"))
        self.status = status


def _check(st):
    if st != 0:
        raise OracleError(st)


# ---------------------------------------------------------------------------
# the restated reference path
# ---------------------------------------------------------------------------
def lu(A, nb: int = 128, dtype=np.float64):
    """El::LU(A, P): returns (packed LU, swap destinations int32[min(m,n)])."""
    W = _f(A, dtype)
    m, n = W.shape
    piv = np.zeros(min(m, n), dtype=np.int32)
    fn = getattr(lib(), "elo_lu_" + _suffix(dtype))
    _check(fn(m, n, _p(W), max(m, 1), nb, _p(piv)))
    return W, piv


def permute_rows(piv, B, inverse=False):
    """Permutation::PermuteRows / InversePermuteRows for a swap sequence."""
    X = _f(B, B.dtype)
    m, k = X.shape
    piv = np.ascontiguousarray(piv, dtype=np.int32)
    getattr(lib(), "elo_permute_rows_" + _suffix(X.dtype))(
        int(inverse), len(piv), _p(piv), m, k, _p(X), max(m, 1))
    return X


def lu_solve_after(LU, piv, B, orientation: int = 0):
    """lu::SolveAfter(orientation, A, P, B); orientation 0 NORMAL, 1 TRANSPOSE."""
    LU = _f(LU, LU.dtype)
    X = _f(B, LU.dtype)
    n = LU.shape[0]
    piv = np.ascontiguousarray(piv, dtype=np.int32)
    fn = getattr(lib(), "elo_lu_solve_after_" + _suffix(LU.dtype))
    _check(fn(orientation, n, _p(LU), max(n, 1), _p(piv), X.shape[1], _p(X),
              max(n, 1)))
    return X


def cholesky(A, uplo: str = "L", nb: int = 128, dtype=np.float64):
    """El::Cholesky(uplo, A); only the uplo triangle is referenced/written."""
    W = _f(A, dtype)
    n = W.shape[0]
    fn = getattr(lib(), "elo_cholesky_" + _suffix(dtype))
    _check(fn(ctypes.c_char(uplo.encode()), n, _p(W), max(n, 1), nb))
    return W


def cholesky_solve_after(C, B, uplo: str = "L"):
    C = _f(C, C.dtype)
    X = _f(B, C.dtype)
    n = C.shape[0]
    fn = getattr(lib(), "elo_cholesky_solve_after_" + _suffix(C.dtype))
    _check(fn(ctypes.c_char(uplo.encode()), n, _p(C), max(n, 1), X.shape[1],
              _p(X), max(n, 1)))
    return X


def linear_solve(A, B, nb: int = 128, dtype=np.float64):
    """El::LinearSolve(A, B) (RowEchelon on [A|B], then the upper solve)."""
    A = _f(A, dtype)
    X = _f(B, dtype)
    n = A.shape[0]
    fn = getattr(lib(), "elo_linear_solve_" + _suffix(dtype))
    _check(fn(n, _p(A), max(n, 1), X.shape[1], _p(X), max(n, 1), nb))
    return X


def hpd_solve(A, B, uplo: str = "L", nb: int = 128, dtype=np.float64):
    A = _f(A, dtype)
    X = _f(B, dtype)
    n = A.shape[0]
    fn = getattr(lib(), "elo_hpd_solve_" + _suffix(dtype))
    _check(fn(ctypes.c_char(uplo.encode()), n, _p(A), max(n, 1), X.shape[1],
              _p(X), max(n, 1), nb))
    return X


# ---------------------------------------------------------------------------
# the reference itself (only where oracle/_ref/elref was built)
# ---------------------------------------------------------------------------
def lu_nopiv(A, nb: int = 128, dtype=np.float64):
    """El::LU(A) without pivoting (src/lapack_like/factor/LU.cpp:21-44): per
    nb-block, lu::Unb on the diagonal block (LU/Local.hpp:42-61: scale by
    1/alpha and a rank-1 update per column; an exact zero pivot raises
    OracleError(3), the reference's SingularMatrixException), then
    Trsm(RIGHT, UPPER, NORMAL, NON_UNIT) on A21, Trsm(LEFT, LOWER, NORMAL,
    UNIT) on A12 and Gemm(-1) on A22."""
    from scipy.linalg import solve_triangular

    W = np.array(A, dtype=dtype, order="F")
    m, n = W.shape
    mn = min(m, n)
    for k in range(0, mn, nb):
        b = min(nb, mn - k)
        A11 = W[k:k + b, k:k + b]
        for j in range(b):
            alpha = A11[j, j]
            if alpha == 0:
                raise OracleError(3)
            A11[j + 1:, j] *= dtype(1) / alpha
            A11[j + 1:, j + 1:] -= np.outer(A11[j + 1:, j], A11[j, j + 1:])
        if k + b < m:
            W[k + b:, k:k + b] = solve_triangular(np.triu(A11).T, W[k + b:, k:k + b].T,
                                                  lower=True).T
        if k + b < n:
            W[k:k + b, k + b:] = solve_triangular(A11, W[k:k + b, k + b:], lower=True,
                                                  unit_diagonal=True)
        if k + b < m and k + b < n:
            W[k + b:, k + b:] -= W[k + b:, k:k + b] @ W[k:k + b, k + b:]
    return W


def _sym_swap_lower(W, to, frm):
    """SymmetricSwap(LOWER, A, to, from) (src/blas_like/level1/Swap.cpp:243-301)
    on real data: bottom, inner (column segment <-> row segment), diagonal and
    left swaps; the corner A(from, to) stays."""
    if to == frm:
        return
    if to > frm:
        to, frm = frm, to
    n = W.shape[0]
    if frm + 1 < n:
        W[frm + 1:, [to, frm]] = W[frm + 1:, [frm, to]]
    if to + 1 < frm:
        a = W[to + 1:frm, to].copy()
        W[to + 1:frm, to] = W[frm, to + 1:frm]
        W[frm, to + 1:frm] = a
    W[to, to], W[frm, frm] = W[frm, frm], W[to, to]
    if to > 0:
        W[[to, frm], :to] = W[[frm, to], :to]


def cholesky_piv(A, uplo: str = "L", nb: int = 128, dtype=np.float64):
    """El::Cholesky(uplo, A, P) with diagonal pivoting (src/lapack_like/factor/
    Cholesky.cpp:44-52 -> Cholesky/PivotedLowerVariant3.hpp:206-255, 345-365):
    lazy panels of nb columns -- per column, the updated diagonal's largest
    magnitude (VectorMaxAbsLoc: first index on ties) picks the pivot,
    HermitianSwap on the lower triangle and on the panel's X / Y rows, the
    column caught up by Gemv with the panel's earlier columns, scaled by
    1/sqrt(pivot) -- then Trrk(LOWER) on the trailing block.  The upper
    variant is the same on the transpose.  At a panel's first column the
    reference's PanelFull reads X(i, -1) of an empty view (memory before the
    buffer); this restatement takes no update there.  With 8- or 16-column
    panels on a correlation matrix that read was measured non-zero on later
    panels and changed the reference's pivots; the fixtures use panel widths
    where it contributes nothing.
    Returns (factor in the uplo triangle, swap destinations)."""
    W = np.array(A, dtype=dtype, order="F")
    if uplo == "U":
        W = np.asfortranarray(W.T)
    n = W.shape[0]
    piv = np.zeros(n, dtype=np.int32)
    for off in range(0, n, nb):
        bs = min(nb, n - off)
        m = n - off
        X = np.zeros((m, bs), dtype=dtype)
        Y = np.zeros((m, bs), dtype=dtype)
        d = np.diag(W)[off:].copy()
        for k in range(bs):
            if k > 0:
                d[k:] -= X[k:, k - 1] * Y[k:, k - 1]
            a = np.abs(d[k:])
            rel = int(np.argmax(a)) if a.size and a.max() > 0 else 0
            frm = k + rel
            _sym_swap_lower(W, off + k, off + frm)
            piv[off + k] = off + frm
            d[[k, frm]] = d[[frm, k]]
            X[[k, frm], :k] = X[[frm, k], :k]
            Y[[k, frm], :k] = Y[[frm, k], :k]
            if k > 0:
                W[off + k:, off + k] -= X[k:, :k] @ Y[k, :k]
            delta = np.sqrt(W[off + k, off + k])
            W[off + k, off + k] = delta
            W[off + k + 1:, off + k] *= dtype(1) / delta
            X[k + 1:, k] = W[off + k + 1:, off + k]
            Y[k + 1:, k] = W[off + k + 1:, off + k]
        if off + bs < n:
            U = X[bs:, :] @ Y[bs:, :].T
            T22 = W[off + bs:, off + bs:]
            il = np.tril_indices(n - off - bs)
            T22[il] -= U[il]
    if uplo == "U":
        W = np.asfortranarray(W.T)
    return W, piv


def cholesky_piv_solve_after(C, piv, B, uplo: str = "L"):
    """cholesky::SolveAfter(uplo, orientation, A, P, B) (Cholesky/SolveAfter.hpp:
    46-76) on real data: P.PermuteRows(B), the two triangular solves,
    P.InversePermuteRows(B)."""
    from scipy.linalg import solve_triangular

    X = permute_rows(piv, np.array(B, dtype=C.dtype, order="F"))
    if uplo == "L":
        X = solve_triangular(C, X, lower=True)
        X = solve_triangular(C, X, lower=True, trans="T")
    else:
        X = solve_triangular(C, X, lower=False, trans="T")
        X = solve_triangular(C, X, lower=False)
    return permute_rows(piv, np.asfortranarray(X), inverse=True)


def lu_full(A, dtype=np.float64):
    """El::LU(A, P, Q) with full pivoting (src/lapack_like/factor/LU/Full.hpp:
    15-59): per step k, MaxAbsLoc of the trailing block (the first maximum
    in column-major order, strict '>' from 0 at (k, k) --
    src/blas_like/level1/MaxAbsLoc.cpp:131-163), RowSwap and ColSwap over the
    whole matrix, a21 *= 1/alpha, Geru(-1, a21, a12, A22) through the same
    BLAS routine (?ger of the SciPy OpenBLAS).  Returns (packed LU, row swap
    destinations, column swap destinations); an exact zero pivot raises
    OracleError(3)."""
    from scipy.linalg import blas

    W = np.array(A, dtype=dtype, order="F")
    m, n = W.shape
    mn = min(m, n)
    p = np.zeros(mn, dtype=np.int32)
    q = np.zeros(mn, dtype=np.int32)
    ger = blas.dger if W.dtype == np.float64 else blas.sger
    for k in range(mn):
        B = np.abs(W[k:, k:])
        flat = int(np.argmax(B.ravel(order="F")))  # first maximum, column-major
        i, j = flat % B.shape[0], flat // B.shape[0]
        if B[i, j] == 0:
            i = j = 0
        ip, jp = k + i, k + j
        p[k], q[k] = ip, jp
        if ip != k:
            W[[k, ip], :] = W[[ip, k], :]
        if jp != k:
            W[:, [k, jp]] = W[:, [jp, k]]
        alpha = W[k, k]
        if alpha == 0:
            raise OracleError(3)
        W[k + 1:, k] *= dtype(1) / alpha
        if k + 1 < m and k + 1 < n:
            W[k + 1:, k + 1:] = ger(-1.0, W[k + 1:, k], W[k, k + 1:], a=W[k + 1:, k + 1:])
    return W, p, q


def lu_full_solve_after(LU, p, q, B, orientation: int = 0):
    """lu::SolveAfter(orientation, A, P, Q, B) (LU/SolveAfter.hpp:120-145):
    NORMAL: P.PermuteRows(B), unit-lower then upper solve,
    Q.InversePermuteRows(B); TRANSPOSE: Q.PermuteRows(B), U^T then L^T
    solve, P.InversePermuteRows(B)."""
    from scipy.linalg import solve_triangular

    X = np.array(B, dtype=LU.dtype, order="F")
    if orientation == 0:
        X = permute_rows(p, X)
        X = solve_triangular(LU, X, lower=True, unit_diagonal=True)
        X = solve_triangular(LU, X, lower=False)
        return permute_rows(q, np.asfortranarray(X), inverse=True)
    X = permute_rows(q, X)
    X = solve_triangular(LU, X, lower=False, trans="T")
    X = solve_triangular(LU, X, lower=True, unit_diagonal=True, trans="T")
    return permute_rows(p, np.asfortranarray(X), inverse=True)


def inverse(A, nb: int = 128, dtype=np.float64):
    """El::Inverse(A) (src/lapack_like/funcs/Inverse/General/LUPartialPiv.hpp:
    21-74): El::LU(A, P) (the C restatement above), TriangularInverse(UPPER,
    NON_UNIT) on U, then from the last nb-block backwards: copy out L11 and
    L21, zero the strictly lower part of the block column A1, A1 -= A2 L21,
    A1 := A1 inv(L11) (Trsm RIGHT, LOWER, NORMAL, UNIT); finally
    inv(A) := inv(A) P, the swap sequence replayed backwards on the columns
    (InversePermuteCols).  A zero pivot raises OracleError(3)."""
    from scipy.linalg import solve_triangular

    W, piv = lu(A, nb, dtype)
    n = W.shape[0]
    if W.shape[1] != n:
        raise OracleError(2)
    eye = np.eye(n, dtype=dtype)
    W = np.asfortranarray(np.triu(solve_triangular(np.triu(W), eye, lower=False))
                          + np.tril(W, -1))
    for k in range(((n - 1) // nb) * nb if n else -1, -1, -nb):
        b = min(nb, n - k)
        L11 = np.tril(W[k:k + b, k:k + b], -1) + np.eye(b, dtype=dtype)
        L21 = W[k + b:, k:k + b].copy()
        W[k:k + b, k:k + b] = np.triu(W[k:k + b, k:k + b])
        W[k + b:, k:k + b] = 0
        if k + b < n:
            W[:, k:k + b] -= W[:, k + b:] @ L21
        W[:, k:k + b] = solve_triangular(L11.T, W[:, k:k + b].T, lower=False,
                                         unit_diagonal=True).T
    for i in range(len(piv) - 1, -1, -1):
        p = int(piv[i])
        if p != i:
            W[:, [i, p]] = W[:, [p, i]]
    return W


def one_condition(A, nb: int = 128, dtype=np.float64):
    """El::OneCondition(A) (src/lapack_like/props/Condition/One.cpp:12-24):
    OneNorm(A) * OneNorm(inv(A)), +inf when the inverse hits a zero pivot."""
    A = np.asarray(A, dtype=dtype)
    n1 = float(np.abs(A).sum(axis=0).max()) if A.size else 0.0
    try:
        X = inverse(A, nb, dtype)
    except OracleError as e:
        if e.status == 3:
            return float("inf")
        raise
    return n1 * float(np.abs(X).sum(axis=0).max()) if X.size else 0.0


def have_reference() -> bool:
    return os.path.exists(REF_EXE)


def write_el_binary(path, A):
    """Elemental's binary matrix layout: [Int h][Int w][column-major data]
    (src/io/Write/Binary.hpp:17-37), 32-bit Int."""
    A = np.asfortranarray(A)
    with open(path, "wb") as f:
        np.array(A.shape, dtype=np.int32).tofile(f)
        A.ravel(order="F").tofile(f)


def read_el_binary(path, dtype):
    with open(path, "rb") as f:
        h, w = np.fromfile(f, dtype=np.int32, count=2)
        d = np.fromfile(f, dtype=dtype, count=int(h) * int(w))
    return d.reshape((int(h), int(w)), order="F")


def ref_run(op, *args, dtype=np.float64, nb=128, inputs=(), out_dtypes=(),
            threads=1):
    """Runs the reference harness oracle/_ref/elref.  `inputs` are arrays
    written as Elemental binary files; `out_dtypes` gives one dtype per output
    file.  Returns (exit status, [output arrays])."""
    sfx = "d" if np.dtype(dtype) == np.float64 else "s"
    with tempfile.TemporaryDirectory() as d:
        ins = []
        for i, a in enumerate(inputs):
            p = os.path.join(d, f"in{i}")
            write_el_binary(p, np.asarray(a, dtype=dtype))
            ins.append(p)
        outs = [os.path.join(d, f"out{i}") for i in range(len(out_dtypes))]
        env = dict(os.environ, OPENBLAS_NUM_THREADS=str(threads))
        r = subprocess.run([REF_EXE, sfx, op, str(nb), *map(str, args), *ins,
                            *outs], env=env, capture_output=True, text=True)
        if r.returncode != 0:
            return r.returncode, []
        return 0, [read_el_binary(p, dt) for p, dt in zip(outs, out_dtypes)]


# ---------------------------------------------------------------------------
# metrics
# ---------------------------------------------------------------------------
def backward_error(A, X, B):
    """Normwise backward error ||B - A X|| / (||A|| ||X|| + ||B||), FP64:
    Frobenius norm for A, 2-norm per column for X and B, max over columns."""
    A = np.asarray(A, dtype=np.float64)
    X = np.asarray(X, dtype=np.float64).reshape(A.shape[1], -1)
    B = np.asarray(B, dtype=np.float64).reshape(A.shape[0], -1)
    R = B - A @ X
    nA = np.linalg.norm(A)
    num = np.linalg.norm(R, axis=0)
    den = nA * np.linalg.norm(X, axis=0) + np.linalg.norm(B, axis=0)
    return float(np.max(num / den))


def pivot_mismatches(piv_a, piv_b):
    piv_a = np.asarray(piv_a).ravel()
    piv_b = np.asarray(piv_b).ravel()
    return int(np.sum(piv_a != piv_b))


def tied_pivot_steps(A, piv, nb=128, ulps=1.0):
    """Steps k at which the reference's pivot candidate is tied (within `ulps`
    units in the last place) with another candidate in column k of the
    partially-eliminated matrix, recomputed by the oracle's own factorization.
    Returns the sorted list of such k."""
    W = _f(A, np.float64)
    m, n = W.shape
    ties = []
    # Replay the factorization one column at a time with the unblocked
    # right-looking schedule: |candidates| agree with the blocked schedule to
    # a few ulps, which is what the tie window is for.
    for k in range(min(m, n)):
        col = np.abs(W[k:, k])
        j = int(np.argmax(col))
        top = col[j]
        if top > 0:
            near = np.nonzero(np.abs(col - top) <= ulps * 4 * np.spacing(top))[0]
            if near.size > 1:
                ties.append(k)
        p = k + j
        if p != k:
            W[[k, p], :] = W[[p, k], :]
        if W[k, k] != 0:
            W[k + 1:, k] *= 1.0 / W[k, k]
            W[k + 1:, k + 1:] -= np.outer(W[k + 1:, k], W[k, k + 1:])
    return ties
