"""GB300-native drop-in for Elemental's sequential dense factor-and-solve path.

The host-side mirror of the reference's Python interface for this path
(python/lapack_like/factor.py:34,149,525,662; python/lapack_like/solve.py:49,217;
python/core/Matrix.py, python/core/Permutation.py): the same names and
argument meanings, over the same C ABI (include/El_gb300.h) — here backed by
libelgb300.so's sm_103a kernels.  Matrices are host numpy arrays in
column-major (Fortran) order, as El::Matrix; errors surface as the
exceptions the reference maps its ElError codes to.

Device-resident work (torch CUDA tensors, no host copies) goes through
``elemental_gb300.device``.
"""
from __future__ import annotations

import ctypes
import sys

import numpy as np

from . import _lib

# Enumerations (include/El/core/types.h:211-228)
NORMAL, TRANSPOSE, ADJOINT = 0, 1, 2
LOWER, UPPER = 0, 1
# Matrix file formats (python/core/environment.py, include/El/core/types.h:237-251)
(AUTO, ASCII, ASCII_MATLAB, BINARY, BINARY_FLAT, BMP, JPG, JPEG, MATRIX_MARKET, PNG, PPM, XBM,
 XPM) = range(13)
# LU pivot types (python/lapack_like/factor.py:493)
LU_PARTIAL, LU_FULL, LU_ROOK, LU_WITHOUT_PIVOTING = 0, 1, 2, 3

_TAG = {np.dtype(np.int32): "i", np.dtype(np.float32): "s", np.dtype(np.float64): "d"}


class ElError(RuntimeError):
    def __init__(self, code, what=""):
        self.code = code
        super().__init__(f"{what}: {_lib.load().ElErrorString(code).decode()} ({code})")


class SingularMatrixException(ElError):
    pass


def _check(rc, what, singular_cls=None):
    if rc == 0:
        return
    if rc == 5 and singular_cls is not None:
        raise singular_cls(rc, what)
    raise ElError(rc, what)


class Matrix:
    """A host El::Matrix<T> handle attached to a column-major numpy array."""

    def __init__(self, array):
        a = np.asfortranarray(array)
        if a.ndim == 1:
            a = a.reshape(-1, 1, order="F")
        if a.dtype not in _TAG:
            raise TypeError(f"unsupported dtype {a.dtype}")
        self.array = a
        self.tag = _TAG[a.dtype]
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        _check(getattr(self.lib, f"ElMatrixCreate_{self.tag}")(ctypes.byref(h)), "Create")
        self.obj = h
        m, n = a.shape
        _check(getattr(self.lib, f"ElMatrixAttach_{self.tag}")(
            h, m, n, a.ctypes.data_as(ctypes.c_void_p), max(m, 1)), "Attach")

    def Height(self):
        return self.array.shape[0]

    def Width(self):
        return self.array.shape[1]

    def ToNumPy(self):
        return self.array

    def __getitem__(self, idx):
        """A[I, J] with integers or unit-step slices: a view sharing this
        matrix's memory (El::View through ElView_*), as the reference's
        Matrix.__getitem__ (python/core/Matrix.py:456-482).  Factoring or
        permuting the view changes the parent in place."""
        i, j = idx

        def bounds(s, n):
            if isinstance(s, (int, np.integer)):
                return int(s), int(s) + 1
            if not isinstance(s, slice) or s.step not in (None, 1):
                raise IndexError("views take integers or unit-step slices")
            b, e, _ = s.indices(n)
            return b, max(b, e)

        (i0, i1), (j0, j1) = bounds(i, self.Height()), bounds(j, self.Width())
        V = Matrix.__new__(Matrix)
        V.array = self.array[i0:i1, j0:j1]
        V.tag, V.lib, V._parent = self.tag, self.lib, self
        h = ctypes.c_void_p()
        _check(getattr(self.lib, f"ElMatrixCreate_{self.tag}")(ctypes.byref(h)), "Create")
        V.obj = h
        _check(getattr(self.lib, f"ElView_{self.tag}")(h, self.obj, _lib.Range(i0, i1),
                                                      _lib.Range(j0, j1)), "View")
        return V

    def __del__(self):
        try:
            getattr(self.lib, f"ElMatrixDestroy_{self.tag}")(self.obj)
        except Exception:
            pass


class Permutation:
    """El::Permutation, a swap sequence (python/core/Permutation.py:56-187)."""

    def __init__(self):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        _check(self.lib.ElPermutationCreate(ctypes.byref(h)), "PermutationCreate")
        self.obj = h
        self._dests = np.zeros(0, dtype=np.int32)

    def Empty(self):
        _check(self.lib.ElPermutationEmpty(self.obj), "Empty")
        self._dests = np.zeros(0, dtype=np.int32)

    def MakeIdentity(self, size):
        _check(self.lib.ElPermutationMakeIdentity(self.obj, int(size)), "MakeIdentity")
        self._dests = np.zeros(0, dtype=np.int32)

    def ReserveSwaps(self, maxSwaps):
        _check(self.lib.ElPermutationReserveSwaps(self.obj, int(maxSwaps)), "ReserveSwaps")

    def Swap(self, origin, dest):
        _check(self.lib.ElPermutationSwap(self.obj, int(origin), int(dest)), "Swap")
        self._dests = np.append(self._dests, np.int32(dest))

    def SwapSequence(self, PAppend, offset=0):
        appended = PAppend._dests + int(offset)
        _check(self.lib.ElPermutationSwapSequence(self.obj, PAppend.obj, int(offset)),
               "SwapSequence")
        self._dests = np.concatenate([self._dests, appended]).astype(np.int32)

    def Height(self):
        v = ctypes.c_int()
        _check(self.lib.ElPermutationHeight(self.obj, ctypes.byref(v)), "Height")
        return v.value

    def Width(self):
        v = ctypes.c_int()
        _check(self.lib.ElPermutationWidth(self.obj, ctypes.byref(v)), "Width")
        return v.value

    def _flag(self, name):
        v = ctypes.c_bool()
        _check(getattr(self.lib, name)(self.obj, ctypes.byref(v)), name)
        return bool(v.value)

    def Parity(self):
        return self._flag("ElPermutationParity")

    def IsSwapSequence(self):
        return self._flag("ElPermutationIsSwapSequence")

    def IsImplicitSwapSequence(self):
        return self._flag("ElPermutationIsImplicitSwapSequence")

    def ExplicitVector(self):
        n = self.Height()
        p = Matrix(np.zeros((n, 1), dtype=np.int32))
        _check(self.lib.ElPermutationExplicitVector(self.obj, p.obj), "ExplicitVector")
        return p.array.ravel().copy()

    def SwapDestinations(self):
        """The destinations of the recorded swaps, in order (as
        Permutation::SwapDestinations, src/lapack_like/perm/Permutation.cpp:444-450)."""
        return self._dests.copy()

    def PermuteRows(self, A: Matrix, offset=0):
        _check(getattr(self.lib, f"ElPermutationPermuteRows_{A.tag}")(self.obj, A.obj, offset),
               "PermuteRows")

    def __del__(self):
        try:
            self.lib.ElPermutationDestroy(self.obj)
        except Exception:
            pass


def _swap_dests_from_explicit(p):
    """Recovers a swap sequence (implicit origins) equivalent to the explicit
    permutation vector p (P A = A(p, :))."""
    n = len(p)
    cur = np.arange(n)
    pos = np.arange(n)  # pos[row label] = current position
    dests = np.empty(n, dtype=np.int32)
    for i in range(n):
        j = pos[p[i]]
        dests[i] = j
        a, b = cur[i], cur[j]
        cur[i], cur[j] = b, a
        pos[a], pos[b] = j, i
    return dests


def Blocksize():
    v = ctypes.c_int()
    _check(_lib.load().ElBlocksize(ctypes.byref(v)), "Blocksize")
    return v.value


def SetBlocksize(nb):
    _check(_lib.load().ElSetBlocksize(int(nb)), "SetBlocksize")


def PushBlocksizeStack(nb):
    _check(_lib.load().ElPushBlocksizeStack(int(nb)), "PushBlocksizeStack")


def PopBlocksizeStack():
    _check(_lib.load().ElPopBlocksizeStack(), "PopBlocksizeStack")


def LU(A: Matrix, pivType=LU_PARTIAL):
    """El.LU(A, pivType) (python/lapack_like/factor.py:525-552): A is
    overwritten by the packed L\\U.  Partial pivoting returns the
    Permutation, LU_FULL the pair (P, Q); LU_WITHOUT_PIVOTING (ElLU_*)
    returns None and raises SingularMatrixException at an exact zero pivot."""
    if pivType == LU_WITHOUT_PIVOTING:
        _check(getattr(A.lib, f"ElLU_{A.tag}")(A.obj), "LU", SingularMatrixException)
        return None
    if pivType == LU_FULL:  # returns (P, Q) (python/lapack_like/factor.py:543-552)
        P, Q = Permutation(), Permutation()
        _check(getattr(A.lib, f"ElLUFullPiv_{A.tag}")(A.obj, P.obj, Q.obj), "LU",
               SingularMatrixException)
        k = min(A.Height(), A.Width())
        P._dests = _swap_dests_from_explicit(P.ExplicitVector())[:k]
        Q._dests = _swap_dests_from_explicit(Q.ExplicitVector())[:k]
        return P, Q
    if pivType != LU_PARTIAL:
        raise ValueError("rook pivoting is not on this path")
    P = Permutation()
    _check(getattr(A.lib, f"ElLUPartialPiv_{A.tag}")(A.obj, P.obj), "LU", SingularMatrixException)
    P._dests = _swap_dests_from_explicit(P.ExplicitVector())[: min(A.Height(), A.Width())]
    return P


def SolveAfterLUPartialPiv(orient, A: Matrix, P: Permutation, B: Matrix):
    _check(getattr(A.lib, f"ElSolveAfterLUPartialPiv_{A.tag}")(orient, A.obj, P.obj, B.obj),
           "SolveAfterLUPartialPiv")


def SolveAfterLUFullPiv(orient, A: Matrix, P: Permutation, Q: Permutation, B: Matrix):
    _check(getattr(A.lib, f"ElSolveAfterLUFullPiv_{A.tag}")(orient, A.obj, P.obj, Q.obj,
                                                            B.obj), "SolveAfterLUFullPiv")


def Cholesky(uplo, A: Matrix, piv=False):
    """El.Cholesky(uplo, A, piv) (python/lapack_like/factor.py:34-60); with
    piv=True, diagonal pivoting (ElCholeskyPiv_*) and the Permutation is
    returned."""
    if piv:
        P = Permutation()
        _check(getattr(A.lib, f"ElCholeskyPiv_{A.tag}")(uplo, A.obj, P.obj), "Cholesky")
        P._dests = _swap_dests_from_explicit(P.ExplicitVector())[: A.Height()]
        return P
    _check(getattr(A.lib, f"ElCholesky_{A.tag}")(uplo, A.obj), "Cholesky",
           SingularMatrixException)


def SolveAfterCholeskyPiv(uplo, orient, A: Matrix, P: Permutation, B: Matrix):
    _check(getattr(A.lib, f"ElSolveAfterCholeskyPiv_{A.tag}")(uplo, orient, A.obj, P.obj,
                                                              B.obj), "SolveAfterCholeskyPiv")


def SolveAfterCholesky(uplo, orient, A: Matrix, B: Matrix):
    _check(getattr(A.lib, f"ElSolveAfterCholesky_{A.tag}")(uplo, orient, A.obj, B.obj),
           "SolveAfterCholesky")


def Read(A: Matrix, filename, fileFormat=AUTO, sequential=False):
    """El.Read(A, filename, fileFormat) (python/io.py:377-): BINARY (.bin) or
    BINARY_FLAT (.dat, into A's current shape); A is resized to the file's
    matrix and its numpy array replaced by the data read.  `sequential`
    concerns distributed matrices only and is ignored."""
    lib, t = A.lib, A.tag
    # A's C++ matrix views the numpy array (it cannot be resized), so the
    # file is read into an owned matrix first
    tmp = ctypes.c_void_p()
    _check(getattr(lib, f"ElMatrixCreate_{t}")(ctypes.byref(tmp)), "Create")
    try:
        _check(getattr(lib, f"ElMatrixResize_{t}")(tmp, A.Height(), A.Width()), "Resize")
        _check(getattr(lib, f"ElRead_{t}")(tmp, str(filename).encode(), int(fileFormat)), "Read")
        h, w, ld, buf = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_void_p()
        getattr(lib, f"ElMatrixHeight_{t}")(tmp, ctypes.byref(h))
        getattr(lib, f"ElMatrixWidth_{t}")(tmp, ctypes.byref(w))
        getattr(lib, f"ElMatrixLDim_{t}")(tmp, ctypes.byref(ld))
        getattr(lib, f"ElMatrixBuffer_{t}")(tmp, ctypes.byref(buf))
        dt = A.array.dtype
        arr = np.empty((h.value, w.value), dtype=dt, order="F")
        if arr.size:
            ptr = ctypes.cast(buf, ctypes.POINTER(np.ctypeslib.as_ctypes_type(dt)))
            raw = np.ctypeslib.as_array(ptr, shape=(w.value * ld.value,))
            arr[:] = raw.reshape(w.value, ld.value)[:, : h.value].T
    finally:
        getattr(lib, f"ElMatrixDestroy_{t}")(tmp)
    A.array = arr
    _check(getattr(A.lib, f"ElMatrixAttach_{A.tag}")(
        A.obj, h.value, w.value, arr.ctypes.data_as(ctypes.c_void_p), max(h.value, 1)),
        "Attach")


def Write(A: Matrix, basename="matrix", fileFormat=BINARY, title=""):
    """El.Write(A, basename, fileFormat, title) (python/io.py:424-): writes
    basename.bin (BINARY) or basename.dat (BINARY_FLAT)."""
    _check(getattr(A.lib, f"ElWrite_{A.tag}")(A.obj, str(basename).encode(), int(fileFormat),
                                              str(title).encode()), "Write")


def Inverse(A: Matrix):
    """El.Inverse(A) (python/lapack_like/funcs.py:85-98): A := inv(A);
    SingularMatrixException at an exact zero pivot."""
    _check(getattr(A.lib, f"ElInverse_{A.tag}")(A.obj), "Inverse", SingularMatrixException)


def OneCondition(A: Matrix):
    """El.OneCondition(A) (python/lapack_like/props.py:144-158): ||A||_1
    ||inv(A)||_1, +inf for a singular A."""
    cond = (ctypes.c_double if A.tag == "d" else ctypes.c_float)()
    _check(getattr(A.lib, f"ElOneCondition_{A.tag}")(A.obj, ctypes.byref(cond)),
           "OneCondition")
    return cond.value


def LinearSolve(A: Matrix, B: Matrix):
    _check(getattr(A.lib, f"ElLinearSolve_{A.tag}")(A.obj, B.obj), "LinearSolve",
           SingularMatrixException)


def HPDSolve(A: Matrix, B: Matrix, uplo=LOWER, orient=NORMAL):
    _check(getattr(A.lib, f"ElHPDSolve_{A.tag}")(uplo, orient, A.obj, B.obj), "HPDSolve",
           SingularMatrixException)


def LinearSolveMixed(A: Matrix, B: Matrix, precision="fp32", method="lu-ir", tol=0.0,
                     max_iters=0, restart=0, fallback=True, nb=0):
    """Added form: El.LinearSolve on host matrices through the mixed-precision
    path (ElLinearSolveMixed_d); returns the refinement info as a dict."""
    from .device import METHODS, PRECISION_NAMES, PRECISIONS

    ctrl = _lib.RefineCtrl(PRECISIONS[precision], METHODS[method], float(tol), int(max_iters),
                           int(restart), 1 if fallback else 0, int(nb))
    inf = _lib.RefineInfo()
    _check(A.lib.ElLinearSolveMixed_d(A.obj, B.obj, ctypes.byref(ctrl), ctypes.byref(inf)),
           "LinearSolveMixed", SingularMatrixException)
    return dict(iterations=inf.iterations, converged=bool(inf.converged),
                fell_back=bool(inf.fell_back), precision=PRECISION_NAMES[inf.precision],
                backward_error=inf.backward_error)


class _HostBlock:
    """Owner of one ElGBHostAlloc block; frees it when the last array using
    it goes away."""

    def __init__(self, nbytes):
        lib = _lib.load()
        p = ctypes.c_void_p()
        _check(lib.ElGBHostAlloc(nbytes, ctypes.byref(p)), "HostAlloc")
        self.ptr = p.value
        self.nbytes = nbytes

    def __del__(self):
        # not during interpreter shutdown: the CUDA runtime may already be
        # torn down, and the process's pages go back to the system anyway
        if getattr(self, "ptr", None) and not sys.is_finalizing():
            _lib.load().ElGBHostFree(self.ptr)
        self.ptr = None


def host_empty(shape, dtype=np.float64, order="F"):
    """numpy array in ElGBHostAlloc memory (registered with the CUDA driver),
    for matrices that move to and from the GPU: attach El.Matrix to it (order
    "F", the column-major layout of El::Matrix)."""
    shape = tuple(int(d) for d in np.atleast_1d(shape))
    dt = np.dtype(dtype)
    nbytes = int(np.prod(shape)) * dt.itemsize
    if nbytes == 0:
        return np.empty(shape, dtype=dt, order=order)
    blk = _HostBlock(nbytes)
    buf = (ctypes.c_char * nbytes).from_address(blk.ptr)
    buf._owner = blk  # the block lives as long as a view of the buffer
    return np.ndarray(shape, dtype=dt, buffer=buf, order=order)


def LastHostCallTimes():
    """Host-side phases of the last completed host-matrix call (ms): upload,
    device work (with its synchronisation), download."""
    lib = _lib.load()
    v = [ctypes.c_double() for _ in range(3)]
    _check(lib.ElGBLastHostCallTimes(*[ctypes.byref(x) for x in v]), "LastHostCallTimes")
    return {"upload_ms": v[0].value, "compute_ms": v[1].value, "download_ms": v[2].value}
