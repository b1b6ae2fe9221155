"""Device-level Python access to libelgb300.so for torch CUDA tensors.

Matrices are column-major, as El::Matrix: an m x n matrix is a torch tensor of
shape (m, n) with strides (1, ld), ld >= m — e.g. ``colmajor(m, n)`` or
``torch.empty(n, m).t()``.  Every call runs on torch's current CUDA stream of
the tensor's device, so it orders with surrounding torch work.  torch here is
only device memory and streams; the arithmetic is the library's kernels.
"""
from __future__ import annotations

import ctypes
import numpy as np

import torch

from . import _lib

_DT = {torch.float64: "d", torch.float32: "s"}

# ElGB precision / method codes (include/elgb300.h)
PRECISIONS = {"fp64": 0, "fp32": 1, "tf32": 2, "bf16": 3, "fp8": 4}
PRECISION_NAMES = {v: k for k, v in PRECISIONS.items()}
METHODS = {"lu-ir": 0, "gmres-ir": 1}
PROFILE_TAGS = {"tc_gemm": 0, "panel": 1, "swap": 2, "trsm": 3, "gemm_simt": 4,
                "residual": 5, "lowprec_solve": 6, "convert": 7}


class ElGBError(RuntimeError):
    pass


class SingularMatrixError(ElGBError):
    """The device path found an exact zero pivot (the reference throws
    SingularMatrixException, src/lapack_like/factor/LU/Panel.hpp:51-52)."""


class NonHPDMatrixError(ElGBError):
    """A non-positive Cholesky pivot (the reference throws
    NonHPDMatrixException, src/lapack_like/factor/Cholesky/LowerVariant3.hpp:29-30)."""


def colmajor(m, n, dtype=torch.float64, device="cuda", ld=None):
    ld = max(m, 1) if ld is None else ld
    return torch.empty((n, ld), dtype=dtype, device=device).t()[:m]


def to_colmajor(x):
    """Column-major copy of a 2-D tensor (or a view of it if already so)."""
    if x.dim() == 1:
        x = x.reshape(-1, 1)
    if x.stride(0) == 1 and (x.shape[1] <= 1 or x.stride(1) >= max(x.shape[0], 1)):
        return x
    return x.t().contiguous().t()


def _ld(x):
    if x.stride(0) != 1 and x.shape[0] > 1:
        raise ValueError("matrix must be column-major (stride(0) == 1)")
    return max(x.stride(1) if x.shape[1] > 1 else x.shape[0], 1)


def _ptr(x):
    return ctypes.c_void_p(x.data_ptr())


class Context:
    """One GPU, one stream binding, one scratch arena (ElGBContext)."""

    def __init__(self, device=None):
        self.lib = _lib.load()
        dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.device = dev
        h = ctypes.c_void_p()
        rc = self.lib.ElGBCreate(ctypes.byref(h), dev.index)
        if rc != 0:
            raise ElGBError(f"ElGBCreate failed ({rc})")
        self.h = h

    def close(self):
        if self.h:
            self.lib.ElGBDestroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _bind(self):
        s = torch.cuda.current_stream(self.device).cuda_stream
        self.lib.ElGBSetStream(self.h, ctypes.c_void_p(s))

    def _rc(self, rc, what):
        if rc != 0:
            raise ElGBError(f"{what} returned ElError {rc}")

    def status(self):
        """(info, err) of the last call; synchronizes the stream."""
        info, err = ctypes.c_int(), ctypes.c_int()
        self._rc(self.lib.ElGBStatus(self.h, ctypes.byref(info), ctypes.byref(err)), "status")
        return info.value, err.value

    def check(self, cholesky=False):
        info, err = self.status()
        if err:
            raise ElGBError(f"device-side bounded wait gave up (code {err})")
        if info:
            raise (NonHPDMatrixError if cholesky else SingularMatrixError)(
                f"info = {info}")

    def set_option(self, option, value):
        """ElGBSetOption: "lookahead" (0/1), "panel_ctas" (0 = auto) or
        "tournament" (0/1: tournament pivoting in lu_mixed's leaf panels)."""
        code = {"lookahead": 1, "panel_ctas": 2, "tournament": 3, "panel_cluster": 4,
                "panel_regs": 5, "residual_df": 6, "panel_trace": 7, "trail_grid": 8,
                "panel_rows": 9, "trail_split": 10, "inv_trsm": 11, "swap_stream": 12, "panel_push": 13, "panel_pdl": 14, "side_tc_min_n": 15, "panel_node": 16}[option]
        self._rc(self.lib.ElGBSetOption(self.h, code, int(value)), "SetOption")

    def panel_trace(self, ncols):
        """Per-column leaf-panel timestamps of the last factorization (see
        ELGB_OPT_PANEL_TRACE): int64 array (ncols, 4), ns."""
        import numpy as np

        out = np.zeros((ncols, 4), dtype=np.uint64)
        self._rc(self.lib.ElGBPanelTrace(self.h, out.ctypes.data_as(ctypes.c_void_p), ncols),
                 "PanelTrace")
        return out.astype(np.int64)

    def launches(self):
        return int(self.lib.ElGBLaunchCount(self.h))

    def profile_start(self, tags=None):
        """Brackets every launch group (tags None) or only the named kernel
        families (PROFILE_TAGS keys) with CUDA events until profile_stop."""
        if tags is None:
            self._rc(self.lib.ElGBProfileStart(self.h), "ProfileStart")
        else:
            mask = 0
            for t in tags:
                mask |= 1 << PROFILE_TAGS[t]
            self._rc(self.lib.ElGBProfileStartTags(self.h, mask), "ProfileStartTags")

    def profile_stop(self):
        """Summed event timing of the tensor-core GEMM launches since
        profile_start: dict(launches, ms, flops, bytes)."""
        n, ms, fl, by = ctypes.c_longlong(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._rc(self.lib.ElGBProfileStop(self.h, ctypes.byref(n), ctypes.byref(ms),
                                          ctypes.byref(fl), ctypes.byref(by)), "ProfileStop")
        out = dict(launches=n.value, ms=ms.value, flops=fl.value, bytes=by.value)
        tags = {}
        for name, tag in PROFILE_TAGS.items():
            self._rc(self.lib.ElGBProfileTag(self.h, tag, ctypes.byref(n), ctypes.byref(ms),
                                             ctypes.byref(fl), ctypes.byref(by)), "ProfileTag")
            tags[name] = dict(launches=n.value, ms=ms.value)
        out["by_kernel"] = tags
        side = {}
        for name, tag in PROFILE_TAGS.items():
            self._rc(self.lib.ElGBProfileTag(self.h, tag + 8, ctypes.byref(n), ctypes.byref(ms),
                                             ctypes.byref(fl), ctypes.byref(by)), "ProfileTag")
            if n.value:
                side[name] = dict(launches=n.value, ms=ms.value)
                if name == "tc_gemm":
                    out["flops_lookahead_tc"] = fl.value
        out["by_kernel_lookahead_stream"] = side
        return out

    def profile_records(self):
        """After profile_stop: every event-bracketed launch group in issue
        order as a structured array (start_ms, dur_ms, tag, side), the start
        relative to the first group."""
        cnt = ctypes.c_int()
        self._rc(self.lib.ElGBProfileRecords(self.h, 0, ctypes.byref(cnt), None, None, None,
                                             None), "ProfileRecords")
        n = cnt.value
        start = np.zeros(n, np.float32)
        dur = np.zeros(n, np.float32)
        tag = np.zeros(n, np.int32)
        side = np.zeros(n, np.int32)
        if n:
            self._rc(self.lib.ElGBProfileRecords(
                self.h, n, ctypes.byref(cnt), start.ctypes.data_as(ctypes.c_void_p),
                dur.ctypes.data_as(ctypes.c_void_p), tag.ctypes.data_as(ctypes.c_void_p),
                side.ctypes.data_as(ctypes.c_void_p)), "ProfileRecords")
        out = np.zeros(n, dtype=[("start_ms", "f4"), ("dur_ms", "f4"), ("tag", "i4"),
                                 ("side", "i4")])
        out["start_ms"], out["dur_ms"], out["tag"], out["side"] = start, dur, tag, side
        return out

    # -- the path -----------------------------------------------------------
    def lu(self, A, piv=None, nb=0):
        """El::LU(A, P) in place; returns the int32 swap destinations."""
        m, n = A.shape
        if piv is None:
            piv = torch.empty(min(m, n), dtype=torch.int32, device=A.device)
        self._bind()
        s = _DT[A.dtype]
        self._rc(getattr(self.lib, f"ElGBLUPartialPiv_{s}")(self.h, m, n, _ptr(A), _ld(A),
                                                            _ptr(piv), nb), "LU")
        return piv

    def lu_mixed(self, A, gemm_kind=2, piv=None, nb=0):
        """El::LU on an FP32 matrix with tensor-core updates (gemm_kind:
        -1 SIMT FP32, 0 BF16, 1 TF32, 2 TF32x3, 3 FP8 E4M3 trailing updates
        with per-panel scales)."""
        m, n = A.shape
        assert A.dtype == torch.float32
        if piv is None:
            piv = torch.empty(min(m, n), dtype=torch.int32, device=A.device)
        self._bind()
        self._rc(self.lib.ElGBLUPartialPivMixed_s(self.h, m, n, _ptr(A), _ld(A), _ptr(piv), nb,
                                                  gemm_kind), "LUMixed")
        return piv

    def gemm_sub_tc(self, A, B, C, gemm_kind=0):
        """C -= A @ B on the tensor cores (FP32 column-major tensors)."""
        m, k = A.shape
        n = B.shape[1]
        self._bind()
        self._rc(self.lib.ElGBGemmSubTC(self.h, gemm_kind, m, n, k, _ptr(A), _ld(A), _ptr(B),
                                        _ld(B), _ptr(C), _ld(C)), "GemmSubTC")
        return C

    def refined_solve(self, A, B, X=None, precision="fp32", method="lu-ir", tol=0.0,
                      max_iters=0, restart=0, fallback=True, nb=0, pivoting="partial"):
        """Mixed-precision solve A X = B (FP64 in/out): low-precision LU on the
        tensor cores (partial pivoting as El::LU, or "tournament" pivoting of
        the leaf panels) + LU-IR or GMRES-IR with an FP64 residual, FP64 LU
        as the fallback.  Returns (X, info dict)."""
        n, q = B.shape
        if X is None:
            X = colmajor(n, q, torch.float64, A.device)
        ctrl = _lib.RefineCtrl(PRECISIONS[precision], METHODS[method], float(tol),
                               int(max_iters), int(restart), 1 if fallback else 0, int(nb),
                               {"partial": 0, "tournament": 1}[pivoting])
        inf = _lib.RefineInfo()
        self._bind()
        self._rc(self.lib.ElGBRefinedSolve_d(self.h, n, _ptr(A), _ld(A), q, _ptr(B), _ld(B),
                                             _ptr(X), _ld(X), ctypes.byref(ctrl),
                                             ctypes.byref(inf)), "RefinedSolve")
        return X, dict(iterations=inf.iterations, converged=bool(inf.converged),
                       fell_back=bool(inf.fell_back),
                       precision=PRECISION_NAMES[inf.precision],
                       backward_error=inf.backward_error)

    def lu_nopiv(self, A, nb=0):
        """El::LU(A) without pivoting, in place (ElGBLUNoPiv_*)."""
        m, n = A.shape
        self._bind()
        self._rc(getattr(self.lib, f"ElGBLUNoPiv_{_DT[A.dtype]}")(self.h, m, n, _ptr(A), _ld(A),
                                                                  nb), "LUNoPiv")
        return A

    def lu_full(self, A, p=None, q=None):
        """El::LU(A, P, Q) with full pivoting, in place; returns the int32
        row and column swap destinations (ElGBLUFullPiv_*)."""
        m, n = A.shape
        k = min(m, n)
        p = torch.empty(k, dtype=torch.int32, device=A.device) if p is None else p
        q = torch.empty(k, dtype=torch.int32, device=A.device) if q is None else q
        self._bind()
        self._rc(getattr(self.lib, f"ElGBLUFullPiv_{_DT[A.dtype]}")(
            self.h, m, n, _ptr(A), _ld(A), _ptr(p), _ptr(q)), "LUFullPiv")
        return p, q

    def lu_full_solve_after(self, A, p, q, B, orientation=0):
        n = A.shape[0]
        self._bind()
        self._rc(getattr(self.lib, f"ElGBSolveAfterLUFullPiv_{_DT[A.dtype]}")(
            self.h, orientation, n, _ptr(A), _ld(A), _ptr(p), _ptr(q), B.shape[1], _ptr(B),
            _ld(B)), "SolveAfterLUFullPiv")
        return B

    def cholesky_piv(self, A, uplo=0, piv=None):
        """El::Cholesky(uplo, A, P) with diagonal pivoting, in place; returns
        the int32 swap destinations (ElGBCholeskyPiv_*)."""
        n = A.shape[0]
        piv = torch.empty(n, dtype=torch.int32, device=A.device) if piv is None else piv
        self._bind()
        self._rc(getattr(self.lib, f"ElGBCholeskyPiv_{_DT[A.dtype]}")(
            self.h, uplo, n, _ptr(A), _ld(A), _ptr(piv)), "CholeskyPiv")
        return piv

    def cholesky_piv_solve_after(self, A, piv, B, uplo=0):
        self._bind()
        self._rc(getattr(self.lib, f"ElGBSolveAfterCholeskyPiv_{_DT[A.dtype]}")(
            self.h, uplo, A.shape[0], _ptr(A), _ld(A), _ptr(piv), B.shape[1], _ptr(B), _ld(B)),
            "SolveAfterCholeskyPiv")
        return B

    def inverse(self, A, nb=0):
        """El::Inverse(A): A := inv(A) in place (ElGBInverse_*)."""
        n = A.shape[0]
        self._bind()
        self._rc(getattr(self.lib, f"ElGBInverse_{_DT[A.dtype]}")(self.h, n, _ptr(A), _ld(A), nb),
                 "Inverse")
        return A

    def one_condition(self, A, nb=0):
        """El::OneCondition(A) = ||A||_1 ||inv(A)||_1 (+inf when singular);
        A is not modified (ElGBOneCondition_*)."""
        n = A.shape[0]
        out = ctypes.c_double()
        self._bind()
        self._rc(getattr(self.lib, f"ElGBOneCondition_{_DT[A.dtype]}")(
            self.h, n, _ptr(A), _ld(A), nb, ctypes.byref(out)), "OneCondition")
        return out.value

    def lu_solve_after(self, A, piv, B, orientation=0):
        n = A.shape[0]
        self._bind()
        s = _DT[A.dtype]
        self._rc(getattr(self.lib, f"ElGBSolveAfterLUPartialPiv_{s}")(
            self.h, orientation, n, _ptr(A), _ld(A), _ptr(piv), B.shape[1], _ptr(B), _ld(B)),
            "SolveAfterLU")
        return B

    def cholesky(self, A, uplo=0, nb=0):
        self._bind()
        s = _DT[A.dtype]
        self._rc(getattr(self.lib, f"ElGBCholesky_{s}")(self.h, uplo, A.shape[0], _ptr(A),
                                                        _ld(A), nb), "Cholesky")
        return A

    def cholesky_solve_after(self, A, B, uplo=0):
        self._bind()
        s = _DT[A.dtype]
        self._rc(getattr(self.lib, f"ElGBSolveAfterCholesky_{s}")(
            self.h, uplo, A.shape[0], _ptr(A), _ld(A), B.shape[1], _ptr(B), _ld(B)),
            "SolveAfterCholesky")
        return B

    def linear_solve(self, A, B, nb=0):
        self._bind()
        s = _DT[A.dtype]
        self._rc(getattr(self.lib, f"ElGBLinearSolve_{s}")(
            self.h, A.shape[0], _ptr(A), _ld(A), B.shape[1], _ptr(B), _ld(B), nb),
            "LinearSolve")
        return B

    def hpd_solve(self, A, B, uplo=0, nb=0):
        self._bind()
        s = _DT[A.dtype]
        self._rc(getattr(self.lib, f"ElGBHPDSolve_{s}")(
            self.h, uplo, A.shape[0], _ptr(A), _ld(A), B.shape[1], _ptr(B), _ld(B), nb),
            "HPDSolve")
        return B

    def residual(self, A, X, B, R=None):
        n, q = B.shape
        if R is None:
            R = colmajor(n, q, torch.float64, A.device)
        self._bind()
        self._rc(self.lib.ElGBResidual_d(self.h, n, q, _ptr(A), _ld(A), _ptr(X), _ld(X),
                                         _ptr(B), _ld(B), _ptr(R), _ld(R)), "Residual")
        return R

    def residual_df(self, A, X, B=None, R=None):
        """R = B - A X (B None: R = A X) to FP64 accuracy in double-float
        arithmetic on the FP32 pipe (ElGBResidualDF_d)."""
        n, q = X.shape
        if R is None:
            R = colmajor(n, q, torch.float64, A.device)
        self._bind()
        bp, bl = (_ptr(B), _ld(B)) if B is not None else (None, n)
        self._rc(self.lib.ElGBResidualDF_d(self.h, n, q, _ptr(A), _ld(A), _ptr(X), _ld(X),
                                           bp, bl, _ptr(R), _ld(R)), "ResidualDF")
        return R

    def backward_error(self, A, X, B):
        n, q = B.shape
        out = ctypes.c_double()
        self._bind()
        self._rc(self.lib.ElGBBackwardError_d(self.h, n, q, _ptr(A), _ld(A), _ptr(X), _ld(X),
                                              _ptr(B), _ld(B), ctypes.byref(out)),
                 "BackwardError")
        return out.value

    def fp64_peak_tflops(self):
        out = ctypes.c_double()
        self._bind()
        self._rc(self.lib.ElGBProbeFP64Peak(self.h, ctypes.byref(out)), "probe")
        return out.value


_default = {}


def context(device=None) -> Context:
    idx = torch.cuda.current_device() if device is None else device
    if idx not in _default:
        _default[idx] = Context(idx)
    return _default[idx]
