"""Loads libelgb300.so (built in-tree by elemental_gb300.build) and declares
the ctypes signatures of its two C interfaces: the Elemental-compatible one
(include/El_gb300.h) and the device-level one (include/elgb300.h).

There is no fallback: if the library is missing or fails to load, importing
raises, so nothing silently runs on the CPU.
"""
from __future__ import annotations

import ctypes
import os

from .build import LIB

_lib = None

c_int, c_double, c_void_p, c_char_p = ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_char_p
c_ll = ctypes.c_longlong
P = ctypes.POINTER


class RefineCtrl(ctypes.Structure):
    """ElGBRefineCtrl (include/elgb300.h)."""
    _fields_ = [("precision", c_int), ("method", c_int), ("tol", c_double),
                ("max_iters", c_int), ("restart", c_int), ("fallback", c_int), ("nb", c_int),
                ("pivoting", c_int)]


class RefineInfo(ctypes.Structure):
    """ElGBRefineInfo (include/elgb300.h)."""
    _fields_ = [("iterations", c_int), ("converged", c_int), ("fell_back", c_int),
                ("precision", c_int), ("backward_error", c_double)]


class BatchResult(ctypes.Structure):
    """ElGBBatchResult (include/elgb300.h)."""
    _fields_ = [("iterations", c_int), ("converged", c_int), ("fell_back", c_int),
                ("info", c_int), ("backward_error", c_double), ("gmres_iterations", c_int),
                ("precision", c_int), ("device_ns", ctypes.c_longlong),
                ("selector_choice", c_int), ("reserved", c_int)]


class BatchOptions(ctypes.Structure):
    """ElGBBatchOptions (include/elgb300.h)."""
    _fields_ = [("kind", c_void_p), ("precision", c_void_p), ("nb_table", c_void_p),
                ("ctas_per_sm", c_int), ("tol", c_double), ("max_iters", c_int),
                ("no_fallback", c_int), ("features_only", c_int), ("features", c_void_p),
                ("method", c_int), ("gmres_restart", c_int), ("gmres_max_iters", c_int),
                ("precision_device", c_void_p), ("phase_ns", c_void_p),
                ("selector_params", c_void_p), ("simt_update", c_int)]


class Range(ctypes.Structure):
    """ElRange_i (reference include/El/core/types.h:36): rows / columns
    [beg, end); end = -100 (El::END) is the full extent."""

    _fields_ = [("beg", ctypes.c_int), ("end", ctypes.c_int)]


def _sig(lib, name, res, *args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = list(args)


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        raise ImportError(
            f"libelgb300.so not built ({LIB}); run "
            "`python -c 'import __graft_entry__ as g; g.build()'` first")
    lib = ctypes.CDLL(LIB, mode=ctypes.RTLD_GLOBAL)
    vp = c_void_p
    # device-level interface
    _sig(lib, "ElGBCreate", c_int, P(vp), c_int)
    _sig(lib, "ElGBDestroy", c_int, vp)
    _sig(lib, "ElGBSetStream", c_int, vp, vp)
    _sig(lib, "ElGBSynchronize", c_int, vp)
    _sig(lib, "ElGBStatus", c_int, vp, P(c_int), P(c_int))
    _sig(lib, "ElGBBlocksize", c_int)
    _sig(lib, "ElGBSetBlocksize", c_int, c_int)
    _sig(lib, "ElGBLaunchCount", c_ll, vp)
    _sig(lib, "ElGBSetOption", c_int, vp, c_int, c_int)
    _sig(lib, "ElGBPanelTrace", c_int, vp, vp, c_int)
    _sig(lib, "ElGBProfileStart", c_int, vp)
    _sig(lib, "ElGBProfileStartTags", c_int, vp, ctypes.c_uint)
    _sig(lib, "ElGBProfileStop", c_int, vp, P(c_ll), P(c_double), P(c_double), P(c_double))
    _sig(lib, "ElGBProfileTag", c_int, vp, c_int, P(c_ll), P(c_double), P(c_double),
         P(c_double))
    _sig(lib, "ElGBProfileRecords", c_int, vp, c_int, P(c_int), vp, vp, vp, vp)
    for s in ("d", "s"):
        _sig(lib, f"ElGBLUPartialPiv_{s}", c_int, vp, c_int, c_int, vp, c_int, vp, c_int)
        _sig(lib, f"ElGBSolveAfterLUPartialPiv_{s}", c_int, vp, c_int, c_int, vp, c_int, vp,
             c_int, vp, c_int)
        _sig(lib, f"ElGBCholesky_{s}", c_int, vp, c_int, c_int, vp, c_int, c_int)
        _sig(lib, f"ElGBSolveAfterCholesky_{s}", c_int, vp, c_int, c_int, vp, c_int, c_int, vp,
             c_int)
        _sig(lib, f"ElGBLinearSolve_{s}", c_int, vp, c_int, vp, c_int, c_int, vp, c_int, c_int)
        _sig(lib, f"ElGBHPDSolve_{s}", c_int, vp, c_int, c_int, vp, c_int, c_int, vp, c_int,
             c_int)
        _sig(lib, f"ElGBLUNoPiv_{s}", c_int, vp, c_int, c_int, vp, c_int, c_int)
        _sig(lib, f"ElGBLUFullPiv_{s}", c_int, vp, c_int, c_int, vp, c_int, vp, vp)
        _sig(lib, f"ElGBCholeskyPiv_{s}", c_int, vp, c_int, c_int, vp, c_int, vp)
        _sig(lib, f"ElGBSolveAfterCholeskyPiv_{s}", c_int, vp, c_int, c_int, vp, c_int, vp,
             c_int, vp, c_int)
        _sig(lib, f"ElGBSolveAfterLUFullPiv_{s}", c_int, vp, c_int, c_int, vp, c_int, vp, vp,
             c_int, vp, c_int)
        _sig(lib, f"ElGBInverse_{s}", c_int, vp, c_int, vp, c_int, c_int)
        _sig(lib, f"ElGBOneCondition_{s}", c_int, vp, c_int, vp, c_int, c_int, P(c_double))
    _sig(lib, "ElGBLUPartialPivMixed_s", c_int, vp, c_int, c_int, vp, c_int, vp, c_int, c_int)
    _sig(lib, "ElGBGemmSubTC", c_int, vp, c_int, c_int, c_int, c_int, vp, c_int, vp, c_int, vp,
         c_int)
    _sig(lib, "ElGBRefinedSolve_d", c_int, vp, c_int, vp, c_int, c_int, vp, c_int, vp, c_int,
         P(RefineCtrl), P(RefineInfo))
    _sig(lib, "ElGBResidual_d", c_int, vp, c_int, c_int, vp, c_int, vp, c_int, vp, c_int, vp,
         c_int)
    _sig(lib, "ElGBResidualDF_d", c_int, vp, c_int, c_int, vp, c_int, vp, c_int, vp, c_int, vp,
         c_int)
    _sig(lib, "ElGBMLPParamCount", c_int)
    _sig(lib, "ElGBMLPForward", c_int, vp, vp, vp, c_int, vp, vp)
    _sig(lib, "ElGBMLPGradient", c_int, vp, vp, vp, vp, c_int, vp, P(ctypes.c_float))
    _sig(lib, "ElGBMLPAdamStep", c_int, vp, vp, vp, vp, vp, ctypes.c_float, ctypes.c_float,
         ctypes.c_float, ctypes.c_float, ctypes.c_float, c_int)
    _sig(lib, "ElGBBatchedPlanCreate", c_int, vp, c_int, vp, c_int, vp, vp, vp,
         P(BatchOptions), P(vp))
    _sig(lib, "ElGBBatchedExecute", c_int, vp)
    _sig(lib, "ElGBBatchedResults", c_int, vp, vp)
    _sig(lib, "ElGBBatchedFlops", c_double, vp)
    _sig(lib, "ElGBBatchedPlanDestroy", c_int, vp)
    _sig(lib, "ElGBResidualNoAlloc_d", c_int, c_int, c_int, vp, c_int, vp, c_int, vp, c_int, vp,
         c_int, vp)
    _sig(lib, "ElGBBackwardError_d", c_int, vp, c_int, c_int, vp, c_int, vp, c_int, vp, c_int,
         P(c_double))
    _sig(lib, "ElGBProbeFP64Peak", c_int, vp, P(c_double))
    # Elemental-compatible interface
    for s in ("i", "s", "d"):
        _sig(lib, f"ElMatrixCreate_{s}", c_int, P(vp))
        _sig(lib, f"ElMatrixDestroy_{s}", c_int, vp)
        _sig(lib, f"ElMatrixAttach_{s}", c_int, vp, c_int, c_int, vp, c_int)
        _sig(lib, f"ElMatrixLockedAttach_{s}", c_int, vp, c_int, c_int, vp, c_int)
        _sig(lib, f"ElMatrixResize_{s}", c_int, vp, c_int, c_int)
        _sig(lib, f"ElMatrixHeight_{s}", c_int, vp, P(c_int))
        _sig(lib, f"ElRead_{s}", c_int, vp, ctypes.c_char_p, c_int)
        _sig(lib, f"ElWrite_{s}", c_int, vp, ctypes.c_char_p, c_int, ctypes.c_char_p)
        _sig(lib, f"ElMatrixWidth_{s}", c_int, vp, P(c_int))
        _sig(lib, f"ElMatrixLDim_{s}", c_int, vp, P(c_int))
        _sig(lib, f"ElMatrixBuffer_{s}", c_int, vp, P(vp))
        _sig(lib, f"ElView_{s}", c_int, vp, vp, Range, Range)
        _sig(lib, f"ElLockedView_{s}", c_int, vp, vp, Range, Range)
    _sig(lib, "ElPermutationCreate", c_int, P(vp))
    _sig(lib, "ElPermutationDestroy", c_int, vp)
    _sig(lib, "ElPermutationHeight", c_int, vp, P(c_int))
    _sig(lib, "ElPermutationWidth", c_int, vp, P(c_int))
    _sig(lib, "ElPermutationEmpty", c_int, vp)
    _sig(lib, "ElPermutationMakeIdentity", c_int, vp, c_int)
    _sig(lib, "ElPermutationReserveSwaps", c_int, vp, c_int)
    _sig(lib, "ElPermutationSwap", c_int, vp, c_int, c_int)
    _sig(lib, "ElPermutationSwapSequence", c_int, vp, vp, c_int)
    _sig(lib, "ElPermutationParity", c_int, vp, P(ctypes.c_bool))
    _sig(lib, "ElPermutationIsSwapSequence", c_int, vp, P(ctypes.c_bool))
    _sig(lib, "ElPermutationIsImplicitSwapSequence", c_int, vp, P(ctypes.c_bool))
    _sig(lib, "ElPermutationExplicitVector", c_int, vp, vp)
    _sig(lib, "ElPermutationPermuteRows_d", c_int, vp, vp, c_int)
    _sig(lib, "ElPermutationPermuteRows_s", c_int, vp, vp, c_int)
    _sig(lib, "ElErrorString", c_char_p, c_int)
    _sig(lib, "ElBlocksize", c_int, P(c_int))
    _sig(lib, "ElSetBlocksize", c_int, c_int)
    _sig(lib, "ElPushBlocksizeStack", c_int, c_int)
    _sig(lib, "ElPopBlocksizeStack", c_int)
    for s in ("s", "d"):
        _sig(lib, f"ElLUPartialPiv_{s}", c_int, vp, vp)
        _sig(lib, f"ElLU_{s}", c_int, vp)
        _sig(lib, f"ElLUFullPiv_{s}", c_int, vp, vp, vp)
        _sig(lib, f"ElCholeskyPiv_{s}", c_int, c_int, vp, vp)
        _sig(lib, f"ElSolveAfterCholeskyPiv_{s}", c_int, c_int, c_int, vp, vp, vp)
        _sig(lib, f"ElSolveAfterLUFullPiv_{s}", c_int, c_int, vp, vp, vp, vp)
        _sig(lib, f"ElInverse_{s}", c_int, vp)
        _sig(lib, f"ElOneCondition_{s}", c_int, vp,
             P(ctypes.c_double if s == "d" else ctypes.c_float))
        _sig(lib, f"ElSolveAfterLUPartialPiv_{s}", c_int, c_int, vp, vp, vp)
        _sig(lib, f"ElCholesky_{s}", c_int, c_int, vp)
        _sig(lib, f"ElSolveAfterCholesky_{s}", c_int, c_int, c_int, vp, vp)
        _sig(lib, f"ElLinearSolve_{s}", c_int, vp, vp)
        _sig(lib, f"ElHPDSolve_{s}", c_int, c_int, c_int, vp, vp)
    _sig(lib, "ElLinearSolveMixed_d", c_int, vp, vp, P(RefineCtrl), P(RefineInfo))
    _sig(lib, "ElGBLastHostCallTimes", c_int, P(ctypes.c_double), P(ctypes.c_double),
         P(ctypes.c_double))
    _sig(lib, "ElGBHostAlloc", c_int, ctypes.c_size_t, P(vp))
    _sig(lib, "ElGBHostFree", c_int, vp)
    _lib = lib
    return lib


def exported_symbols_from_headers():
    """Names of every function declared in include/*.h (for export checks)."""
    import re

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    inc = os.path.join(root, "include")
    names = set()
    for f in sorted(os.listdir(inc)):
        if not f.endswith(".h"):
            continue
        txt = open(os.path.join(inc, f)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        # expand the per-type macro blocks
        for m in re.finditer(r"#define (EL_GB_\w+)\(S, T\)(.*?)\n(?=\S)", txt, flags=re.S):
            body = m.group(2)
            for use in re.finditer(r"^" + m.group(1) + r"\((\w), [\w ]+\)", txt, flags=re.M):
                for fn in re.findall(r"(\w+)##S\(", body):
                    names.add(fn + use.group(1))
        for fn in re.findall(r"^\s*(?:const\s+)?\w[\w\s\*]*?\b(El\w+)\s*\(", txt, flags=re.M):
            if "##" not in fn:
                names.add(fn)
    return sorted(names)
