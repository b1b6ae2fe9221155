"""Batched uneven-size solves (added form 2) from Python: packs a list of
systems into the device layout of ElGBBatchedPlanCreate (include/elgb300.h),
keeps the plan (descriptors, workspaces, CUDA graph) and replays it."""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .device import Context, context

KIND = {"lu": 0, "chol": 1}
PREC = {"fp64": 0, "fp32": 1, "bf16": 2}
# refinement of low-precision factors: LU-IR then flexible GMRES-IR when it
# stalls ("auto"), LU-IR only, or FGMRES-IR only
METHOD = {"auto": 0, "lu-ir": 1, "gmres-ir": 2}


class BatchedSolver:
    """Solve A_i X_i = B_i for many small systems in one persistent launch.

    systems: list of (A_i (n_i x n_i), B_i (n_i x q)) numpy FP64 arrays, or
    pre-packed device tensors via from_packed().  kinds / precisions: lists of
    "lu" / "chol" and "fp32" / "fp64".
    """

    def __init__(self, ns, q, A_packed, B_packed, kinds=None, precisions=None, nb_table=None,
                 ctas_per_sm=1, tol=1e-13, max_iters=10, fallback=True, features_only=False,
                 method="auto", gmres_restart=0, gmres_max_iters=0, precision_device=None,
                 phases=False, selector_params=None, simt_update=False,
                 ctx: Context | None = None):
        self.ctx = ctx or context()
        self.lib = _lib.load()
        self.ns = np.ascontiguousarray(ns, dtype=np.int32)
        self.count = len(self.ns)
        self.q = q
        self.A = A_packed
        self.B = B_packed
        self.X = torch.empty_like(B_packed)
        self.features = (torch.empty(len(ns), 16, dtype=torch.float32, device=A_packed.device)
                         if features_only or selector_params is not None else None)
        self.selector_params = selector_params
        k = np.ascontiguousarray([KIND[x] for x in kinds] if kinds is not None
                                 else np.zeros(self.count), dtype=np.int32)
        pr = np.ascontiguousarray([PREC[x] for x in precisions] if precisions is not None
                                  else np.ones(self.count), dtype=np.int32)
        self.kinds, self.precs = k, pr
        nbt = None
        if nb_table is not None:
            nbt = np.ascontiguousarray(nb_table, dtype=np.int32)
        h = ctypes.c_void_p()
        vp = ctypes.c_void_p
        opt = _lib.BatchOptions(
            k.ctypes.data_as(vp).value, pr.ctypes.data_as(vp).value,
            nbt.ctypes.data_as(vp).value if nbt is not None else None, int(ctas_per_sm),
            float(tol), int(max_iters), 0 if fallback else 1, 1 if features_only else 0,
            self.features.data_ptr() if self.features is not None else None, METHOD[method],
            int(gmres_restart), int(gmres_max_iters),
            precision_device.data_ptr() if precision_device is not None else None,
            None)
        self.precision_device = precision_device
        self.phase_ns = None
        if phases:
            self.phase_ns = torch.zeros(self.count, len(self.PHASES), dtype=torch.int64,
                                        device=A_packed.device)
            opt.phase_ns = self.phase_ns.data_ptr()
        if selector_params is not None:
            opt.selector_params = selector_params.data_ptr()
        opt.simt_update = 1 if simt_update else 0
        self._keep = (k, pr, nbt)
        rc = self.lib.ElGBBatchedPlanCreate(
            self.ctx.h, self.count, self.ns.ctypes.data_as(vp), q, vp(self.A.data_ptr()),
            vp(self.B.data_ptr()), vp(self.X.data_ptr()), ctypes.byref(opt), ctypes.byref(h))
        if rc != 0:
            raise RuntimeError(f"ElGBBatchedPlanCreate returned {rc}")
        self.h = h

    @staticmethod
    def pack(systems, q, device="cuda"):
        """systems: list of (A, B) numpy arrays -> (ns, A_packed, B_packed)."""
        ns = [a.shape[0] for a, _ in systems]
        A = np.concatenate([np.asfortranarray(a).ravel(order="F") for a, _ in systems])
        B = np.concatenate([np.asfortranarray(b.reshape(b.shape[0], q)).ravel(order="F")
                            for _, b in systems])
        return ns, torch.from_numpy(A).to(device), torch.from_numpy(B).to(device)

    @staticmethod
    def subset(ns, q, A_packed, B_packed, idx):
        """The systems `idx` (sorted indices) of a packed batch, repacked:
        (ns, A, B) for a rank's share (elemental_gb300.shard)."""
        ns = np.asarray(ns, dtype=np.int64)
        aoff = np.concatenate([[0], np.cumsum(ns ** 2)])
        boff = np.concatenate([[0], np.cumsum(ns * q)])
        A = torch.cat([A_packed[aoff[i]:aoff[i + 1]] for i in idx]) if len(idx) else A_packed[:0]
        B = torch.cat([B_packed[boff[i]:boff[i + 1]] for i in idx]) if len(idx) else B_packed[:0]
        return ns[idx].astype(np.int32), A, B

    def run(self):
        """Enqueue one replay of the captured launch on the context stream."""
        self.ctx._bind()
        rc = self.lib.ElGBBatchedExecute(self.h)
        if rc != 0:
            raise RuntimeError(f"ElGBBatchedExecute returned {rc}")

    def results(self):
        out = (_lib.BatchResult * self.count)()
        rc = self.lib.ElGBBatchedResults(self.h, out)
        if rc != 0:
            raise RuntimeError(f"ElGBBatchedResults returned {rc}")
        return [dict(iterations=r.iterations, converged=bool(r.converged),
                     fell_back=bool(r.fell_back), info=r.info,
                     backward_error=r.backward_error, gmres_iterations=r.gmres_iterations,
                     precision=r.precision, device_ms=r.device_ns * 1e-6,
                     selector_choice=r.selector_choice) for r in out]

    PHASES = ("panel", "swaps", "u12_solve", "trailing_update", "lu_ir", "fgmres_ir",
              "fp64_path", "features", "ir_residual", "ir_lowprec_solve")

    def phase_ms(self):
        """Per-system device time by phase (requires phases=True): dict of
        numpy arrays in ms."""
        ph = self.phase_ns.cpu().numpy() * 1e-6
        return {k: ph[:, i] for i, k in enumerate(self.PHASES)}

    def solution(self, i):
        off = int(np.sum(self.ns[:i].astype(np.int64))) * self.q
        n = int(self.ns[i])
        return self.X[off:off + n * self.q].reshape(self.q, n).t().cpu().numpy()

    def flops(self):
        return float(self.lib.ElGBBatchedFlops(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.ElGBBatchedPlanDestroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
