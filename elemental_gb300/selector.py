"""Learned precision selection (added form 3).

A 16 -> 64 -> 64 -> 3 FP32 MLP (mlp.cu's hand-written kernels) maps cheap
per-matrix features to the lowest factorization precision whose refinement
converges:

    class 0  FP64 factors (the plain path)
    class 1  FP32 factors + FP64 refinement
    class 2  BF16 operand products (FP32 storage) + FP64 refinement

The class index is the batched solver's precision code, so the network's
argmax (written on the device by ElGBMLPForward) is handed to the batched
plan as its run-time precision array: features -> MLP -> solve run as three
device launches with no host round trip.  Whatever the choice, refinement
that stalls falls back BF16 -> FP32 -> FP64, so the FP64 LU is both the
fallback and, through its FP64 residual, the arbiter of every result's error.

Training data are outcomes the solver itself generates: every training
system is solved once per low precision with the fallback switched off, and
its label is the lowest precision that reached the target backward error.

The features (batched.cu, compute_features) come from one FP32 LU of each
system: log2 n, a Hager/Higham estimate of kappa_1, norm ratios
||A||_1, ||A||_inf, max|a| over ||A||_F, the FP32 LU's growth and pivot
spread, and the estimator's own diagnostics.

Reference semantics: the refinement the labels come from follows
include/El/lapack_like/solve/Refined.hpp:44-119 (keep an update only if it
lowers the residual) and FGMRES.hpp:37-290; the condition estimate follows
the 1-norm estimator behind src/lapack_like/props/Condition/One.cpp:12-24.
"""
from __future__ import annotations

import ctypes
import json

import numpy as np
import torch

from . import _lib
from .batched import BatchedSolver
from .device import context

CLASSES = ("fp64", "fp32", "bf16")
NFEAT = 16
# unit roundoffs of the factor precisions (the kappa-threshold rule's theory
# thresholds are 1 / u_f: LU-IR converges while kappa * u_f < 1)
UNIT_ROUNDOFF = {"fp32": 2.0 ** -24, "bf16": 2.0 ** -8}


# ---------------------------------------------------------------------------
# seeded workloads: A = U diag(sigma) V^T, U, V Haar, kappa log-uniform
# ---------------------------------------------------------------------------
def conditioned_systems(count, seed, nmin=64, nmax=2048, kmin=1e1, kmax=1e12, nrhs=1,
                        device="cuda"):
    """`count` systems with n log-uniform in [nmin, nmax] and cond_2(A)
    log-uniform in [kmin, kmax]: A = U diag(sigma) V^T with sigma geometric
    from 1 to 1/kappa (Haar.cpp:14-21 construction for U, V: Q of the QR of
    a Gaussian, sign-fixed).  One Haar pair is drawn per distinct n and each
    system of that size uses it under its own random signed column
    permutations (still Haar-distributed per system).  The QR runs in FP32;
    the product is formed in FP64, so cond_2(A) = kappa to ~1e-5 relative.
    B iid N(0, 1).  Returns a dict with ns, kappa, packed A and B (device
    FP64, column-major per system, consecutive)."""
    rng = np.random.default_rng(int(seed))
    ns = np.floor(np.exp(rng.uniform(np.log(nmin), np.log(nmax + 1), count))).astype(np.int32)
    ns = np.clip(ns, nmin, nmax)
    kappa = np.exp(rng.uniform(np.log(kmin), np.log(kmax), count))
    a_off = np.concatenate([[0], np.cumsum(ns.astype(np.int64) ** 2)])
    b_off = np.concatenate([[0], np.cumsum(ns.astype(np.int64) * nrhs)])
    A = torch.empty(int(a_off[-1]), dtype=torch.float64, device=device)
    B = torch.empty(int(b_off[-1]), dtype=torch.float64, device=device)
    g = torch.Generator(device=device).manual_seed(int(seed))
    by_n = {}
    for i, n in enumerate(ns):
        by_n.setdefault(int(n), []).append(i)
    for n, idx in by_n.items():
        UV = []
        for _ in range(2):
            G = torch.randn(n, n, generator=g, device=device, dtype=torch.float32)
            Q, R = torch.linalg.qr(G)
            UV.append((Q * torch.sign(torch.diagonal(R))[None, :]).double())
        U, V = UV
        for i in idx:
            p1 = torch.randperm(n, generator=g, device=device)
            p2 = torch.randperm(n, generator=g, device=device)
            s1 = torch.randint(0, 2, (n,), generator=g, device=device).double() * 2 - 1
            s2 = torch.randint(0, 2, (n,), generator=g, device=device).double() * 2 - 1
            sig = torch.pow(torch.tensor(float(kappa[i]), dtype=torch.float64, device=device),
                            -torch.arange(n, device=device, dtype=torch.float64) / max(n - 1, 1))
            Ai = (U[:, p1] * (s1 * sig)[None, :]) @ (V[:, p2] * s2[None, :]).t()
            # column-major packing: the transpose's row-major bytes
            A[a_off[i]:a_off[i + 1]] = Ai.t().contiguous().view(-1)
    B[:] = torch.randn(B.numel(), generator=g, device=device, dtype=torch.float64)
    return dict(ns=ns, kappa=kappa, A=A, B=B, nrhs=nrhs, seed=int(seed))


# ---------------------------------------------------------------------------
# features and solver outcomes
# ---------------------------------------------------------------------------
def extract_features(systems, ctx=None, nb_table=None):
    """The 16 features of every system (one batched launch).  Returns
    (features (count x 16 FP32, device), kappa_1 estimates (numpy), ms)."""
    ctx = ctx or context()
    solver = BatchedSolver(systems["ns"], systems["nrhs"], systems["A"], systems["B"],
                           features_only=True, nb_table=nb_table, ctx=ctx)
    try:
        ms = _timed(ctx, solver.run)
        est = np.array([r["backward_error"] for r in solver.results()])
        return solver.features.clone(), est, ms
    finally:
        solver.close()


def solve_with(systems, precisions, fallback=True, method="auto", ctx=None, nb_table=None,
               tol=1e-13, precision_device=None, gmres_max_iters=0):
    """Solve every system with the given per-system precision names (or a
    device int32 array of codes); returns (results, ms, X)."""
    ctx = ctx or context()
    solver = BatchedSolver(systems["ns"], systems["nrhs"], systems["A"], systems["B"],
                           precisions=precisions, fallback=fallback, method=method,
                           nb_table=nb_table, tol=tol, precision_device=precision_device,
                           gmres_max_iters=gmres_max_iters, ctx=ctx)
    try:
        ms = _timed(ctx, solver.run)
        return solver.results(), ms, solver.X
    finally:
        solver.close()


def outcome_labels(systems, ctx=None, nb_table=None, tol=1e-13, gmres_max_iters=0):
    """Label of each system: the lowest precision (highest class code) whose
    refinement reached `tol` with the fallback switched off."""
    count = len(systems["ns"])
    labels = np.zeros(count, dtype=np.int32)
    info = {}
    for code in (1, 2):
        res, ms, _ = solve_with(systems, [CLASSES[code]] * count, fallback=False, ctx=ctx,
                                nb_table=nb_table, tol=tol, gmres_max_iters=gmres_max_iters)
        ok = np.array([r["converged"] for r in res])
        labels[ok] = code
        info[CLASSES[code]] = dict(ms=ms, converged=int(ok.sum()))
    return labels, info


# ---------------------------------------------------------------------------
# the network
# ---------------------------------------------------------------------------
def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _timed(ctx, fn):
    torch.cuda.synchronize()
    s = torch.cuda.Event(enable_timing=True)
    e = torch.cuda.Event(enable_timing=True)
    s.record()
    fn()
    e.record()
    e.synchronize()
    return s.elapsed_time(e)


class PrecisionSelector:
    """The 16 -> 64 -> 64 -> 3 MLP, trained and run by the library's own
    kernels (ElGBMLPGradient / ElGBMLPAdamStep / ElGBMLPForward).  Feature
    standardisation is folded into the first layer after training, so the
    deployed network reads raw features."""

    SHAPES = (("W1", (16, 64)), ("b1", (64,)), ("W2", (64, 64)), ("b2", (64,)),
              ("W3", (64, 3)), ("b3", (3,)))

    def __init__(self, seed=0, ctx=None):
        self.ctx = ctx or context()
        self.lib = _lib.load()
        self.nparam = self.lib.ElGBMLPParamCount()
        rng = np.random.default_rng(int(seed))
        th = []
        for _, shp in self.SHAPES:
            if len(shp) == 2:
                th.append((rng.standard_normal(shp) * np.sqrt(2.0 / shp[0])).ravel())
            else:
                th.append(np.zeros(shp))
        self.params = torch.from_numpy(np.concatenate(th).astype(np.float32)).cuda()
        assert self.params.numel() == self.nparam
        self.mean = np.zeros(NFEAT, np.float32)
        self.std = np.ones(NFEAT, np.float32)
        self.folded = False
        self.history = []

    # -- training ------------------------------------------------------------
    def fit(self, features, labels, epochs=200, batch=512, lr=3e-3, weight_decay=1e-4, seed=0,
            class_weight=None):
        """Adam on the mean cross-entropy.  features: (N, 16) FP32 device
        tensor; labels: (N,) int.  class_weight (3,): optional per-class
        sample replication factors to offset imbalance (integers)."""
        X = features.float()
        y = torch.as_tensor(np.asarray(labels, dtype=np.int32), device=X.device)
        if class_weight is not None:
            reps = torch.as_tensor(np.asarray(class_weight, dtype=np.int64), device=X.device)
            r = reps[y.long()]
            idx = torch.repeat_interleave(torch.arange(len(y), device=X.device), r)
            X, y = X[idx], y[idx]
        xs = X.cpu().numpy().astype(np.float64)
        self.mean = xs.mean(0).astype(np.float32)
        self.std = np.maximum(xs.std(0), 1e-3).astype(np.float32)
        Xn = ((X - torch.from_numpy(self.mean).to(X.device)) /
              torch.from_numpy(self.std).to(X.device)).contiguous()
        N = Xn.shape[0]
        grad = torch.zeros_like(self.params)
        m = torch.zeros_like(self.params)
        v = torch.zeros_like(self.params)
        g = torch.Generator(device=X.device).manual_seed(int(seed))
        self.ctx._bind()
        step = 0
        loss = ctypes.c_float()
        for ep in range(epochs):
            perm = torch.randperm(N, generator=g, device=X.device)
            for b0 in range(0, N, batch):
                sel = perm[b0:b0 + batch]
                xb = Xn[sel].contiguous()
                yb = y[sel].contiguous()
                rc = self.lib.ElGBMLPGradient(self.ctx.h, _p(self.params), _p(xb), _p(yb),
                                              int(sel.numel()), _p(grad), None)
                if rc != 0:
                    raise RuntimeError(f"ElGBMLPGradient returned {rc}")
                step += 1
                rc = self.lib.ElGBMLPAdamStep(self.ctx.h, _p(self.params), _p(grad), _p(m),
                                              _p(v), lr, 0.9, 0.999, 1e-8, weight_decay, step)
                if rc != 0:
                    raise RuntimeError(f"ElGBMLPAdamStep returned {rc}")
            if ep == epochs - 1 or ep % 20 == 0:
                rc = self.lib.ElGBMLPGradient(self.ctx.h, _p(self.params), _p(Xn), _p(y), N,
                                              _p(grad), ctypes.byref(loss))
                if rc != 0:
                    raise RuntimeError(f"ElGBMLPGradient returned {rc}")
                self.history.append((ep, float(loss.value)))
        self._fold()
        return self

    def _fold(self):
        """W1' = W1 / std (row-wise), b1' = b1 - (mean / std) W1."""
        th = self.params.double().cpu().numpy()
        W1 = th[:16 * 64].reshape(16, 64)
        b1 = th[16 * 64:16 * 64 + 64]
        s = self.std.astype(np.float64)[:, None]
        mu = self.mean.astype(np.float64)[:, None]
        b1 = b1 - ((mu / s) * W1).sum(0)
        W1 = W1 / s
        th[:16 * 64] = W1.ravel()
        th[16 * 64:16 * 64 + 64] = b1
        self.params = torch.from_numpy(th.astype(np.float32)).cuda()
        self.mean[:] = 0
        self.std[:] = 1
        self.folded = True

    # -- inference -----------------------------------------------------------
    def predict_device(self, features, out=None, probs=None):
        """argmax class per row of `features` into a device int32 tensor
        (one ElGBMLPForward launch; no host synchronisation)."""
        B = features.shape[0]
        if out is None:
            out = torch.empty(B, dtype=torch.int32, device=features.device)
        self.ctx._bind()
        rc = self.lib.ElGBMLPForward(self.ctx.h, _p(self.params), _p(features.contiguous()), B,
                                     _p(probs) if probs is not None else None, _p(out))
        if rc != 0:
            raise RuntimeError(f"ElGBMLPForward returned {rc}")
        return out

    def predict(self, features):
        return self.predict_device(features).cpu().numpy()

    # -- persistence ----------------------------------------------------------
    def save(self, path):
        np.savez(path, params=self.params.cpu().numpy(), folded=self.folded,
                 history=np.array(self.history, dtype=np.float64).reshape(-1, 2))

    @classmethod
    def load(cls, path, ctx=None):
        z = np.load(path)
        sel = cls(ctx=ctx)
        sel.params = torch.from_numpy(z["params"].astype(np.float32)).cuda()
        sel.folded = bool(z["folded"])
        return sel


# ---------------------------------------------------------------------------
# the rule it is compared with
# ---------------------------------------------------------------------------
LOG10_KAPPA_FEATURE = 1  # features[:, 1] = log10 of the kappa_1 estimate


def kappa_rule(log10_kappa, t_bf16, t_fp32):
    """Fixed kappa-threshold rule on the condition estimate: BF16 below
    t_bf16, FP32 below t_fp32, else FP64.  Works on numpy or torch."""
    if isinstance(log10_kappa, torch.Tensor):
        lk = log10_kappa
        return torch.where(lk < np.log10(t_bf16), 2,
                           torch.where(lk < np.log10(t_fp32), 1, 0)).to(torch.int32)
    lk = np.asarray(log10_kappa)
    return np.where(lk < np.log10(t_bf16), 2, np.where(lk < np.log10(t_fp32), 1, 0)).astype(
        np.int32)


THEORY_THRESHOLDS = (1.0 / UNIT_ROUNDOFF["bf16"], 1.0 / UNIT_ROUNDOFF["fp32"])


def rule_network(t_bf16, t_fp32, slope=1e4, device="cuda"):
    """The kappa-threshold rule written as parameters of the same 16-64-64-3
    network, so that it runs through the identical fused select-and-solve
    launch: with f = features[1] = log10 kappa_est, a = log10 t_bf16,
    b = log10 t_fp32, h0 = relu(f - a), h1 = relu(f - b) and logits
    (FP64, FP32, BF16) = (-2 + 2 M h1, -1, -M h0).  The argmax is BF16 for
    f < a, FP32 for a < f < b and FP64 for f > b, exactly except within
    1/M decades of a threshold."""
    a, b = float(np.log10(t_bf16)), float(np.log10(t_fp32))
    W1 = np.zeros((16, 64)); b1 = np.zeros(64)
    W1[LOG10_KAPPA_FEATURE, 0] = 1.0; b1[0] = -a
    W1[LOG10_KAPPA_FEATURE, 1] = 1.0; b1[1] = -b
    W2 = np.zeros((64, 64)); b2 = np.zeros(64)
    W2[0, 0] = 1.0; W2[1, 1] = 1.0
    W3 = np.zeros((64, 3)); b3 = np.array([-2.0, -1.0, 0.0])
    W3[1, 0] = 2.0 * slope
    W3[0, 2] = -slope
    th = np.concatenate([W1.ravel(), b1, W2.ravel(), b2, W3.ravel(), b3]).astype(np.float32)
    return torch.from_numpy(th).to(device)


def solve_selected(systems, params, ctx=None, nb_table=None, tol=1e-13, phases=False,
                   gmres_max_iters=0):
    """The fused select-and-solve launch: per system, features from an FP32
    LU (kept), the network `params`' class, then the solve in that
    precision (BF16 / FP32 classes refine with the kept FP32 factors, FP64
    refactors; refinement that stalls falls back to FP64).  Returns
    (results, ms, solver) -- close() the solver when done."""
    ctx = ctx or context()
    solver = BatchedSolver(systems["ns"], systems["nrhs"], systems["A"], systems["B"],
                           selector_params=params, nb_table=nb_table, tol=tol, phases=phases,
                           gmres_max_iters=gmres_max_iters, ctx=ctx)
    ms = _timed(ctx, solver.run)
    return solver.results(), ms, solver


def fit_kappa_rule(log10_kappa, labels):
    """Best fixed thresholds (label accuracy) on training data, over a grid
    of 0.25-decade steps."""
    lk = np.asarray(log10_kappa)
    grid = np.arange(0.0, 16.01, 0.25)
    best = (-1.0, None)
    for a in grid:
        for b in grid[grid >= a]:
            acc = float((kappa_rule(lk, 10 ** a, 10 ** b) == labels).mean())
            if acc > best[0]:
                best = (acc, (10 ** a, 10 ** b))
    return best[1], best[0]


def summarize(results, ms, label=None):
    be = np.array([r["backward_error"] for r in results])
    return dict(ms=ms, solves_per_s=len(results) / (ms * 1e-3),
                max_backward_error=float(be.max()) if len(be) else 0.0,
                all_converged=bool(all(r["converged"] for r in results)),
                fell_back=int(sum(r["fell_back"] for r in results)),
                gmres_iterations=int(sum(r["gmres_iterations"] for r in results)),
                **({"policy": label} if label else {}))


def dumps(obj):
    return json.dumps(obj, default=lambda o: o.tolist() if hasattr(o, "tolist") else str(o))
