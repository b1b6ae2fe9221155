"""Batched uneven-size solves in one persistent, graph-replayed launch
(batched.cu) against the FP64 oracle, LU and Cholesky, FP32+IR and FP64."""
import numpy as np
import pytest

from elemental_gb300 import matrices as mats
from elemental_gb300.batched import BatchedSolver
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def make(count, lo, hi, q, seed, spd_every=2, kappa=None):
    rng = np.random.default_rng(seed)
    systems, kinds = [], []
    for i in range(count):
        n = int(rng.integers(lo, hi + 1))
        if i % spd_every == 1:
            A = mats.spd(n, seed * 1000 + i)
            kinds.append("chol")
        elif kappa is not None:
            A = mats.conditioned(n, kappa, seed * 1000 + i)
            kinds.append("lu")
        else:
            A = mats.gaussian(n, n, seed * 1000 + i)
            kinds.append("lu")
        systems.append((A, mats.gaussian(n, q, seed * 7 + i)))
    return systems, kinds


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_batched_mixed_lu_cholesky(ctx, prec):
    q = 4
    systems, kinds = make(40, 1, 300, q, 11)
    ns, A, B = BatchedSolver.pack(systems, q)
    bs = BatchedSolver(ns, q, A, B, kinds=kinds, precisions=[prec] * len(ns),
                       nb_table=[8, 16, 32, 32, 32, 32, 16, 16], ctx=ctx)
    for _ in range(2):  # the captured graph replays
        bs.run()
    res = bs.results()
    for i, ((Ai, Bi), r) in enumerate(zip(systems, res)):
        X = bs.solution(i)
        be = O.backward_error(Ai, X, Bi)
        assert r["converged"], (i, r)
        assert be <= 1e-13, (i, be, r)
        assert abs(be - r["backward_error"]) <= 0.05 * be + 1e-18
        if kinds[i] == "lu" and prec == "fp64":
            LU, piv = O.lu(Ai, nb=128)
            Xr = O.lu_solve_after(LU, piv, Bi)
            assert np.abs(X - Xr).max() <= 1e-9 * max(1, np.abs(Xr).max())


def test_batched_ill_conditioned_falls_back(ctx):
    q = 2
    systems, kinds = make(6, 64, 128, q, 5, spd_every=1000, kappa=1e12)
    ns, A, B = BatchedSolver.pack(systems, q)
    bs = BatchedSolver(ns, q, A, B, kinds=kinds, max_iters=5, ctx=ctx)
    bs.run()
    res = bs.results()
    for i, ((Ai, Bi), r) in enumerate(zip(systems, res)):
        assert O.backward_error(Ai, bs.solution(i), Bi) <= 1e-13
    assert any(r["fell_back"] or r["iterations"] > 1 for r in res)


def test_batched_singular_reports_info(ctx):
    q = 1
    A = mats.gaussian(50, 50, 1)
    A[:, 10] = 0.0
    systems = [(A, mats.gaussian(50, 1, 2)), (mats.gaussian(20, 20, 3), mats.gaussian(20, 1, 4))]
    ns, Ap, Bp = BatchedSolver.pack(systems, q)
    bs = BatchedSolver(ns, q, Ap, Bp, ctx=ctx)
    bs.run()
    res = bs.results()
    assert res[0]["info"] > 0 and not res[0]["converged"]
    assert res[1]["converged"]


def test_batched_fgmres_ir_reaches_target_where_lu_ir_stalls(ctx):
    """kappa = 1e8 with FP32 factors: kappa * u_fp32 > 1, so LU-IR stalls on
    some systems; flexible GMRES-IR (FP64 Arnoldi, the FP32 factors as
    preconditioner) reaches 1e-13 on more of them, fallback switched off."""
    q = 1
    systems, kinds = make(12, 64, 200, q, 21, spd_every=1000, kappa=1e8)
    ns, A, B = BatchedSolver.pack(systems, q)
    lu_only = BatchedSolver(ns, q, A, B, kinds=kinds, fallback=False, method="lu-ir", ctx=ctx)
    lu_only.run()
    n_lu = sum(r["converged"] for r in lu_only.results())
    lu_only.close()
    assert n_lu < len(ns)
    bs = BatchedSolver(ns, q, A, B, kinds=kinds, fallback=False, method="auto", ctx=ctx)
    bs.run()
    res = bs.results()
    assert sum(r["converged"] for r in res) > n_lu
    for i, ((Ai, Bi), r) in enumerate(zip(systems, res)):
        assert not r["fell_back"]
        be = O.backward_error(Ai, bs.solution(i), Bi)
        assert abs(be - r["backward_error"]) <= 0.05 * be + 1e-18, (i, be, r)
        if r["converged"]:
            assert be <= 1e-13, (i, r)
    assert sum(r["gmres_iterations"] for r in res) > 0


def test_batched_fgmres_only_method(ctx):
    q = 2
    systems, kinds = make(6, 30, 150, q, 23, spd_every=3, kappa=1e6)
    ns, A, B = BatchedSolver.pack(systems, q)
    bs = BatchedSolver(ns, q, A, B, kinds=kinds, fallback=False, method="gmres-ir", ctx=ctx)
    bs.run()
    for i, ((Ai, Bi), r) in enumerate(zip(systems, bs.results())):
        assert r["converged"], (i, r)
        assert r["iterations"] == 0 and (r["gmres_iterations"] > 0 or r["backward_error"] <= 1e-13)
        assert O.backward_error(Ai, bs.solution(i), Bi) <= 1e-13


def test_batched_runtime_precision_and_cascade(ctx):
    """Per-system precision read from device memory at run time (the
    selector's output); with two LU-IR steps allowed, BF16 choices on
    kappa = 1e13 systems cascade to FP32 and FP64 and still meet the
    target; `precision` reports the factors the result came from."""
    import torch
    q = 1
    systems, kinds = make(9, 40, 160, q, 25, spd_every=1000, kappa=1e13)
    ns, A, B = BatchedSolver.pack(systems, q)
    asked = [0, 1, 2] * 3
    codes = torch.tensor(asked, dtype=torch.int32, device="cuda")
    bs = BatchedSolver(ns, q, A, B, kinds=kinds, precision_device=codes, method="lu-ir",
                       max_iters=2, ctx=ctx)
    bs.run()
    res = bs.results()
    for i, ((Ai, Bi), r) in enumerate(zip(systems, res)):
        assert r["converged"], (i, r)
        assert O.backward_error(Ai, bs.solution(i), Bi) <= 1e-13
        assert r["precision"] <= asked[i]
        assert r["fell_back"] == (r["precision"] != asked[i])
    assert any(r["fell_back"] for i, r in enumerate(res) if asked[i] == 2)
    # a second replay reads the array again
    codes.fill_(0)
    bs.run()
    assert all(r["precision"] == 0 and not r["fell_back"] for r in bs.results())


def test_batched_features(ctx):
    """The selector's features: finite, log2 n exact, and the Hager/Higham
    estimate of kappa_1 within a small factor of numpy's exact kappa_1 for
    matrices an FP32 LU resolves."""
    q = 1
    rng = np.random.default_rng(3)
    systems, kinds, kap = [], [], []
    for i in range(8):
        n = int(rng.integers(32, 300))
        k = [1e2, 1e4, 1e5, 1e3][i % 4]
        systems.append((mats.conditioned(n, k, 500 + i), mats.gaussian(n, q, 600 + i)))
        kinds.append("lu")
        kap.append(np.linalg.cond(systems[-1][0], 1))
    ns, A, B = BatchedSolver.pack(systems, q)
    bs = BatchedSolver(ns, q, A, B, kinds=kinds, features_only=True, ctx=ctx)
    bs.run()
    res = bs.results()
    F = bs.features.cpu().numpy()
    assert np.isfinite(F).all()
    assert np.allclose(F[:, 0], np.log2(ns), atol=1e-5)
    for i, r in enumerate(res):
        ratio = r["backward_error"] / kap[i]
        assert 0.1 <= ratio <= 1.01, (i, ratio)
        assert abs(F[i, 1] - np.log10(r["backward_error"])) < 1e-3


def test_batched_norm_features_match_numpy(ctx):
    """The one-pass scan of A behind the norm features (||A||_1, ||A||_inf,
    max |a|, sum |a_ii| over ||A||_F, and ||A||_F itself) against numpy on
    uneven sizes from 1 to 2400 (ragged final row chunks of a column)."""
    q = 1
    rng = np.random.default_rng(11)
    sizes = [1, 17, 100, 257, 640, 2400]
    systems = [(rng.standard_normal((n, n)) * rng.uniform(0.1, 10.0),
                mats.gaussian(n, q, 700 + i)) for i, n in enumerate(sizes)]
    ns, A, B = BatchedSolver.pack(systems, q)
    bs = BatchedSolver(ns, q, A, B, features_only=True, ctx=ctx)
    bs.run()
    F = bs.features.cpu().numpy().astype(np.float64)
    for i, (Ai, _) in enumerate(systems):
        fro = np.linalg.norm(Ai)
        amax = np.abs(Ai).max()
        exp = {2: np.log10(np.abs(Ai).sum(0).max() / fro),
               3: np.log10(np.abs(Ai).sum(1).max() / fro),
               4: np.log10(amax / fro),
               7: np.log10(max(np.abs(np.diag(Ai)).sum() / (len(Ai) * amax), 1e-30)),
               9: np.log10(fro)}
        for k, v in exp.items():
            assert abs(F[i, k] - v) < 2e-6 * max(1.0, abs(v)), (sizes[i], k, F[i, k], v)


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_batched_two_level_blocking(ctx, prec):
    """n ~ 1300 with a 32-column block but a shared-memory panel of at most 24
    columns: sub-panels update only their block, the block updates the
    trailing matrix with K = 32 (tensor cores).  The factorization must be
    as good as a one-level one: LU-IR converges in a few steps, no fallback."""
    q = 1
    systems, kinds = make(3, 1250, 1350, q, 31, spd_every=1000)
    ns, A, B = BatchedSolver.pack(systems, q)
    # BF16 factors need FGMRES-IR at this size (kappa * u_bf16 > 1)
    bs = BatchedSolver(ns, q, A, B, kinds=kinds, precisions=[prec] * len(ns),
                       nb_table=[32] * 8, fallback=False,
                       method="lu-ir" if prec == "fp32" else "auto", ctx=ctx)
    bs.run()
    for i, ((Ai, Bi), r) in enumerate(zip(systems, bs.results())):
        assert r["converged"] and not r["fell_back"], (i, r)
        if prec == "fp32":
            assert r["iterations"] <= 4, (i, r)
        assert O.backward_error(Ai, bs.solution(i), Bi) <= 1e-13
