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
