"""Host logic of the learned precision selector (no GPU): the seeded
conditioned workload, the kappa-threshold rule and its network form, and
the threshold fit."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from elemental_gb300 import selector as S  # noqa: E402
from oracle import mlp_oracle as MO  # noqa: E402


def test_conditioned_systems_have_the_requested_condition_number():
    d = S.conditioned_systems(8, 5, nmin=16, nmax=48, kmin=1e2, kmax=1e10, nrhs=2,
                              device="cpu")
    assert len(d["ns"]) == 8 and d["B"].numel() == 2 * int(d["ns"].sum())
    off = 0
    for n, k in zip(d["ns"], d["kappa"]):
        A = d["A"][off:off + n * n].numpy().reshape(n, n, order="F")
        off += n * n
        assert abs(np.linalg.cond(A) / k - 1) < 1e-4
        # Haar factors: the largest singular value is 1
        assert abs(np.linalg.norm(A, 2) - 1) < 1e-5
    assert off == d["A"].numel()


def test_conditioned_systems_are_seeded():
    a = S.conditioned_systems(3, 11, nmin=8, nmax=24, device="cpu")
    b = S.conditioned_systems(3, 11, nmin=8, nmax=24, device="cpu")
    c = S.conditioned_systems(3, 12, nmin=8, nmax=24, device="cpu")
    assert np.array_equal(a["ns"], b["ns"]) and torch.equal(a["A"], b["A"])
    assert not (np.array_equal(a["ns"], c["ns"]) and torch.equal(a["A"], c["A"]))


@pytest.mark.parametrize("t", [(256.0, 1.6777216e7), (1e3, 1e9), (10.0, 10.0)])
def test_rule_network_computes_the_kappa_rule(t):
    th = S.rule_network(*t, device="cpu").numpy().astype(np.float64)
    assert th.size == MO.NPARAM
    X = np.zeros((400, 16))
    X[:, 1] = np.linspace(-1, 14, 400)
    X[:, 0] = 9.0  # other features must not matter
    X[:, 5] = -3.0
    got = MO.forward(th, X)["probs"].argmax(1)
    want = S.kappa_rule(X[:, 1], *t)
    # exact except within 1/slope decades of a threshold
    near = np.minimum(np.abs(X[:, 1] - np.log10(t[0])), np.abs(X[:, 1] - np.log10(t[1]))) < 1e-3
    assert np.array_equal(got[~near], want[~near])


def test_fit_kappa_rule_recovers_thresholds():
    rng = np.random.default_rng(0)
    lk = rng.uniform(0, 12, 3000)
    y = S.kappa_rule(lk, 10 ** 2.5, 10 ** 8.0)
    th, acc = S.fit_kappa_rule(lk, y)
    assert acc >= 0.995
    assert abs(np.log10(th[0]) - 2.5) <= 0.25 and abs(np.log10(th[1]) - 8.0) <= 0.25
