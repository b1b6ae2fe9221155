"""bench.py's JSON-line contract on the CPU: the reference arm (the oracle's
El::LU + lu::SolveAfter restatement on the host cores) on a tiny sample
prints one JSON line with the keys the contract names."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--cpu-n", "256"], cwd=ROOT, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference"
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 0
    assert "workload" in d["config"]
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0


def test_workload_sizes_resolve():
    sys.path.insert(0, ROOT)
    import bench

    old = sys.argv
    try:
        sys.argv = ["bench.py", "--workload", "inverse"]
        a = bench.parse()
        assert a.n is None and a.workload == "inverse"
    finally:
        sys.argv = old


def test_cholesky_workload_and_kappa_option_parse():
    sys.path.insert(0, ROOT)
    import bench

    old = sys.argv
    try:
        sys.argv = ["bench.py", "--workload", "cholesky"]
        a = bench.parse()
        assert a.workload == "cholesky" and a.kappa == 0.0
        sys.argv = ["bench.py", "--kappa", "1e8"]
        assert bench.parse().kappa == 1e8
    finally:
        sys.argv = old


def test_haar_conditioned_has_the_requested_condition_number():
    """The Haar-conditioned headline input: ||A||_2 = 1, cond_2(A) = kappa."""
    import numpy as np
    import torch

    sys.path.insert(0, ROOT)
    import bench

    for n, kappa in ((40, 1e2), (120, 1e8)):
        g = torch.Generator(device="cpu")
        g.manual_seed(n)
        s = np.linalg.svd(bench.haar_conditioned(n, kappa, g, device="cpu").numpy(),
                          compute_uv=False)
        assert abs(s[0] - 1.0) <= 1e-5
        assert abs(s[0] / s[-1] / kappa - 1.0) <= 1e-4
