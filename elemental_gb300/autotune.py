"""Autotuner of the batched solver's panel widths.

The batched launch (batched.cu) factors each system in one CTA with a panel
of nb columns staged in shared memory; the best nb depends on the system
size (wider panels halve the trailing matrix's traffic per column but
lengthen the panel's column chain and are capped by shared memory).  This
module times candidate widths per size bucket on the GPU it runs on and
keeps the winners in a JSON table next to it:

    python -m elemental_gb300.autotune            # tune FP32 and FP64, write the table
    python -m elemental_gb300.autotune --show     # print the table in use

Size buckets: n <= 32, 64, 128, 256, 512, 1024, 2048, larger (the
nb_table layout of ElGBBatchOptions).  A missing table means the defaults
below.
"""
from __future__ import annotations

import argparse
import json
import os
import time

BUCKETS = (32, 64, 128, 256, 512, 1024, 2048, 4096)
# representative size of each bucket (its upper three quarters)
SIZES = (24, 48, 96, 192, 384, 768, 1536, 3072)
CANDIDATES = (8, 16, 32, 64)
DEFAULT = {"fp32": [8, 16, 32, 32, 32, 32, 16, 16], "fp64": [8, 16, 16, 16, 16, 16, 8, 8]}
TABLE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning", "batched_nb.json")


def _load():
    try:
        with open(TABLE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


def nb_table(precision="fp32"):
    """The tuned panel widths for a factor precision ("fp32" serves BF16
    too), else the defaults."""
    t = _load()
    if t and precision in t.get("nb_table", {}):
        return list(t["nb_table"][precision])
    return list(DEFAULT[precision])


def time_bucket(ctx, n, precision, nb, count, steps=2):
    """Mean device ms per system of `count` N(0, 1) systems of order n at
    panel width nb (one batched launch, warm replay first)."""
    import torch

    from .batched import BatchedSolver

    g = torch.Generator(device="cuda").manual_seed(1000 + n)
    A = torch.randn(count * n * n, generator=g, device="cuda", dtype=torch.float64)
    B = torch.randn(count * n, generator=g, device="cuda", dtype=torch.float64)
    bs = BatchedSolver([n] * count, 1, A, B, precisions=[precision] * count,
                       nb_table=[nb] * len(BUCKETS), method="lu-ir", fallback=False, ctx=ctx)
    try:
        bs.run()
        torch.cuda.synchronize()
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record()
        for _ in range(steps):
            bs.run()
        e.record()
        e.synchronize()
        return s.elapsed_time(e) / steps / count
    finally:
        bs.close()


def tune(precisions=("fp32", "fp64"), ctx=None, log=print):
    """Time every candidate width per bucket; returns the table dict."""
    import torch

    from .device import context

    ctx = ctx or context()
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    sms = props.multi_processor_count
    out = {"device": props.name, "sms": sms, "date": time.strftime("%Y-%m-%d"),
           "nb_table": {}, "ms_per_system": {}}
    for prec in precisions:
        best, timings = [], {}
        for n in SIZES:
            count = sms if n >= 1024 else 2 * sms
            t = {nb: time_bucket(ctx, n, prec, nb, count) for nb in CANDIDATES}
            timings[str(n)] = {str(k): round(v, 4) for k, v in t.items()}
            best.append(min(t, key=t.get))
            log(f"{prec} n={n}: " + ", ".join(f"nb {k}: {v:.3f} ms" for k, v in t.items()))
        out["nb_table"][prec] = best
        out["ms_per_system"][prec] = timings
    return out


def main(argv=None):
    p = argparse.ArgumentParser(description="tune the batched solver's panel widths")
    p.add_argument("--show", action="store_true")
    p.add_argument("--out", default=TABLE)
    a = p.parse_args(argv)
    if a.show:
        print(json.dumps({"table": TABLE, "fp32": nb_table("fp32"), "fp64": nb_table("fp64")}))
        return
    res = tune()
    os.makedirs(os.path.dirname(a.out), exist_ok=True)
    with open(a.out, "w") as f:
        json.dump(res, f, indent=1)
    print(json.dumps(res["nb_table"]))


if __name__ == "__main__":
    main()
