"""Single-kernel cases of the factor-and-solve path, for timing and for
profiler captures (one warm-up call, then one measured call, so a profiler
can skip the first launch of the kernel it targets).

    python kernel_cases.py tc_gemm --m 16384 --n 16384 --k 512 --kind 2
    python kernel_cases.py lu --n 8192 --kind 2
    python kernel_cases.py refine --n 8192 --nrhs 16
    python kernel_cases.py lu64 --n 4096
    python kernel_cases.py batched --n 1024 --count 152 --precision fp32
    python kernel_cases.py lufull --n 2048
    python kernel_cases.py residual --n 32768 --nrhs 16
    python kernel_cases.py lu_breakdown --n 32768 --nb 512
    python kernel_cases.py panel_trace --n 32768 --nb 512
    python kernel_cases.py leaf_costs --m 8192 --n 512 --nb 512

Each prints one JSON line with the event-timed duration of the measured
call and its algorithmic work.  Inputs are seeded N(0, 1), generated on the
device.
"""
import argparse
import json

import torch

from elemental_gb300 import device as D

KIND_NAMES = {-1: "simt-fp32", 0: "bf16", 1: "tf32", 2: "tf32x3"}


def _timed(fn):
    torch.cuda.synchronize()
    s = torch.cuda.Event(enable_timing=True)
    e = torch.cuda.Event(enable_timing=True)
    s.record()
    fn()
    e.record()
    e.synchronize()
    return s.elapsed_time(e)


def case_tc_gemm(ctx, a):
    """C (m x n) -= A (m x k) B (k x n) on the tensor cores: the trailing
    update of El::LU (src/lapack_like/factor/LU.cpp:131-133)."""
    g = torch.Generator(device="cuda").manual_seed(a.seed)
    A = D.colmajor(a.m, a.k, torch.float32)
    B = D.colmajor(a.k, a.n, torch.float32)
    C = D.colmajor(a.m, a.n, torch.float32)
    A.copy_(torch.randn(a.m, a.k, device="cuda", generator=g))
    B.copy_(torch.randn(a.k, a.n, device="cuda", generator=g))
    C.zero_()
    ctx.gemm_sub_tc(A, B, C, a.kind)
    ms = _timed(lambda: ctx.gemm_sub_tc(A, B, C, a.kind))
    flops = 2.0 * a.m * a.n * a.k
    return dict(case="tc_gemm", m=a.m, n=a.n, k=a.k, kind=KIND_NAMES[a.kind], ms=ms,
                tflops=flops / (ms * 1e-3) / 1e12,
                algorithmic_bytes=4.0 * (a.m * a.k + a.k * a.n + 2 * a.m * a.n))


def case_lu(ctx, a):
    """El::LU on an FP32 matrix with tensor-core updates (the low-precision
    factorization of the refinement)."""
    g = torch.Generator(device="cuda").manual_seed(a.seed)
    A0 = torch.randn(a.n, a.n, device="cuda", generator=g).t()
    A = A0.clone()
    ctx.lu_mixed(A, gemm_kind=a.kind, nb=a.nb)
    A.copy_(A0)
    ms = _timed(lambda: ctx.lu_mixed(A, gemm_kind=a.kind, nb=a.nb))
    flops = 2.0 / 3.0 * a.n ** 3
    return dict(case="lu", n=a.n, kind=KIND_NAMES[a.kind], ms=ms,
                tflops=flops / (ms * 1e-3) / 1e12)


def case_lu64(ctx, a):
    """El::LU in FP64 (the plain path)."""
    g = torch.Generator(device="cuda").manual_seed(a.seed)
    A0 = torch.randn(a.n, a.n, device="cuda", generator=g, dtype=torch.float64).t()
    A = A0.clone()
    ctx.lu(A, nb=a.nb)
    A.copy_(A0)
    ms = _timed(lambda: ctx.lu(A, nb=a.nb))
    flops = 2.0 / 3.0 * a.n ** 3
    return dict(case="lu64", n=a.n, ms=ms, tflops=flops / (ms * 1e-3) / 1e12)


def case_refine(ctx, a):
    """Mixed-precision LU-IR (FP32 factors, FP64 residual)."""
    g = torch.Generator(device="cuda").manual_seed(a.seed)
    A = D.colmajor(a.n, a.n)
    B = D.colmajor(a.n, a.nrhs)
    A.copy_(torch.randn(a.n, a.n, device="cuda", generator=g, dtype=torch.float64))
    B.copy_(torch.randn(a.n, a.nrhs, device="cuda", generator=g, dtype=torch.float64))
    ctx.refined_solve(A, B, precision="fp32", method=a.method)
    info = {}

    def run():
        info.update(ctx.refined_solve(A, B, precision="fp32", method=a.method)[1])

    ms = _timed(run)
    out = dict(case="refine", n=a.n, nrhs=a.nrhs, method=a.method, ms=ms, **info)
    if a.records:
        import numpy as np

        ctx.profile_start()
        out["ms_profiled"] = _timed(run)
        ctx.profile_stop()
        rec = ctx.profile_records()
        np.save(a.records, rec)
        out["tagged_ms"] = {str(t): round(float(rec["dur_ms"][rec["tag"] == t].sum()), 2)
                            for t in sorted(set(rec["tag"].tolist()))}
    return out


def case_batched(ctx, a):
    """`count` N(0, 1) LU systems of order n, one persistent batched launch
    (warm-up replay, then the measured replay)."""
    from elemental_gb300.batched import BatchedSolver
    g = torch.Generator(device="cuda").manual_seed(a.seed)
    A = torch.randn(a.count * a.n * a.n, device="cuda", generator=g, dtype=torch.float64)
    B = torch.randn(a.count * a.n * a.nrhs, device="cuda", generator=g, dtype=torch.float64)
    bs = BatchedSolver([a.n] * a.count, a.nrhs, A, B, precisions=[a.precision] * a.count,
                       fallback=False, method="lu-ir", ctx=ctx, phases=True,
                       simt_update=a.simt,
                       nb_table=[a.nb] * 8 if a.nb else None)
    bs.run()
    ms = _timed(bs.run)
    res = bs.results()
    dev = [r["device_ms"] for r in res]
    flops = a.count * 2.0 / 3.0 * a.n ** 3
    out = dict(case="batched", n=a.n, count=a.count, nrhs=a.nrhs, precision=a.precision,
               update="simt" if a.simt else "tcgen05", ms=ms,
               tflops=flops / (ms * 1e-3) / 1e12, converged=sum(r["converged"] for r in res),
               device_ms_mean=sum(dev) / len(dev), device_ms_max=max(dev),
               gflops_per_system_cta=2.0 / 3.0 * a.n ** 3 / (sum(dev) / len(dev) * 1e-3) / 1e9,
               iterations_mean=sum(r["iterations"] for r in res) / len(res),
               phase_ms_mean={k: round(float(v.mean()), 3) for k, v in bs.phase_ms().items()})
    bs.close()
    return out


def case_lufull(ctx, a):
    """El::LU(A, P, Q) with full pivoting (src/lapack_like/factor/LU/Full.hpp):
    two kernels per step (swap / update + next pivot search)."""
    g = torch.Generator(device="cuda").manual_seed(a.seed)
    A0 = D.colmajor(a.n, a.n)
    A0.copy_(torch.randn(a.n, a.n, device="cuda", generator=g, dtype=torch.float64).t())
    A = D.colmajor(a.n, a.n)
    A.copy_(A0)
    ctx.lu_full(A)
    A.copy_(A0)
    ms = _timed(lambda: ctx.lu_full(A))
    return dict(case="lufull", n=a.n, ms=ms, gflops=2.0 / 3.0 * a.n ** 3 / (ms * 1e-3) / 1e9,
                trailing_traffic_gbs=16.0 * a.n ** 3 / 3.0 / (ms * 1e-3) / 1e9,
                status=ctx.status())


def case_residual(ctx, a):
    """The refinement's residual R = B - A X (n x nrhs): double-float on the
    FP32 pipe (ElGBResidualDF_d, including its split of A) and FP64
    (ElGBResidual_d), each timed once after a warm-up call."""
    g = torch.Generator(device="cuda").manual_seed(a.seed)
    A = D.colmajor(a.n, a.n)
    X = D.colmajor(a.n, a.nrhs)
    B = D.colmajor(a.n, a.nrhs)
    A.copy_(torch.randn(a.n, a.n, device="cuda", generator=g, dtype=torch.float64))
    X.copy_(torch.randn(a.n, a.nrhs, device="cuda", generator=g, dtype=torch.float64))
    B.copy_(torch.randn(a.n, a.nrhs, device="cuda", generator=g, dtype=torch.float64))
    ctx.residual_df(A, X, B)
    ms_df = _timed(lambda: ctx.residual_df(A, X, B))
    ctx.residual(A, X, B)
    ms_64 = _timed(lambda: ctx.residual(A, X, B))
    fl = 2.0 * a.n * a.n * a.nrhs
    return dict(case="residual", n=a.n, nrhs=a.nrhs, ms_df_with_split=ms_df, ms_fp64=ms_64,
                tflops_eq_df=fl / (ms_df * 1e-3) / 1e12, tflops_fp64=fl / (ms_64 * 1e-3) / 1e12)


def _stream_overlap(rec, segments=8):
    """From the profiler's launch groups: how long the main stream, the
    look-ahead panel stream, both or neither had a launch group running, in
    total and per eighth of the run."""
    import numpy as np

    if len(rec) == 0:
        return {}
    t = np.concatenate([rec["start_ms"], rec["start_ms"] + rec["dur_ms"]])
    edges = np.unique(np.concatenate([t, np.linspace(t.min(), t.max(), segments + 1)]))
    mid = 0.5 * (edges[1:] + edges[:-1])
    width = np.diff(edges)

    def busy(sel):
        s = rec["start_ms"][sel]
        e = s + rec["dur_ms"][sel]
        order = np.argsort(s)
        s, e = s[order], np.maximum.accumulate(e[order])
        i = np.searchsorted(s, mid, side="right") - 1
        return (i >= 0) & (e[np.maximum(i, 0)] > mid)

    m, sd = busy(rec["side"] != 1), busy(rec["side"] == 1)
    seg = np.minimum(((mid - t.min()) / (t.max() - t.min()) * segments).astype(int),
                     segments - 1)
    out = {}
    for name, mask in (("both", m & sd), ("main_only", m & ~sd), ("side_only", ~m & sd),
                       ("neither", ~m & ~sd)):
        out[name + "_ms"] = round(float(width[mask].sum()), 2)
        out[name + "_ms_by_eighth"] = [round(float(width[mask & (seg == k)].sum()), 2)
                                       for k in range(segments)]
    out["span_ms"] = round(float(t.max() - t.min()), 2)
    return out


def case_lu_breakdown(ctx, a):
    """El::LU on an FP32 matrix (tensor-core updates) with the per-kernel
    event timing of the library's profiler: panel, swaps, TRSM, GEMMs."""
    g = torch.Generator(device="cuda").manual_seed(a.seed)
    A0 = torch.randn(a.n, a.n, device="cuda", generator=g).t()
    A = A0.clone()
    ctx.set_option("lookahead", a.lookahead)
    ctx.set_option("trail_grid", a.trail_grid)
    ctx.lu_mixed(A, gemm_kind=a.kind, nb=a.nb)
    A.copy_(A0)
    ctx.profile_start()
    ms = _timed(lambda: ctx.lu_mixed(A, gemm_kind=a.kind, nb=a.nb))
    prof = ctx.profile_stop()
    rec = ctx.profile_records()
    if a.records:
        import numpy as np

        np.save(a.records, rec)
    ctx.set_option("lookahead", 1)
    ctx.set_option("trail_grid", 2)
    return dict(case="lu_breakdown", n=a.n, kind=KIND_NAMES[a.kind], lookahead=a.lookahead,
                trail_grid=a.trail_grid, ms=ms, timeline=_stream_overlap(rec),
                tflops=2.0 / 3.0 * a.n ** 3 / (ms * 1e-3) / 1e12,
                kernel_ms={k: round(v["ms"], 3) for k, v in prof["by_kernel"].items()},
                kernel_ms_lookahead_stream={k: round(v["ms"], 3)
                                            for k, v in prof["by_kernel_lookahead_stream"].items()},
                kernel_launches={k: v["launches"] for k, v in prof["by_kernel"].items()})


def case_panel_trace(ctx, a):
    """El::LU on an FP32 matrix (tensor-core updates) with the leaf-panel
    trace on: per pivot step, the time from publishing the candidate to the
    end of the previous step's deferred update (publish + deferred update),
    from there to the complete exchange (exchange wait), and the step's
    front half (swap, multipliers, next column, argmax); medians over the
    columns of the leaves of each height band."""
    import numpy as np

    g = torch.Generator(device="cuda").manual_seed(a.seed)
    A0 = torch.randn(a.n, a.n, device="cuda", generator=g).t()
    A = A0.clone()
    ctx.set_option("panel_trace", a.n)
    ctx.set_option("lookahead", a.lookahead)
    ctx.set_option("trail_grid", a.trail_grid)
    ctx.set_option("panel_cluster", a.panel_cluster)
    ctx.set_option("panel_rows", a.panel_rows)
    ctx.set_option("panel_regs", a.panel_regs)
    ctx.set_option("trail_split", a.trail_split)
    ctx.set_option("panel_push", a.panel_push)
    try:
        ctx.lu_mixed(A, gemm_kind=a.kind, nb=a.nb)
        A.copy_(A0)
        ms = _timed(lambda: ctx.lu_mixed(A, gemm_kind=a.kind, nb=a.nb))
        tr = ctx.panel_trace(a.n)
    finally:
        ctx.set_option("panel_trace", 0)
        ctx.set_option("lookahead", 1)
        ctx.set_option("trail_grid", 2)
        ctx.set_option("panel_cluster", 16)
        ctx.set_option("panel_rows", 512)
        ctx.set_option("panel_regs", 2)
        ctx.set_option("trail_split", 1)
        ctx.set_option("panel_push", 1)
    ok = np.all(tr > 0, axis=1)
    cols = np.arange(a.n)
    d_pub = (tr[:, 1] - tr[:, 0]) / 1e3
    d_x = (tr[:, 2] - tr[:, 1]) / 1e3
    d_front = (tr[:, 3] - tr[:, 2]) / 1e3
    step = np.full(a.n, np.nan)
    same_leaf = (cols[1:] // 32) == (cols[:-1] // 32)
    step[:-1][same_leaf] = (tr[1:, 0] - tr[:-1, 0])[same_leaf] / 1e3
    bands = {}
    for lo, hi in [(0, 8192), (8192, 16384), (16384, 24576), (24576, a.n)]:
        sel = ok & (a.n - cols > lo) & (a.n - cols <= hi)
        if not sel.any():
            continue
        bands[f"rows {lo + 1}-{hi}"] = {
            "columns": int(sel.sum()),
            "us_publish_and_deferred_update": round(float(np.median(d_pub[sel])), 3),
            "us_exchange_wait": round(float(np.median(d_x[sel])), 3),
            "us_front_half": round(float(np.median(d_front[sel])), 3),
            "us_per_step": round(float(np.nanmedian(step[sel])), 3)}
    tot_steps = float(np.nansum(step[ok])) / 1e3
    return dict(case="panel_trace", n=a.n, kind=KIND_NAMES[a.kind], lookahead=a.lookahead,
                trail_grid=a.trail_grid, panel_cluster=a.panel_cluster,
                panel_rows=a.panel_rows, panel_regs=a.panel_regs, trail_split=a.trail_split,
                panel_push=a.panel_push,
                ms=ms, traced=int(ok.sum()),
                leaf_step_ms_total=tot_steps, bands=bands)


def case_leaf_costs(ctx, a):
    """Fixed cost of the leaf-panel launches: per leaf, the event-timed launch
    group minus the traced span from its first pivot step's start to its
    last step's end (load, exchange set-up, write-back, the interchanges on
    the block's other columns, launch), for an m x n FP32 LU with block
    size nb and one stream (so that the leaves run in column order)."""
    import numpy as np

    m, n, nb = a.m, a.n, a.nb
    g = torch.Generator(device="cuda").manual_seed(a.seed)
    A0 = torch.randn(n, m, device="cuda", generator=g).t()
    A = A0.clone()
    ctx.set_option("panel_trace", n)
    ctx.set_option("lookahead", 0)
    try:
        ctx.lu_mixed(A, gemm_kind=a.kind, nb=nb)
        A.copy_(A0)
        torch.cuda.synchronize()
        ctx.profile_start()
        ctx.lu_mixed(A, gemm_kind=a.kind, nb=nb)
        ctx.profile_stop()
        rec = ctx.profile_records()
        tr = ctx.panel_trace(n)
    finally:
        ctx.set_option("panel_trace", 0)
        ctx.set_option("lookahead", 1)
    pan = rec[rec["tag"] == 1]
    pan = pan[np.argsort(pan["start_ms"])]
    lw = 16 if 16384 < m <= 32768 else 32  # the leaf width of the first block
    c0s = list(range(0, n, lw))[:len(pan)]
    dur = pan["dur_ms"] * 1e3
    span = np.array([(tr[c + lw - 1, 3] - tr[c, 0]) / 1e3 for c in c0s])
    return dict(case="leaf_costs", m=m, n=n, nb=nb, leaf_width=lw, leaves=len(pan),
                us_launch_median=round(float(np.median(dur)), 1),
                us_steps_median=round(float(np.median(span)), 1),
                us_fixed_median=round(float(np.median(dur - span)), 1))


CASES = {"leaf_costs": case_leaf_costs, "tc_gemm": case_tc_gemm, "lu": case_lu, "lu64": case_lu64, "refine": case_refine,
         "batched": case_batched, "lufull": case_lufull, "residual": case_residual,
         "lu_breakdown": case_lu_breakdown, "panel_trace": case_panel_trace}


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("case", choices=sorted(CASES))
    p.add_argument("--m", type=int, default=16384)
    p.add_argument("--n", type=int, default=8192)
    p.add_argument("--k", type=int, default=512)
    p.add_argument("--kind", type=int, default=2, choices=sorted(KIND_NAMES))
    p.add_argument("--nb", type=int, default=0)
    p.add_argument("--nrhs", type=int, default=16)
    p.add_argument("--method", default="lu-ir", choices=["lu-ir", "gmres-ir"])
    p.add_argument("--count", type=int, default=152)
    p.add_argument("--simt", action="store_true", help="batched: SIMT trailing updates")
    p.add_argument("--precision", default="fp32", choices=["fp64", "fp32", "bf16"])
    p.add_argument("--seed", type=int, default=20261204)
    p.add_argument("--lookahead", type=int, default=1,
                   help="lu_breakdown, panel_trace: 0 = one stream")
    p.add_argument("--trail-grid", type=int, default=2,
                   help="lu_breakdown, panel_trace: ELGB_OPT_TRAIL_GRID")
    p.add_argument("--panel-cluster", type=int, default=16,
                   help="panel_trace: ELGB_OPT_PANEL_CLUSTER (1 = cooperative leaf panels only)")
    p.add_argument("--panel-rows", type=int, default=512,
                   help="panel_trace: ELGB_OPT_PANEL_ROWS")
    p.add_argument("--trail-split", type=int, default=1,
                   help="panel_trace: ELGB_OPT_TRAIL_SPLIT")
    p.add_argument("--panel-push", type=int, default=1,
                   help="panel_trace: ELGB_OPT_PANEL_PUSH (0 = cluster-barrier exchange)")
    p.add_argument("--panel-regs", type=int, default=2,
                   help="panel_trace: ELGB_OPT_PANEL_REGS (2 = register cluster kernel)")
    p.add_argument("--records", default="",
                   help="lu_breakdown: save the profiler's launch groups (.npy)")
    a = p.parse_args(argv)
    ctx = D.context(0)
    out = CASES[a.case](ctx, a)
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
