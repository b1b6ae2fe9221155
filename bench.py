#!/usr/bin/env python3
"""Benchmark of the GB300 dense factor-and-solve path.

Headline workload (default): mixed-precision solve of A X = B, A n x n and B
n x 16 iid N(0,1) in FP64 (n = 32768, the largest single-GPU size of the
plain-FP64 configuration), by FP32 factors (TF32x3 tcgen05 trailing updates)
and LU-IR with an FP64 residual, to a normwise backward error <= n eps64.
One step = one full solve (factor + refine) of the system.  Beside it the
plain FP64 GPU LU (getrf + getrs) is timed once on the same system, and the
reference's CPU algorithm (the oracle restatement of El::LU +
lu::SolveAfter over OpenBLAS, all host threads) on a bounded sample.

  value  solves/s with A, B resident in HBM (CUDA events, max over ranks)
  e2e    the same solve through the Elemental-style C ABI on pinned host
         buffers (ElLinearSolveMixed_d): H2D of A and B, D2H of X per step

Other workloads (`--workload`): `batched` (4096 uneven LU / Cholesky systems
in one persistent launch), `selector` (10,000 conditioned systems through the
learned precision selector), `inverse` (El::Inverse and El::OneCondition of
one n = 8192 FP64 matrix), `cholesky` (plain FP64 El::HPDSolve = potrf + potrs
of one SPD n = 16384 system G^T G / n + I with 16 RHS).

`--impl reference` times the CPU reference arm alone.  Under torchrun each
rank solves its own system (replicas; the factorization does not shard).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "solves/s & TFLOP/s-eq at FP64 backward err: mixed-prec IR vs plain FP64 LU"
EPS64 = 2.220446049250313e-16


def flops_per_solve(n, q):
    return 2.0 / 3.0 * n ** 3 + 2.0 * n * n * q


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--n", type=int, default=None,
                   help="matrix size (default 32768 for lu-ir, 8192 for inverse, 16384 for "
                        "cholesky)")
    p.add_argument("--nrhs", type=int, default=16)
    p.add_argument("--precision", default="fp32",
                   choices=["fp32", "tf32", "bf16", "fp8", "fp64"])
    p.add_argument("--method", default="lu-ir", choices=["lu-ir", "gmres-ir"])
    p.add_argument("--nb", type=int, default=0)
    p.add_argument("--fp64-compare", default="on", choices=["on", "off"])
    p.add_argument("--e2e", default="on", choices=["on", "off"])
    p.add_argument("--cpu-baseline", default="on", choices=["on", "off"])
    p.add_argument("--cpu-n", type=int, default=8192)
    p.add_argument("--seed", type=int, default=20261204 + 1)
    p.add_argument("--workload", default="lu-ir",
                   choices=["lu-ir", "batched", "selector", "inverse", "cholesky"],
                   help="lu-ir: one large mixed-precision solve (default); batched: 4096 "
                        "uneven LU/Cholesky systems in one launch; selector: 10,000 "
                        "conditioned systems through the learned precision selector; "
                        "inverse: El::Inverse and El::OneCondition of one FP64 matrix; "
                        "cholesky: plain FP64 El::HPDSolve of one SPD system")
    p.add_argument("--kappa", type=float, default=0.0,
                   help="lu-ir: A = U diag(sigma) V^T with U, V Haar and cond_2(A) = kappa "
                        "(0, the default: A iid N(0,1))")
    p.add_argument("--tol", type=float, default=0.0,
                   help="lu-ir: target normwise backward error (0, the default: n*eps64)")
    p.add_argument("--max-iters", type=int, default=0,
                   help="lu-ir: refinement steps (GMRES-IR: inner iterations) before the FP64 "
                        "fallback (0: the library's default)")
    p.add_argument("--restart", type=int, default=0, help="lu-ir, GMRES-IR: restart length")
    p.add_argument("--count", type=int, default=0, help="systems (batched / selector)")
    p.add_argument("--train-count", type=int, default=3000, help="selector training systems")
    return p.parse_args()


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons, power = [], None, set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
                power.append(float(f[3]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm),
                "power_w_max": max(power) if power else None}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d, "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, \
            "fallback"


# ---------------------------------------------------------------------------
# CPU reference arm: the oracle's restatement of El::LU + lu::SolveAfter
# ---------------------------------------------------------------------------
def cpu_sample(n_sample, q, seed, reps=1):
    import numpy as np

    from oracle import oracle as O

    threads = os.cpu_count() or 1
    O.lib(threads)
    rng = np.random.default_rng(seed)
    A = np.asfortranarray(rng.standard_normal((n_sample, n_sample)))
    B = np.asfortranarray(rng.standard_normal((n_sample, q)))
    best = None
    berr = None
    for _ in range(reps):
        t0 = time.perf_counter()
        LU, piv = O.lu(A, nb=128)
        X = O.lu_solve_after(LU, piv, B)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
        berr = O.backward_error(A, X, B)
    return best, threads, berr


def reference_arm(args, rank):
    if rank != 0:
        return 0
    n, q = args.n, args.nrhs
    ns = min(args.cpu_n, n)
    scale = flops_per_solve(n, q) / flops_per_solve(ns, q)
    for _ in range(max(args.warmup, 0)):
        cpu_sample(ns, q, args.seed)
    times = []
    for _ in range(args.steps):
        t, threads, berr = cpu_sample(ns, q, args.seed)
        times.append(t)
    tot = sum(times)
    value = args.steps / (tot * scale)
    sample = (f"El::LU + lu::SolveAfter restatement (oracle/el_oracle.c over OpenBLAS), "
              f"N(0,1) n={ns}, {q} RHS, FP64, nb=128; each step one sample solve, value "
              f"scaled to n={n} by the flop count (x{scale:.1f})")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic: seeded iid N(0,1)",
        "config": {"workload": f"FP64 LU + solve, n={n}, {q} RHS, N(0,1) (CPU sample n={ns})",
                   "n": n, "nrhs": q, "parallelism": "cpu"},
        "tflops_eq": value * flops_per_solve(n, q) / 1e12,
        "backward_error_sample": berr,
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def haar_conditioned(n, kappa, g, device="cuda"):
    """A = U diag(sigma) V^T with sigma_i = kappa^(-i/(n-1)), so ||A||_2 = 1
    and cond_2(A) = kappa: U, V the sign-fixed Q factors of Gaussian QRs (the
    construction of src/matrices/random/misc/Haar.cpp:14-21), run in FP32 and
    widened exactly to FP64 (orthogonal to ~1e-6, so cond_2(A) = kappa to
    ~1e-5 relative); the product is formed in FP64 so that singular values far
    below FP32's unit roundoff survive.  Returns a row-major n x n FP64 tensor
    (input synthesis, not timed)."""
    import torch

    i = torch.arange(n, dtype=torch.float64, device=device)
    sig = torch.pow(torch.full_like(i, float(kappa)), -i / max(n - 1, 1))
    Q = []
    for _ in range(2):
        G = torch.randn(n, n, generator=g, device=device, dtype=torch.float32)
        Qf, R = torch.linalg.qr(G)
        del G
        Qf.mul_(torch.sign(torch.diagonal(R))[None, :])
        del R
        Q.append(Qf.double())
        del Qf
    U, V = Q
    U.mul_(sig[None, :])
    return U @ V.t()


def host_thp_gib():
    """Transparent huge pages backing this process's anonymous memory (GiB),
    or None where the kernel does not report them: the host buffers' page
    size, beside their measured upload rate."""
    try:
        with open("/proc/self/smaps_rollup") as f:
            for line in f:
                if line.startswith("AnonHugePages:"):
                    return int(line.split()[1]) / (1 << 20)
    except OSError:
        pass
    return None


def host_tensor(shape):
    """FP64 host buffer for the end-to-end arms: the library's host memory
    (ElGBHostAlloc: anonymous pages registered with the CUDA driver), viewed
    as a torch tensor.  Host -> device copies from it kept ~200 GB/s after
    GPU compute on GB300, where cudaHostAlloc memory (torch's pin_memory)
    fell to 40-100 GB/s."""
    import numpy as np
    import torch

    import elemental_gb300 as El

    return torch.from_numpy(El.host_empty(shape, np.float64, order="C"))


def host_backward_error(AT, X, B, block=1024):
    """Normwise backward error max_j ||b_j - A x_j||_2 / (||A||_F ||x_j||_2 +
    ||b_j||_2) recomputed on the host in FP64 (numpy over OpenBLAS), from
    AT = A^T as a row-major (n, n) array (the pinned host copy of the
    column-major A), X and B (n, q).  Row blocks keep the temporaries small."""
    import numpy as np

    n = AT.shape[0]
    R = np.array(B, dtype=np.float64, copy=True)
    nA2 = 0.0
    for j0 in range(0, n, block):
        blk = AT[j0:j0 + block]          # rows j0.. of A^T = columns j0.. of A
        R -= blk.T @ X[j0:j0 + block]
        nA2 += float(np.einsum("ij,ij->", blk, blk))
    num = np.linalg.norm(R, axis=0)
    den = np.sqrt(nA2) * np.linalg.norm(X, axis=0) + np.linalg.norm(B, axis=0)
    return float(np.max(num / den))


def gpu_arm(args, rank, world, local_rank):
    import numpy as np
    import torch

    import elemental_gb300 as El
    from elemental_gb300 import device as D

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    n, q = args.n, args.nrhs
    ctx = D.context(local_rank)
    g = torch.Generator(device="cuda")
    g.manual_seed(args.seed + 7919 * rank)
    A = D.colmajor(n, n)
    if args.kappa > 0:
        A.copy_(haar_conditioned(n, args.kappa, g))
    else:
        A.copy_(torch.randn(n, n, generator=g, device="cuda", dtype=torch.float64).t())
    B = D.colmajor(n, q)
    B.copy_(torch.randn(q, n, generator=g, device="cuda", dtype=torch.float64).t())
    X = D.colmajor(n, q)
    # the host copies of the system for the end-to-end arm, made first, as a
    # caller's data exists before any solve; in the library's host memory
    # (host_tensor)
    if args.e2e == "on":
        Ah = host_tensor((n, n))
        Ah.copy_(A.t())  # row-major (n, n) of A^T = column-major A
        B0 = host_tensor((q, n))
        B0.copy_(B.t())
        Bh = host_tensor((q, n))
    torch.cuda.synchronize()

    def solve(tol=args.tol):
        return ctx.refined_solve(A, B, X, precision=args.precision, method=args.method,
                                 nb=args.nb, tol=tol, max_iters=args.max_iters,
                                 restart=args.restart)

    info = None
    for _ in range(max(args.warmup, 0)):
        _, info = solve()
    barrier()
    clocks = ClockSampler(local_rank)
    clocks.start()
    l0 = ctx.launches()
    # inside the timed region only the dominant kernel is bracketed with
    # events (for the roofline); the per-family breakdown comes from one
    # extra, untimed, fully bracketed solve after it
    ctx.profile_start(tags=["tc_gemm"])
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    infos = []
    e0.record(stream)
    for _ in range(args.steps):
        _, info = solve()
        infos.append(info)
    e1.record(stream)
    e1.synchronize()
    barrier()
    prof = ctx.profile_stop()
    launches = ctx.launches() - l0
    clk = clocks.stop()
    ctx.profile_start()
    solve()
    prof_all = ctx.profile_stop()
    t = e0.elapsed_time(e1) / 1e3
    tmax = t
    if dist is not None:
        tt = torch.tensor([t], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        tmax = float(tt.item())
    value = args.steps * world / tmax
    berr = max(i["backward_error"] for i in infos)
    iters = max(i["iterations"] for i in infos)

    # end to end through the Elemental-style C ABI on registered host
    # buffers, right after the device arm (before the ~20 s FP64 comparison)
    e2e = None
    if args.e2e == "on":
        Am = El.Matrix(Ah.numpy().T)
        assert Am.array.ctypes.data == Ah.data_ptr()
        Bh.copy_(B0)
        Bm = El.Matrix(Bh.numpy().T)
        assert Bm.array.ctypes.data == Bh.data_ptr()
        El.LinearSolveMixed(Am, Bm, precision=args.precision, method=args.method, nb=args.nb,
                            tol=args.tol)
        # the host -> device rate of this same pinned buffer through torch
        # (64 MiB chunks), beside the library's own upload phase below
        flat = Ah.view(-1)
        dflat = torch.empty(flat.numel(), dtype=torch.float64, device="cuda")
        ck = (64 << 20) // 8
        torch.cuda.synchronize()
        tt = time.perf_counter()
        for i in range(0, flat.numel(), ck):
            dflat[i:i + ck].copy_(flat[i:i + ck], non_blocking=True)
        torch.cuda.synchronize()
        torch_h2d = 8 * flat.numel() / (time.perf_counter() - tt) / 1e9
        del dflat
        tot = 0.0
        einfo = None
        phases = {"upload_ms": 0.0, "compute_ms": 0.0, "download_ms": 0.0}
        for _ in range(args.steps):
            Bh.copy_(B0)
            barrier()
            t0 = time.perf_counter()
            einfo = El.LinearSolveMixed(Am, Bm, precision=args.precision, method=args.method,
                                        nb=args.nb, tol=args.tol)
            tot += time.perf_counter() - t0
            for k, v in El.LastHostCallTimes().items():
                phases[k] += v / args.steps
        te = tot
        if dist is not None:
            tt = torch.tensor([te], device="cuda")
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            te = float(tt.item())
        Xh = torch.from_numpy(Bm.array.T.copy())
        err = float((Xh.cuda() - X.t()).abs().max())
        # the solution returned through the public API, re-checked on the
        # host in FP64 against the host copies of A and B (not timed)
        th = time.perf_counter()
        host_berr = host_backward_error(Ah.numpy(), Bm.array, B0.numpy().T)
        th = time.perf_counter() - th
        e2e = {"value": args.steps * world / te, "unit": "solves/s",
               "h2d_bytes_per_step": 8 * n * n + 8 * n * q, "d2h_bytes_per_step": 8 * n * q,
               "api": "ElLinearSolveMixed_d (El::Matrix handles on ElGBHostAlloc host memory, pinned by registration)",
               "max_abs_diff_vs_device_run": err,
               "iterations": einfo["iterations"] if einfo else None,
               "backward_error": einfo["backward_error"] if einfo else None,
               "backward_error_host_fp64": host_berr,
               "host_check": f"||B - A X|| / (||A||_F ||X|| + ||B||) per column, numpy FP64 "
                             f"on the host ({th:.1f} s, not timed)",
               "phases_ms_per_step": phases,
               "h2d_gbs_torch_same_buffer": torch_h2d,
               "host_thp_gib": host_thp_gib(),
               "h2d_gbs": (8 * n * n + 8 * n * q) / (phases["upload_ms"] * 1e-3) / 1e9
               if phases["upload_ms"] > 0 else None}
        del Ah, B0, Bh, Am, Bm

    # plain FP64 GPU LU on the same system (one step; warm-up on a small case)
    fp64 = None
    if args.fp64_compare == "on" and rank == 0:
        As = D.colmajor(512, 512)
        As.copy_(torch.randn(512, 512, device="cuda", dtype=torch.float64))
        Bs = D.colmajor(512, q)
        Bs.copy_(torch.randn(512, q, device="cuda", dtype=torch.float64))
        ctx.refined_solve(As, Bs, precision="fp64")
        torch.cuda.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        _, finfo = ctx.refined_solve(A, B, X, precision="fp64")
        f1.record(stream)
        f1.synchronize()
        tf = f0.elapsed_time(f1) / 1e3
        fp64 = {"ms": tf * 1e3, "solves_per_s": 1.0 / tf,
                "tflops_eq": flops_per_solve(n, q) / tf / 1e12,
                "backward_error": finfo["backward_error"],
                "fp64_fma_peak_tflops_probe": ctx.fp64_peak_tflops(),
                "speedup_mixed_vs_fp64": tf / (tmax / args.steps)}
        # the mixed solve run on to the FP64 LU's own backward error on this
        # system (one solve, events on the same stream)
        lvl = finfo["backward_error"]
        f0.record(stream)
        _, linfo = ctx.refined_solve(A, B, X, precision=args.precision, method=args.method,
                                     nb=args.nb, tol=lvl, fallback=False)
        f1.record(stream)
        f1.synchronize()
        tl = f0.elapsed_time(f1) / 1e3
        fp64["mixed_to_fp64_level"] = {
            "tol": lvl, "ms": tl * 1e3, "iterations": linfo["iterations"],
            "backward_error": linfo["backward_error"], "fell_back": linfo["fell_back"],
            "speedup_vs_fp64": tf / tl}

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0

    peaks, peak_kind = measured_peaks()
    tf_achieved = prof["flops"] / (prof["ms"] * 1e-3) / 1e12 if prof["ms"] > 0 else None
    peak = peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops"))
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "tc_gemm_traffic.json")
    if os.path.exists(tpath) and prof["launches"] and args.precision == "fp32":
        with open(tpath) as f:
            tj = json.load(f)
        # DRAM bytes over algorithmic bytes from one ncu capture of the
        # largest trailing update of the n = 32768 factorization, applied to
        # the average launch of this run
        traffic = tj["dram_over_algorithmic"] * prof["bytes"] / prof["launches"]
    roofline = {
        "kernel": "tc_gemm_persistent_kernel (tcgen05 trailing update, "
                  f"{ {'fp32': 'TF32x3', 'tf32': 'TF32', 'bf16': 'BF16', 'fp8': 'E4M3', 'fp64': 'n/a'}[args.precision] } operands)",
        "bound": "tensor", "achieved": tf_achieved, "peak": peak, "unit": "TFLOP/s",
        "frac": (tf_achieved / peak) if tf_achieved else None,
        "peak_source": f"{peak_kind} bf16 dense (sustained): the kernel is timed inside a long step",
        "traffic": traffic,
        "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of one "
                           "tc_gemm_persistent_kernel launch (32768 x 32256 x 512, TF32x3) "
                           "over its algorithmic bytes, times this run's average algorithmic "
                           "bytes per launch (profiles/tc_gemm_traffic.json)")
        if traffic is not None else None,
        "launches": prof["launches"], "kernel_ms_total": prof["ms"],
        "algorithmic_flops_per_launch": prof["flops"] / max(prof["launches"], 1),
        "algorithmic_bytes_per_launch": prof["bytes"] / max(prof["launches"], 1),
        "achieved_gbs": prof["bytes"] / (prof["ms"] * 1e-3) / 1e9 if prof["ms"] > 0 else None,
        "share_of_step_time": prof["ms"] * 1e-3 / tmax if tmax > 0 else None,
    }
    # the trailing update alone (the launches on the main stream), which
    # holds all GPCs but one while the look-ahead panel runs beside it
    side = prof.get("by_kernel_lookahead_stream", {}).get("tc_gemm")
    tc_all = prof["by_kernel"].get("tc_gemm")
    if side and tc_all and tc_all["ms"] > side["ms"]:
        roofline["trailing_update_only"] = {
            "launches": tc_all["launches"] - side["launches"],
            "achieved": (prof["flops"] - prof.get("flops_lookahead_tc", 0.0))
            / ((tc_all["ms"] - side["ms"]) * 1e-3) / 1e12
            if prof.get("flops_lookahead_tc") is not None else None,
            "note": "beside the look-ahead panel the update holds all GPCs but one "
                    "(16-CTA clusters, ELGB_OPT_TRAIL_GRID); the look-ahead stream's own "
                    "small updates are the rest of the launches"}
    # the operand kind's own ceiling on the same tensor pipe: TF32 issues at
    # half the bf16 rate, TF32x3 issues three TF32 products per update, E4M3
    # at twice the bf16 rate
    per_bf16 = {"fp32": 6.0, "tf32": 2.0, "bf16": 1.0, "fp8": 0.5}.get(args.precision)
    if per_bf16 and peak and tf_achieved:
        roofline["operand_ceiling_tflops"] = peak / per_bf16
        roofline["frac_of_operand_ceiling"] = tf_achieved * per_bf16 / peak
    breakdown = {k: {"launches": v["launches"], "ms_per_step": v["ms"]}
                 for k, v in prof_all["by_kernel"].items()}
    for k, v in prof_all.get("by_kernel_lookahead_stream", {}).items():
        breakdown[k]["lookahead_stream_ms_per_step"] = v["ms"]
    breakdown["note"] = ("one extra solve after the timed region with every launch group "
                         "bracketed by events (the brackets lengthen it by ~5 %)")
    cpu = None
    if args.cpu_baseline == "on":
        ns = min(args.cpu_n, n)
        tcpu, threads, cberr = cpu_sample(ns, q, args.seed)
        scale = flops_per_solve(n, q) / flops_per_solve(ns, q)
        cpu = {"value": 1.0 / (tcpu * scale), "unit": "solves/s", "cores": threads,
               "kind": "port",
               "sample": f"El::LU + lu::SolveAfter restatement over OpenBLAS, N(0,1) n={ns}, "
                         f"{q} RHS, {threads} threads: {tcpu:.3f} s, scaled to n={n} by flops "
                         f"(x{scale:.1f})",
               "backward_error_sample": cberr}
    prec_desc = {"fp32": "FP32 factors via TF32x3 tcgen05 updates",
                 "tf32": "FP32 storage, TF32 tcgen05 updates",
                 "bf16": "FP32 storage, BF16 tcgen05 updates",
                 "fp8": "FP32 storage, FP8 E4M3 tcgen05 trailing updates, per-panel scales",
                 "fp64": "plain FP64 getrf + getrs"}[args.precision]
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tmax / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp32": "f64+tf32x3", "tf32": "f64+tf32", "bf16": "f64+bf16", "fp8": "f64+e4m3",
                  "fp64": "f64"}[args.precision],
        "data": ("synthetic: seeded iid N(0,1) FP64 (device Philox generator)"
                 if args.kappa <= 0 else
                 f"synthetic: seeded A = U diag(sigma) V^T, U, V Haar, cond_2(A) = "
                 f"{args.kappa:g}; B iid N(0,1) (device Philox generator)"),
        "config": {"workload": f"mixed-precision {args.method.upper()} ({prec_desc}, FP64 "
                               f"residual) of A X = B, n={n}, {q} RHS, "
                               + ("A,B iid N(0,1)" if args.kappa <= 0 else
                                  f"A Haar-conditioned kappa={args.kappa:g}")
                               + ", to backward error <= n*eps64",
                   "n": n, "nrhs": q, "precision": args.precision, "method": args.method,
                   "kappa": args.kappa if args.kappa > 0 else None,
                   "tol": args.tol if args.tol > 0 else n * EPS64,
                   "max_iters": args.max_iters or None, "restart": args.restart or None,
                   "nb": args.nb or 512, "l2": "inputs larger than L2 (A is 8 GiB)",
                   "parallelism": f"replicas x{world}"},
        "tflops_eq": value * flops_per_solve(n, q) / 1e12,
        "backward_error": berr, "backward_error_bound": n * EPS64, "iterations": iters,
        "fell_back": any(i["fell_back"] for i in infos),
        "fp64_gpu": fp64,
        "e2e": e2e,
        "roofline": roofline,
        "cpu_baseline": cpu,
        "gpu_launches": launches,
        "kernel_time_breakdown": breakdown,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# batched workload: 4096 uneven systems, half LU / half Cholesky, 4 RHS
# ---------------------------------------------------------------------------
def _batched_systems(count, seed, q, device):
    """n ~ U{16..512}; even index: A iid N(0,1) (LU), odd: G^T G / n + I
    (Cholesky); B iid N(0,1).  Generated on the device in FP64."""
    import numpy as np
    import torch

    rng = np.random.default_rng(seed)
    ns = rng.integers(16, 513, count).astype(np.int32)
    kinds = ["lu" if i % 2 == 0 else "chol" for i in range(count)]
    aoff = np.concatenate([[0], np.cumsum(ns.astype(np.int64) ** 2)])
    A = torch.empty(int(aoff[-1]), dtype=torch.float64, device=device)
    g = torch.Generator(device=device).manual_seed(seed)
    for i, n in enumerate(ns):
        n = int(n)
        G = torch.randn(n, n, generator=g, device=device, dtype=torch.float64)
        if kinds[i] == "chol":
            G = G.t() @ G / n + torch.eye(n, device=device, dtype=torch.float64)
        A[aoff[i]:aoff[i + 1]] = G.t().contiguous().view(-1)
    B = torch.randn(int(ns.sum()) * q, generator=g, device=device, dtype=torch.float64)
    return ns, kinds, A, B


def _timed_replays(solver, steps, warmup, barrier):
    import torch

    for _ in range(max(warmup, 0)):
        solver.run()
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        solver.run()
    e1.record()
    e1.synchronize()
    barrier()
    return e0.elapsed_time(e1) / 1e3


def _dist_setup(world, local_rank):
    import torch

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def tmax(t):
        if dist is None:
            return t
        tt = torch.tensor([t], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        return float(tt.item())

    return dist, barrier, tmax


def batched_arm(args, rank, world, local_rank):
    import numpy as np
    import torch

    from elemental_gb300 import autotune
    from elemental_gb300 import device as D
    from elemental_gb300.batched import BatchedSolver

    from elemental_gb300 import shard

    dist, barrier, tmax_of = _dist_setup(world, local_rank)
    count, q = args.count or 4096, 4
    ctx = D.context(local_rank)
    # one batch for the whole job; each rank solves its cost-balanced share
    ns, kinds, A, B = _batched_systems(count, args.seed + 4, q, "cuda")
    my_count = count
    if world > 1:
        mine = shard.partition_by_cost(ns, world, kinds)[rank]
        kinds = [kinds[i] for i in mine]
        ns, A, B = BatchedSolver.subset(ns, q, A, B, mine)
    my_count = len(ns)
    nbt = autotune.nb_table("fp32")
    bs = BatchedSolver(ns, q, A, B, kinds=kinds, precisions=["fp32"] * my_count, nb_table=nbt,
                       ctx=ctx)
    clocks = ClockSampler(local_rank)
    l0 = ctx.launches()
    clocks.start()
    t = _timed_replays(bs, args.steps, args.warmup, barrier)
    clk = clocks.stop()
    launches = ctx.launches() - l0 - max(args.warmup, 0)
    t = tmax_of(t)
    res = bs.results()
    value = count * args.steps / t  # the whole batch, split over the ranks
    flops = bs.flops()
    berr = max(r["backward_error"] for r in res)
    ok = all(r["converged"] for r in res)
    # e2e: host (pinned) packed inputs -> device, one replay, solutions -> host
    Ah = host_tensor((A.numel(),))
    Bh = host_tensor((B.numel(),))
    Xh = host_tensor((B.numel(),))
    Ah.copy_(A)
    Bh.copy_(B)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        A.copy_(Ah, non_blocking=True)
        B.copy_(Bh, non_blocking=True)
        bs.run()
        Xh.copy_(bs.X, non_blocking=True)
        torch.cuda.synchronize()
    te = tmax_of(time.perf_counter() - t0)
    e2e = {"value": count * args.steps / te, "unit": "solves/s",
           "h2d_bytes_per_step": 8 * (A.numel() + B.numel()), "d2h_bytes_per_step": 8 * B.numel(),
           "api": "BatchedSolver.run (ElGBBatchedExecute) with H2D of the packed systems and "
                  "D2H of the solutions"}
    # always-FP64 in the same engine, and a per-matrix FP64 loop of the plain path
    bs64 = BatchedSolver(ns, q, A, B, kinds=kinds, precisions=["fp64"] * my_count, nb_table=nbt,
                         ctx=ctx)
    t64 = _timed_replays(bs64, 1, 1, barrier)
    res64 = bs64.results()
    bs64.close()
    sample = min(256, my_count)
    loop_t = 0.0
    aoff = np.concatenate([[0], np.cumsum(ns.astype(np.int64) ** 2)])
    boff = np.concatenate([[0], np.cumsum(ns.astype(np.int64) * q)])
    mats = []
    for i in range(sample):
        n = int(ns[i])
        Ai = D.colmajor(n, n)
        Ai.copy_(A[aoff[i]:aoff[i + 1]].view(n, n).t())
        Bi = D.colmajor(n, q)
        Bi.copy_(B[boff[i]:boff[i + 1]].view(q, n).t())
        mats.append((Ai, Bi))
    for Ai, Bi in mats[:4]:
        ctx.linear_solve(Ai.clone(), Bi.clone())
    barrier()
    t0 = time.perf_counter()
    for i, (Ai, Bi) in enumerate(mats):
        if kinds[i] == "lu":
            ctx.linear_solve(Ai, Bi.clone())
        else:
            ctx.hpd_solve(Ai, Bi.clone())
    torch.cuda.synchronize()
    loop_t = time.perf_counter() - t0
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0
    cpu = cpu_full = cpu_chp = None
    if args.cpu_baseline == "on":
        from oracle import oracle as O
        threads = os.cpu_count() or 1
        O.lib(threads)
        Ahost = A.cpu().numpy()
        Bhost = B.cpu().numpy()
        csample = min(512, my_count)
        t0 = time.perf_counter()
        for i in range(csample):
            n = int(ns[i])
            Ai = Ahost[aoff[i]:aoff[i + 1]].reshape(n, n, order="F")
            Bi = Bhost[boff[i]:boff[i + 1]].reshape(n, q, order="F")
            if kinds[i] == "lu":
                O.linear_solve(Ai, Bi)
            else:
                O.hpd_solve(Ai, Bi)
        tc = time.perf_counter() - t0
        cpu = {"value": csample / tc, "unit": "solves/s", "cores": threads, "kind": "port",
               "sample": f"El::LinearSolve / El::HPDSolve restatement over OpenBLAS, the first "
                         f"{csample} systems one by one, {threads} threads: {tc:.2f} s"}
    peaks, peak_kind = measured_peaks()
    alg_bytes = float(sum(8 * int(n) * int(n) + 24 * int(n) * q for n in ns))
    achieved = alg_bytes / (t / args.steps) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
        "dtype": "f64+f32", "data": "synthetic: seeded N(0,1) / G^T G/n + I, FP64, on the device",
        "config": {"workload": f"batched uneven solves: {count} systems, n ~ U{{16..512}}, half "
                               f"LU (N(0,1)) half Cholesky (G^T G/n + I), {q} RHS, FP32 factors + "
                               f"FP64 refinement, one persistent graph-replayed launch",
                   "count": count, "nrhs": q, "nb_table": nbt,
                   "l2": "inputs (%.1f GB) larger than L2" % (8 * A.numel() / 1e9),
                   "parallelism": f"systems split by cost over {world} rank(s)"},
        "tflops_eq": flops * args.steps * world / t / 1e12,
        "backward_error": berr, "all_converged": ok,
        "fp64_batched": {"solves_per_s": my_count / t64, "ms": 1e3 * t64,
                         "max_backward_error": max(r["backward_error"] for r in res64),
                         "speedup_fp32_ir_vs_fp64": t64 / (t / args.steps)},
        "fp64_per_matrix_loop": {"solves_per_s": sample / loop_t, "sample": sample,
                                 "api": "ElGBLinearSolve_d / ElGBHPDSolve_d one system at a "
                                        "time"},
        "e2e": e2e,
        "roofline": {"kernel": "batched_solve_kernel", "bound": "hbm", "achieved": achieved,
                     "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"] if peaks.get("hbm_gbs") else None,
                     "traffic": None,
                     "note": "algorithmic bytes = each system's A and B read once and X "
                             "written once; the per-CTA factorizations are SM-bound, so this "
                             "fraction is low by construction"},
        "cpu_baseline": cpu,
        "gpu_launches": launches,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    bs.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# learned selector workload: 10,000 conditioned systems
# ---------------------------------------------------------------------------
def selector_arm(args, rank, world, local_rank):
    import numpy as np

    from elemental_gb300 import autotune
    from elemental_gb300 import device as D
    from elemental_gb300 import selector as S
    from elemental_gb300.batched import BatchedSolver

    dist, barrier, tmax_of = _dist_setup(world, local_rank)
    ctx = D.context(local_rank)
    count = args.count or 10000
    t_setup = time.perf_counter()
    tr = S.conditioned_systems(args.train_count, args.seed + 5 + 104729 * rank)
    te = S.conditioned_systems(count, args.seed + 6 + 7919 * rank)
    nbt = autotune.nb_table("fp32")
    F, _, _ = S.extract_features(tr, ctx, nb_table=nbt)
    y, _ = S.outcome_labels(tr, ctx, nb_table=nbt)
    sel = S.PrecisionSelector(seed=0, ctx=ctx).fit(F, y, epochs=200, batch=256)
    th_fit, _ = S.fit_kappa_rule(F[:, S.LOG10_KAPPA_FEATURE].cpu().numpy(), y)
    setup_s = time.perf_counter() - t_setup
    ns = te["ns"]
    policies = {}

    def run(name, solver):
        t = tmax_of(_timed_replays(solver, args.steps, args.warmup, barrier))
        res = solver.results()
        d = S.summarize(res, t * 1e3 / args.steps)
        d["solves_per_s"] = count * args.steps * world / t
        d["device_s"] = sum(r["device_ms"] for r in res) * 1e-3
        if name != "fp64":
            d["choices"] = np.bincount([r["selector_choice"] for r in res], minlength=3).tolist()
        policies[name] = d
        solver.close()

    clocks = ClockSampler(local_rank)
    clocks.start()
    l0 = ctx.launches()
    run("mlp", BatchedSolver(ns, 1, te["A"], te["B"], selector_params=sel.params,
                             nb_table=nbt, ctx=ctx))
    launches = ctx.launches() - l0 - max(args.warmup, 0)
    clk = clocks.stop()
    run("fp64", BatchedSolver(ns, 1, te["A"], te["B"], precisions=["fp64"] * count,
                              nb_table=nbt, ctx=ctx))
    run("kappa_rule_theory", BatchedSolver(ns, 1, te["A"], te["B"], nb_table=nbt, ctx=ctx,
                                           selector_params=S.rule_network(*S.THEORY_THRESHOLDS)))
    run("kappa_rule_fitted", BatchedSolver(ns, 1, te["A"], te["B"], nb_table=nbt, ctx=ctx,
                                           selector_params=S.rule_network(*th_fit)))
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0
    m = policies["mlp"]
    line = {
        "metric": METRIC, "value": m["solves_per_s"], "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": m["ms"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64+f32", "data": "synthetic: seeded U diag(sigma) V^T, U, V Haar, FP64",
        "config": {"workload": f"learned precision selection: {count} systems, n log-uniform "
                               f"[64, 2048], kappa log-uniform [1e1, 1e12], 1 RHS, to backward "
                               f"error <= 1e-13; features -> MLP 16-64-64-3 -> solve fused in "
                               f"one launch; trained on {args.train_count} solver outcomes "
                               f"from a disjoint seed",
                   "count": count, "train_count": args.train_count, "nb_table": nbt,
                   "l2": "inputs larger than L2", "parallelism": f"independent systems x{world}"},
        "backward_error": m["max_backward_error"], "all_converged": m["all_converged"],
        "policies": policies,
        "speedup_vs_always_fp64": m["solves_per_s"] / policies["fp64"]["solves_per_s"],
        "setup_s": setup_s,
        "e2e": None, "roofline": None, "cpu_baseline": None,
        "gpu_launches": launches, "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# El::Inverse / El::OneCondition of one FP64 matrix
# ---------------------------------------------------------------------------
def inverse_arm(args, rank, world, local_rank):
    import numpy as np

    import elemental_gb300 as El
    from elemental_gb300 import device as D

    import torch

    dist, barrier, tmax_of = _dist_setup(world, local_rank)
    ctx = D.context(local_rank)
    n = args.n
    g = torch.Generator(device="cuda")
    g.manual_seed(args.seed + 7919 * rank)
    A0 = D.colmajor(n, n)
    A0.copy_(torch.randn(n, n, generator=g, device="cuda", dtype=torch.float64).t())
    A = D.colmajor(n, n)
    flops = 2.0 * n ** 3  # LAPACK's count for an inverse (getrf + getri)

    def step():
        A.copy_(A0)
        ctx.inverse(A)

    for _ in range(max(args.warmup, 0)):
        step()
    barrier()
    clocks = ClockSampler(local_rank)
    clocks.start()
    l0 = ctx.launches()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    e1.synchronize()
    barrier()
    launches = ctx.launches() - l0
    clk = clocks.stop()
    t = tmax_of(e0.elapsed_time(e1) / 1e3)
    info = ctx.status()
    X = A.cpu().numpy()
    Ah = A0.cpu().numpy()
    resid = float(np.linalg.norm(Ah @ X - np.eye(n)) /
                  (np.linalg.norm(Ah) * np.linalg.norm(X)))
    # OneCondition: wall clock (it synchronizes to read the norms)
    ctx.one_condition(A0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    cond = ctx.one_condition(A0)
    t_cond = time.perf_counter() - t0
    # end to end through Elemental's C ABI on pinned host memory
    e2e = None
    if args.e2e == "on":
        Hp = host_tensor((n, n))
        H0 = host_tensor((n, n))
        H0.copy_(A0.t())
        Hp.copy_(H0)
        M = El.Matrix(Hp.numpy().T)
        El.Inverse(M)
        te = 0.0
        for _ in range(args.steps):
            Hp.copy_(H0)
            t0 = time.perf_counter()
            El.Inverse(M)
            te += time.perf_counter() - t0
        e2e = {"value": args.steps * world / tmax_of(te), "unit": "inverses/s",
               "h2d_bytes_per_step": 8 * n * n, "d2h_bytes_per_step": 8 * n * n,
               "api": "ElInverse_d (El::Matrix handle on ElGBHostAlloc host memory, pinned by registration)",
               "max_abs_diff_vs_device_run": float(np.abs(M.array - X).max())}
        del M, Hp, H0
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0
    cpu = cpu_full = cpu_chp = None
    if args.cpu_baseline == "on":
        from oracle import oracle as O

        ns = min(2048, n)
        threads = os.cpu_count() or 1
        O.set_threads(threads)
        As = np.random.default_rng(args.seed).standard_normal((ns, ns))
        O.inverse(As, nb=128)
        t0 = time.perf_counter()
        O.inverse(As, nb=128)
        tc = time.perf_counter() - t0
        nf = 512
        Fs = np.random.default_rng(args.seed + 1).standard_normal((nf, nf))
        t0 = time.perf_counter()
        O.lu_full(Fs)
        tf = time.perf_counter() - t0
        cpu_full = {"n": nf, "seconds": tf, "scaled_seconds_at_gpu_n": tf * (min(n, 4096) / nf) ** 3,
                    "kind": "port", "cores": threads}
        Gs = np.random.default_rng(args.seed + 2).standard_normal((nf, nf))
        Ss = Gs.T @ Gs / nf + np.eye(nf)
        t0 = time.perf_counter()
        O.cholesky_piv(Ss, "L", nb=128)
        tcp = time.perf_counter() - t0
        cpu_chp = {"n": nf, "seconds": tcp,
                   "scaled_seconds_at_gpu_n": tcp * (min(n, 4096) / nf) ** 3,
                   "kind": "port", "cores": threads}
        cpu = {"value": (ns / n) ** 3 / tc, "unit": "inverses/s", "cores": threads,
               "kind": "port",
               "sample": f"El::Inverse restatement (El::LU + TriangularInverse + the backward "
                         f"sweep, OpenBLAS) at n={ns}, {threads} threads: {tc:.3f} s, scaled "
                         f"to n={n} by n^3"}
    # El::LU(A, P, Q) with full pivoting (unblocked, as the reference) of an
    # n_full x n_full matrix, and the oracle's restatement on a CPU sample
    n_full = min(n, 4096)
    F0 = D.colmajor(n_full, n_full)
    F0.copy_(A0[:n_full, :n_full])
    F = D.colmajor(n_full, n_full)
    F.copy_(F0)
    ctx.lu_full(F)
    F.copy_(F0)
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    ctx.lu_full(F)
    f1.record(stream)
    f1.synchronize()
    t_full = f0.elapsed_time(f1) / 1e3
    lu_full = {"n": n_full, "seconds": t_full,
               "gflops_eq": 2.0 / 3.0 * n_full ** 3 / t_full / 1e9,
               "bound": "one pass over the trailing block per step (read + write)",
               "achieved_gbs": 16.0 * n_full ** 3 / 3.0 / t_full / 1e9,
               "status": ctx.status()}
    del F, F0
    # El::Cholesky(LOWER, A, P) with diagonal pivoting of an SPD matrix
    # G^T G / n + I (G the same leading block; input synthesis, not timed)
    G = A0[:n_full, :n_full]
    S0 = D.colmajor(n_full, n_full)
    S0.copy_((G.t() @ G) / n_full + torch.eye(n_full, dtype=torch.float64, device="cuda"))
    S = D.colmajor(n_full, n_full)
    S.copy_(S0)
    ctx.cholesky_piv(S)
    S.copy_(S0)
    torch.cuda.synchronize()
    f0.record(stream)
    ctx.cholesky_piv(S)
    f1.record(stream)
    f1.synchronize()
    t_chp = f0.elapsed_time(f1) / 1e3
    chol_piv = {"n": n_full, "seconds": t_chp,
                "gflops_eq": 1.0 / 3.0 * n_full ** 3 / t_chp / 1e9,
                "bound": "one pass over the trailing lower triangle per step",
                "status": ctx.status()}
    del S, S0, G
    value = args.steps * world / t
    fp64_peak = ctx.fp64_peak_tflops()
    line = {
        "metric": METRIC, "value": value, "unit": "inverses/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded iid N(0,1) FP64 (device Philox generator)",
        "config": {"workload": f"El::Inverse of one n={n} FP64 matrix (getrf + getrs on the "
                               f"identity), N(0,1); El::OneCondition of the same matrix; "
                               f"El::LU with full pivoting of its leading "
                               f"{min(n, 4096)} x {min(n, 4096)} block; El::Cholesky with "
                               f"diagonal pivoting of G^T G / n + I of that block",
                   "n": n, "l2": "inputs larger than L2" if 8 * n * n > 129e6 else "in L2",
                   "parallelism": f"replicas x{world}"},
        "tflops_eq": flops * value / world / 1e12,
        "residual_AX_minus_I": resid, "status": info,
        "one_condition": {"value": cond, "seconds": t_cond},
        "lu_full_pivoting": dict(lu_full, cpu_sample=cpu_full if cpu else None),
        "cholesky_diagonal_pivoting": dict(chol_piv, cpu_sample=cpu_chp if cpu else None),
        "roofline": {"bound": "fp64 FMA pipe (tcgen05 has no FP64 kind)",
                     "achieved": flops * value / world / 1e12, "peak": fp64_peak,
                     "unit": "TFLOP/s", "frac": flops * value / world / 1e12 / fp64_peak,
                     "peak_source": "FP64 FMA throughput probe (ElGBProbeFP64Peak) on this GPU",
                     "traffic": None},
        "e2e": e2e, "cpu_baseline": cpu, "gpu_launches": launches, "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# plain FP64 El::HPDSolve (potrf + potrs) of one SPD system
# ---------------------------------------------------------------------------
def cholesky_arm(args, rank, world, local_rank):
    """El::HPDSolve(LOWER, NORMAL, A, B) (src/lapack_like/solve/HPD.cpp:47-55):
    a copy of A, El::Cholesky (LowerVariant3Blocked) and cholesky::SolveAfter
    on A = G^T G / n + I, G iid N(0,1), B n x nrhs iid N(0,1).  One step = one
    HPDSolve; the FP64 FMA pipe bounds it (tcgen05 has no FP64 kind)."""
    import numpy as np

    import elemental_gb300 as El
    from elemental_gb300 import device as D

    import torch

    dist, barrier, tmax_of = _dist_setup(world, local_rank)
    ctx = D.context(local_rank)
    n, q = args.n, args.nrhs
    g = torch.Generator(device="cuda")
    g.manual_seed(args.seed + 7919 * rank)
    # input synthesis, not timed: G^T G in FP32 (exactly symmetric after the
    # averaging below), then FP64 + I, so that every eigenvalue is >= ~1
    G = torch.randn(n, n, generator=g, device="cuda", dtype=torch.float32)
    S = (G.t() @ G).double().div_(n)
    del G
    S = S.add_(S.t().clone()).mul_(0.5)
    S.diagonal().add_(1.0)
    A0 = D.colmajor(n, n)
    A0.copy_(S)
    del S
    B0 = D.colmajor(n, q)
    B0.copy_(torch.randn(q, n, generator=g, device="cuda", dtype=torch.float64).t())
    X = D.colmajor(n, q)
    flops = 1.0 / 3.0 * n ** 3 + 2.0 * n * n * q

    def step():
        X.copy_(B0)
        ctx.hpd_solve(A0, X, uplo=0, nb=args.nb)

    for _ in range(max(args.warmup, 0)):
        step()
    barrier()
    clocks = ClockSampler(local_rank)
    clocks.start()
    l0 = ctx.launches()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    e1.synchronize()
    barrier()
    launches = ctx.launches() - l0
    clk = clocks.stop()
    t = tmax_of(e0.elapsed_time(e1) / 1e3)
    info = ctx.status()
    berr = ctx.backward_error(A0, X, B0)
    # end to end through Elemental's C ABI on pinned host memory
    e2e = None
    if args.e2e == "on":
        Ah = host_tensor((n, n))
        Ah.copy_(A0.t())
        Bh0 = host_tensor((q, n))
        Bh0.copy_(B0.t())
        Bh = host_tensor((q, n))
        Am = El.Matrix(Ah.numpy().T)
        Bh.copy_(Bh0)
        Bm = El.Matrix(Bh.numpy().T)
        El.HPDSolve(Am, Bm)
        te = 0.0
        for _ in range(args.steps):
            Bh.copy_(Bh0)
            t0 = time.perf_counter()
            El.HPDSolve(Am, Bm)
            te += time.perf_counter() - t0
        Xd = X.cpu().numpy()
        e2e = {"value": args.steps * world / tmax_of(te), "unit": "solves/s",
               "h2d_bytes_per_step": 8 * n * n + 8 * n * q, "d2h_bytes_per_step": 8 * n * q,
               "api": "ElHPDSolve_d (El::Matrix handles on ElGBHostAlloc host memory, pinned by registration)",
               "max_abs_diff_vs_device_run": float(np.abs(Bm.array - Xd).max())}
        del Am, Bm, Ah, Bh, Bh0
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0
    cpu = None
    if args.cpu_baseline == "on":
        from oracle import oracle as O

        ns = min(4096, n)
        threads = os.cpu_count() or 1
        O.set_threads(threads)
        rng = np.random.default_rng(args.seed)
        Gs = rng.standard_normal((ns, ns))
        Ss = Gs.T @ Gs / ns + np.eye(ns)
        Bs = rng.standard_normal((ns, q))
        O.hpd_solve(Ss, Bs, "L", nb=128)
        t0 = time.perf_counter()
        Xs = O.hpd_solve(Ss, Bs, "L", nb=128)
        tc = time.perf_counter() - t0
        fs = 1.0 / 3.0 * ns ** 3 + 2.0 * ns * ns * q
        cpu = {"value": fs / flops / tc, "unit": "solves/s", "cores": threads, "kind": "port",
               "sample": f"El::HPDSolve restatement (El::Cholesky LowerVariant3Blocked + "
                         f"cholesky::SolveAfter, OpenBLAS) at n={ns}, {q} RHS, {threads} "
                         f"threads: {tc:.3f} s, scaled to n={n} by the flop count",
               "backward_error_sample": float(O.backward_error(Ss, Xs, Bs))}
    value = args.steps * world / t
    fp64_peak = ctx.fp64_peak_tflops()
    achieved = flops * value / world / 1e12
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: SPD G^T G / n + I, G and B seeded iid N(0,1) (device Philox "
                "generator)",
        "config": {"workload": f"plain FP64 El::HPDSolve (copy + potrf + potrs, lower) of one "
                               f"n={n} SPD system, {q} RHS",
                   "n": n, "nrhs": q,
                   "l2": "inputs larger than L2" if 8 * n * n > 129e6 else "in L2",
                   "parallelism": f"replicas x{world}"},
        "tflops_eq": achieved, "backward_error": berr,
        "backward_error_bound_n_eps64": n * EPS64, "status": info,
        "roofline": {"bound": "fp64 FMA pipe (tcgen05 has no FP64 kind)",
                     "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp64_peak if fp64_peak else None,
                     "peak_source": "FP64 FMA throughput probe (ElGBProbeFP64Peak) on this GPU",
                     "traffic": None},
        "e2e": e2e, "cpu_baseline": cpu, "gpu_launches": launches, "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.n is None:
        args.n = {"inverse": 8192, "cholesky": 16384}.get(args.workload, 32768)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return reference_arm(args, rank)
    if args.workload == "batched":
        return batched_arm(args, rank, world, local_rank)
    if args.workload == "selector":
        return selector_arm(args, rank, world, local_rank)
    if args.workload == "inverse":
        return inverse_arm(args, rank, world, local_rank)
    if args.workload == "cholesky":
        return cholesky_arm(args, rank, world, local_rank)
    return gpu_arm(args, rank, world, local_rank)


if __name__ == "__main__":
    sys.exit(main())
