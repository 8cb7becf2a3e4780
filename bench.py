"""Benchmark of the LU-solve hot path on GB300.

Headline workload (a "step"): one dense solve x = A^-1 b at n = 8192 with one
right-hand side, A = U diag(s) V^T, U and V Haar-orthogonal (Q of the QR of a
seeded Gaussian, columns sign-fixed by diag(R)), s log-spaced from 1 to
1/cond.  The step runs the mixed-precision path (FP32 factorisation + FP64
iterative refinement to a normwise backward error <= 1e-12) when it is
available, otherwise the plain FP64 LU path.  Throughput is reported as
FP64-equivalent TFLOP/s, (2n^3/3 + 2n^2 nrhs) per solve.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times TMV's own CPU path on the host cores on the same
workload (TMV 0.76 compiled from its sources on this machine where the build
step found them, else the oracle's C restatement of the same algorithm) and
prints the same JSON line with "impl": "reference".
Inputs are 512 MiB (A in FP64), larger than the 129 MB L2, so no flush is
needed between steps.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "n=8192 LU-solve TFLOP/s mixed+IR vs FP64 GPU at 1e-12 rel err; batched solves/s"


def max_over_ranks(ms: float, device) -> float:
    """The slowest rank's time (replicas: every rank runs its own workload),
    then a barrier so that no rank starts other work inside another's
    measurement.  Works with any process-group backend (nccl on the GPUs,
    gloo in the CPU tests)."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def aggregate_value(units_per_rank: float, world: int, ms: float) -> float:
    """Whole-job throughput: the units all ranks processed over the slowest
    rank's time (weak scaling, fixed work per rank)."""
    return units_per_rank * world / (ms * 1e-3)


def lu_solve_flops(n: int, nrhs: int) -> float:
    return 2.0 * n ** 3 / 3.0 + 2.0 * n * n * nrhs


def haar_matrix_torch(n: int, cond: float, seed: int, dev):
    """A = U diag(s) V^T in FP64 on the device (setup, not timed)."""
    import torch

    rng = np.random.default_rng(seed)
    out = []
    for _ in range(2):
        g = torch.from_numpy(rng.standard_normal((n, n))).to(dev)
        q, r = torch.linalg.qr(g)
        q *= torch.sign(torch.diagonal(r)).unsqueeze(0)
        out.append(q)
        del g, r
    U, V = out
    s = torch.logspace(0, -np.log10(cond), n, dtype=torch.float64, device=dev)
    A = (U * s.unsqueeze(0)) @ V.t()
    b = torch.from_numpy(rng.standard_normal(n)).to(dev)
    return A, b


def haar_matrix_numpy(n: int, cond: float, seed: int):
    rng = np.random.default_rng(seed)
    qs = []
    for _ in range(2):
        q, r = np.linalg.qr(rng.standard_normal((n, n)))
        qs.append(q * np.sign(np.diag(r))[None, :])
    U, V = qs
    s = np.logspace(0, -np.log10(cond), n)
    A = (U * s[None, :]) @ V.T
    b = rng.standard_normal(n)
    return np.asfortranarray(A), b


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi every 20 ms from
    start() to stop(), each line stamped with the host time it was read;
    window() marks the timed region, and stop() summarises the samples read
    inside it (or, if the region was shorter than the sampling period, all
    samples under load, saying so)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int = 0):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[tuple[float, str]] = []
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def window(self, t0: float, t1: float):
        self.t0, self.t1 = t0, t1

    def median_between(self, t0: float, t1: float) -> float | None:
        """Median SM clock (MHz) of the samples read between t0 and t1."""
        time.sleep(0.05)
        sm = []
        for t, ln in list(self.lines):
            if t0 <= t <= t1:
                f = [x.strip() for x in ln.split(",")]
                try:
                    sm.append(float(f[1]))
                except (IndexError, ValueError):
                    pass
        return float(np.median(sm)) if sm else None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.05)  # the last in-window sample
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

        def summarise(lines):
            sm, mx, reasons = [], None, set()
            for _, ln in lines:
                f = [x.strip() for x in ln.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx = float(f[2])
                except ValueError:
                    continue
                for nm, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
            return sm, mx, reasons

        inside = [x for x in self.lines if self.t0 is not None and self.t0 <= x[0] <= self.t1]
        sm, mx, reasons = summarise(inside)
        scope = "timed region"
        if not sm:
            sm, mx, reasons = summarise(self.lines)
            scope = "all samples under load (timed region shorter than the sampling period)"
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm), "scope": scope}


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        d["_source"] = "measured"
        return d
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
            "_source": "fallback"}


# The FP64 FMA rate every FP64-bound fraction is measured against: taken in
# this process by the library's DFMA throughput kernel (tmvg_probe_fp64_rate)
# right after the headline's timed region, under the same sampled clocks.
FP64_PEAK: dict = {"tflops": None}


def measure_fp64_peak(h, clocks) -> dict:
    t0 = time.time()
    tf = h.fp64_rate()
    t1 = time.time()
    FP64_PEAK.update({"tflops": round(tf, 4), "sm_mhz": clocks.median_between(t0, t1),
                      "source": "tmvg_probe_fp64_rate (DFMA throughput kernel) in this run"})
    return dict(FP64_PEAK)


def fp64_roofline(achieved_tflops: float) -> dict:
    pk = FP64_PEAK["tflops"]
    return {"bound": "fp64", "achieved": round(achieved_tflops, 4), "peak": pk, "unit": "TFLOP/s",
            "frac": round(achieved_tflops / pk, 4) if pk else None,
            "peak_source": FP64_PEAK.get("source", "not measured")}


def run_gpu(args) -> dict:
    import torch

    from tmv_gb300 import linalg
    from tmv_gb300 import _lib

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)

    if args.path in ("band", "complex"):
        h = linalg.handle(local)
        FP64_PEAK.update({"tflops": round(h.fp64_rate(), 4), "source": "tmvg_probe_fp64_rate in this run"})
        with_cpu = rank == 0 and not args.no_cpu_baseline
        w = (band_workloads(dev, with_cpu, args.band_count) if args.path == "band"
             else complex_workload(dev, with_cpu))
        return {"path": args.path, "fp64_peak": dict(FP64_PEAK), "workloads": w} if rank == 0 else None

    if args.path == "batched":
        h = linalg.handle(local)
        FP64_PEAK.update({"tflops": round(h.fp64_rate(), 4), "source": "tmvg_probe_fp64_rate in this run"})
        b = batched_bench(dev, args, with_cpu=(rank == 0 and not args.no_cpu_baseline))
        out = {"metric": "batched uneven FP64 LU solves/s", "value": b["value"], "unit": "solves/s",
               "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
               "ms_per_step": b["ms_per_batch"], "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64", "data": "synthetic",
               "config": {"workload": b["config"], "systems": b["systems"]},
               "roofline": b["roofline"], "gpu_launches": 1}
        if "cpu_baseline" in b:
            out["cpu_baseline"] = b["cpu_baseline"]
        out["mixed"] = b["mixed"]
        if world > 1:
            torch.distributed.destroy_process_group()
        return out if rank == 0 else None

    n, nrhs, cond = args.n, 1, args.cond
    cache = Path(args.matrix_cache) if args.matrix_cache else None
    if cache is not None and cache.exists():
        saved = torch.load(cache, map_location=dev)
        A, b = saved["A"], saved["b"]
    else:
        A, b = haar_matrix_torch(n, cond, seed=3 + rank, dev=dev)
        if cache is not None:
            torch.save({"A": A, "b": b}, cache)
    Acm = linalg.colmajor(A)
    del A
    B = b.view(n, 1).clone()
    h = linalg.handle(local)
    stream = torch.cuda.current_stream(dev)
    mixed = args.path == "mixed"
    Xm = torch.empty((nrhs, n), dtype=torch.float64, device=dev).t()
    infos = []

    def step():
        if mixed:
            _, info = linalg.solve_mixed(Acm, B, max_iter=10, tol=1e-12, X=Xm)
            infos.append((info.iterations, info.converged, info.backward_error))
            return Xm
        X, LU, P = linalg.divide(Acm, B)
        return X

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            out = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps, out

    clocks = ClockSampler(local)
    clocks.start()
    # the plain FP64 GPU LU on the same system (the comparison point)
    if args.no_extras:
        fp64_ms, X64 = float("nan"), None
    else:
        fp64_ms, X64 = timed(lambda: linalg.divide(Acm, B)[0], steps=2, warmup=1)

    for _ in range(args.warmup):
        X = step()
    torch.cuda.synchronize()
    infos.clear()
    launches0 = h.launches()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    tw0 = time.time()
    e0.record(stream)
    for _ in range(args.steps):
        X = step()
    e1.record(stream)
    torch.cuda.synchronize()
    clocks.window(tw0, time.time())
    fp64_peak = measure_fp64_peak(h, clocks)
    ms = e0.elapsed_time(e1)
    if world > 1:
        ms = max_over_ranks(ms, dev)
    clk = clocks.stop()
    launches = (h.launches() - launches0) // max(args.steps, 1)
    ms_step = ms / args.steps
    # per-kernel-class breakdown in a second pass of the same steps: the
    # library records CUDA events on its streams around every span, which
    # costs about 3 % of a step, so the timed pass above runs without them
    bsteps = max(1, min(args.steps, 3))
    h.timing_enable(True)
    torch.cuda.synchronize()
    b0 = torch.cuda.Event(enable_timing=True)
    b1 = torch.cuda.Event(enable_timing=True)
    b0.record(stream)
    for _ in range(bsteps):
        step()
    b1.record(stream)
    torch.cuda.synchronize()
    kernels = kernel_breakdown(h, bsteps, b0.elapsed_time(b1) / bsteps)
    h.timing_enable(False)
    flops = lu_solve_flops(n, nrhs)
    value = aggregate_value(flops, world, ms_step) / 1e12

    # accuracy of the last solve: normwise backward error, and forward
    # difference from the FP64 GPU LU solution
    x = X[:, 0]
    r = B[:, 0] - Acm @ x
    berr = float(r.abs().max() / (Acm.abs().sum(dim=1).max() * x.abs().max() + B.abs().max()))
    fwd = float((X - X64).norm() / X64.norm()) if X64 is not None else None

    roof = dominant_roofline(kernels, mixed)
    e2e = None if args.no_extras else e2e_host(args, Acm, B, n, nrhs, mixed)

    if rank == 0 and not args.no_cpu_baseline and not args.no_extras:
        cpu = cpu_baseline(np.asfortranarray(Acm.cpu().numpy()), B.cpu().numpy(), n, cond)
    else:
        cpu = None
    its = [i[0] for i in infos]
    sweep = None
    if mixed and not args.no_extras and not args.no_sweep:
        sweep = cond_sweep(dev, n, cond, Acm, B, X64, fp64_ms)
    out = {
        "metric": METRIC, "value": round(value, 4), "unit": "TFLOP/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms_step, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64" if mixed else "f64", "data": "synthetic",
        "fp64_gpu_lu": {"value": round(flops / (fp64_ms * 1e-3) / 1e12, 4), "unit": "TFLOP/s",
                        "ms_per_solve": round(fp64_ms, 3)},
        "speedup_vs_fp64_gpu_lu": (round(fp64_ms / ms_step, 3) if X64 is not None else None),
        "accuracy": {"backward_error": berr, "forward_rel_diff_vs_fp64_gpu_lu": fwd,
                     "ir_iterations": (max(its) if its else None),
                     "converged": all(i[1] == 1 for i in infos) if infos else None},
        "equal_accuracy": (sweep["equal_accuracy_at_headline_cond"] if sweep else None),
        "config": {"workload": (f"dense solve n={n}, 1 RHS, cond={cond:g}, Haar U/V; "
                                + ("FP32 LU + FP64 iterative refinement to backward error 1e-12"
                                   if mixed else "FP64 GPU LU")),
                   "path": args.path, "n": n, "nrhs": nrhs, "cond": cond,
                   "l2": "inputs larger than L2 (A is 512 MiB FP64); no flush"},
        "roofline": roof, "e2e": e2e, "gpu_launches": int(launches),
        "clocks": clk, "fp64_peak": fp64_peak,
        "cond_sweep": (sweep["rows"] if sweep else None), "kernels": kernels,
    }
    if cpu is not None:
        out["cpu_baseline"] = cpu
    if not args.no_extras and not args.no_batched:
        out["batched"] = batched_bench(dev, args, with_cpu=(rank == 0 and not args.no_cpu_baseline))
    if not args.no_extras:
        out["other_workloads"] = other_workloads(dev, with_cpu=(rank == 0 and not args.no_cpu_baseline))
    if world > 1:
        torch.distributed.destroy_process_group()
    return out if rank == 0 else None


def cond_sweep(dev, n: int, head_cond: float, A_head, B_head, X64_head, fp64_ms_head) -> dict:
    """The mixed solve against the FP64 GPU LU at every condition number of
    the workload (1e2, 1e4, 1e6; n = 8192, Haar U/V, 1 right-hand side):
    * at the headline tolerance (normwise backward error <= 1e-12);
    * at equal accuracy: the largest tolerance in (1e-14, 3e-15, 1e-15, 4e-16)
      whose solution differs from the FP64 GPU LU's by at most 50 cond eps
      (relative 2-norm), the accuracy of the FP64 LU itself;
    each with its time, refinement steps and speed-up over the FP64 GPU LU on
    the same system (CUDA events, device-resident inputs)."""
    import torch

    from tmv_gb300 import linalg

    stream = torch.cuda.current_stream(dev)

    def timed(fn, reps, warm=1):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            r = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps, r

    eps = float(np.finfo(np.float64).eps)
    rows, head = [], None
    for cond in (1e2, 1e4, 1e6):
        if cond == head_cond:
            A, B, X64, fp64_ms = A_head, B_head, X64_head, fp64_ms_head
        else:
            a, b = haar_matrix_torch(n, cond, seed=3, dev=dev)
            A = linalg.colmajor(a)
            del a
            B = b.view(n, 1).clone()
            fp64_ms, X64 = timed(lambda: linalg.divide(A, B)[0], reps=2)
        bound = 50.0 * cond * eps

        def mixed_at(tol, max_iter):
            ms, (X, info) = timed(lambda: linalg.solve_mixed(A, B, max_iter=max_iter, tol=tol,
                                                             raise_not_converged=False), reps=3)
            fwd = float((X - X64).norm() / X64.norm())
            return {"tol": tol, "ms_per_solve": round(ms, 3),
                    "tflops": round(lu_solve_flops(n, 1) / (ms * 1e-3) / 1e12, 4),
                    "ir_iterations": int(info.iterations), "converged": int(info.converged) == 1,
                    "backward_error": float(info.backward_error),
                    "forward_rel_diff_vs_fp64_gpu_lu": fwd,
                    "speedup_vs_fp64_gpu_lu": round(fp64_ms / ms, 3)}

        row = {"cond": cond, "fp64_gpu_lu_ms": round(fp64_ms, 3),
               "mixed_tol_1e-12": mixed_at(1e-12, 10), "equal_accuracy_bound": bound}
        eq = None
        for tol in (1e-14, 3e-15, 1e-15, 4e-16):
            r = mixed_at(tol, 30)
            if r["converged"] and r["forward_rel_diff_vs_fp64_gpu_lu"] <= bound:
                eq = r
                break
        row["mixed_equal_accuracy"] = eq
        rows.append(row)
        if cond == head_cond:
            head = eq
        del A, B, X64
        torch.cuda.empty_cache()
    return {"rows": rows, "equal_accuracy_at_headline_cond": head}


def batched_workload(count: int, seed: int = 4):
    """Systems n_i ~ U{8..256}, nrhs_i ~ U{1..16}; A_i ~ N(0,1) + 2 sqrt(n_i) I,
    B_i ~ N(0,1), packed column-major in order."""
    rng = np.random.default_rng(seed)
    n = rng.integers(8, 257, size=count).astype(np.int64)
    r = rng.integers(1, 17, size=count).astype(np.int64)
    return n, r


def batched_bench(dev, args, with_cpu: bool) -> dict:
    import torch

    from tmv_gb300.batched import BatchPlan

    count = args.batch_count
    n, r = batched_workload(count)
    plan = BatchPlan(n, r, tune=True)
    g = torch.Generator(device=dev)
    g.manual_seed(4)
    A0 = torch.randn(plan.a_elems, dtype=torch.float64, device=dev, generator=g)
    B0 = torch.randn(plan.b_elems, dtype=torch.float64, device=dev, generator=g)
    # diagonal shift 2 sqrt(n_i)
    idx = np.concatenate([plan.a_off[s] + np.arange(n[s]) * (n[s] + 1) for s in range(count)])
    shift = np.repeat(2.0 * np.sqrt(n.astype(np.float64)), n)
    A0[torch.from_numpy(idx).to(dev)] += torch.from_numpy(shift).to(dev)
    A, B = A0.clone(), B0.clone()
    P = torch.empty(plan.p_elems, dtype=torch.int64, device=dev)
    st = torch.empty(count, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(max(args.warmup, 1)):
        A.copy_(A0)
        B.copy_(B0)
        plan.solve(A, B, P, st)
    total = 0.0
    steps = max(args.steps, 1)
    for _ in range(steps):
        A.copy_(A0)
        B.copy_(B0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plan.solve(A, B, P, st)
        e1.record(stream)
        torch.cuda.synchronize()
        total += e0.elapsed_time(e1)
    ms = total / steps
    bad = int((st != 0).sum().item())
    tflops = plan.flops / (ms * 1e-3) / 1e12
    out = {"value": round(count / (ms * 1e-3), 1), "unit": "solves/s", "systems": count,
           "ms_per_batch": round(ms, 3), "tflops_fp64": round(tflops, 4),
           "roofline": {"kernel": "batched_lu_kernel (FP64 LU + solve, one persistent launch)",
                        **fp64_roofline(tflops),
                        "algorithmic_flop_per_launch": plan.flops},
           "panel_widths_by_class": plan.panel_widths, "singular_systems": bad,
           "config": "n_i ~ U{8..256}, nrhs_i ~ U{1..16}, A_i ~ N(0,1) + 2 sqrt(n_i) I, FP64, "
                     "CUDA graph replay, tiles from the autotuner"}
    # the same batch with FP32 factors and FP64 refinement to a backward error
    # of 1e-12 per column (A is read, not modified; B receives X)
    X64 = B.clone()
    for _ in range(max(args.warmup, 1)):
        B.copy_(B0)
        plan.solve_mixed(A0, B, max_iter=10, tol=1e-12, P=P, status=st)
    total = 0.0
    for _ in range(steps):
        B.copy_(B0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _, _, iters, berr = plan.solve_mixed(A0, B, max_iter=10, tol=1e-12, P=P, status=st)
        e1.record(stream)
        torch.cuda.synchronize()
        total += e0.elapsed_time(e1)
    mms = total / steps
    out["mixed"] = {
        "value": round(count / (mms * 1e-3), 1), "unit": "solves/s", "ms_per_batch": round(mms, 3),
        "fp64_equivalent_tflops": round(plan.flops / (mms * 1e-3) / 1e12, 4),
        "speedup_vs_fp64_batched": round(ms / mms, 3),
        "iterations_max": int(iters.max().item()), "iterations_mean": round(float(iters.float().mean().item()), 3),
        "backward_error_max": float(berr.max().item()),
        "forward_rel_diff_vs_fp64_batched": float(((B - X64).abs().max() / X64.abs().max()).item()),
        "unconverged_or_singular": int((st != 0).sum().item()),
        "kernel": "batched_mixed_kernel (FP32 LU + FP64 residual refinement, one persistent launch)",
        # the FP64 solves' work (2n^3/3 + 2n^2 r per system), delivered at the
        # same 1e-12 backward error, against the FP64 FMA rate
        "roofline": {**fp64_roofline(plan.flops / (mms * 1e-3) / 1e12), "work": "FP64-equivalent"},
        "config": "the same 20000 systems; per column ||b - A x||_inf <= 1e-12 (||A||_inf ||x||_inf + ||b||_inf), "
                  "at most 10 corrections"}
    if with_cpu:
        orc, kind, what = cpu_reference()
        cores = os.cpu_count() or 1
        orc.set_threads(cores)
        m = min(count, args.batch_cpu_sample)
        hA = A0[: int(plan.a_off[m - 1] + n[m - 1] ** 2)].cpu().numpy()
        hB = B0[: int(plan.b_off[m - 1] + n[m - 1] * r[m - 1])].cpu().numpy().copy()
        t0 = time.perf_counter()
        orc.batched_divide(n[:m], r[:m], plan.a_off[:m], plan.b_off[:m], hA, hB)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(m / dt, 1), "unit": "solves/s", "cores": cores,
                               "kind": kind,
                               "sample": f"first {m} systems of the batch, OpenMP over systems "
                                         f"({dt:.2f} s); {what}"}
    plan.close()
    return out


# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) per algorithmic
# byte of each kernel class, from one ncu capture of the class's main kernel
# on the n = 8192 workload (commands and figures in profiles/):
#   panel: lu_panel_leaf_kernel, k = 320: 2.08 MB / 4.03 MB
#   trailing_update: tf32x3_update_kernel, k = 256: 432.1 MB / 495.7 MB
#   tri_solve: trsv_pub_async_kernel: 140.4 MB / 138.5 MB
# The traffic of a span is its algorithmic bytes times the ratio.
NCU_TRAFFIC_PER_ALG_BYTE: dict = {"panel": 0.516, "trailing_update": 0.872, "tri_solve": 1.014}

KERNEL_NAMES = {
    "panel": "lu_panel_leaf_kernel (16-CTA cluster, 512 threads, one register-resident FP32 panel row "
             "per thread, 8-column leaves)",
    "trailing_update": "U12 solve + A22 -= L21 U12 (FP32: u12_reg_kernel + tf32x3_update_kernel "
                       "on tcgen05; FP64: u12_reg_kernel + gemm_simt_kernel<double>)",
    "tri_solve": "trsv_pub_async_kernel (FP32 inverse-block triangular solve, tiles staged in "
                 "shared memory by cp.async, link blocks, helper CTAs for long block rows)",
    "residual": "residual_partial_kernel + residual_final_kernel (FP64 b - A x)",
}


def kernel_breakdown(h, steps: int, ms_step: float) -> dict:
    """Per kernel class: spans, event time, share of the step and achieved
    bandwidth / flop rate over the breakdown pass (CUDA events recorded by
    the library on its streams around every span; ms_step is that pass's
    own time per step)."""
    out = {}
    for cls in ("panel", "trailing_update", "tri_solve", "residual"):
        t = h.timing(cls)
        if t["spans"] == 0 or t["total_ms"] <= 0:
            continue
        sec = t["total_ms"] * 1e-3
        out[cls] = {"spans_per_step": t["spans"] / steps,
                    "ms_per_step": round(t["total_ms"] / steps, 3),
                    "share_of_step": round(t["total_ms"] / steps / ms_step, 4),
                    "ms_per_span": round(t["total_ms"] / t["spans"], 4),
                    "alg_bytes_per_span": t["bytes"] / t["spans"],
                    "alg_flops_per_span": t["flops"] / t["spans"],
                    "achieved_gbs": round(t["bytes"] / sec / 1e9, 2),
                    "achieved_tflops": round(t["flops"] / sec / 1e12, 4)}
    return out


def dominant_roofline(kernels: dict, mixed: bool) -> dict | None:
    """Roofline of the kernel class with the largest share of the step.

    The FP32 factorisation's classes and the FP64 residual are bounded by
    HBM bandwidth (arithmetic intensity below the ridge; the panel is in
    practice latency-bound and its fraction shows it).  The FP64 trailing
    update is bounded by the FP64 DFMA rate."""
    if not kernels:
        return None
    cls = max(kernels, key=lambda k: kernels[k]["ms_per_step"])
    k = kernels[cls]
    pk = peaks()
    if cls == "trailing_update" and not mixed:
        ach, peak = k["achieved_tflops"], FP64_PEAK["tflops"]
        out = {"bound": "fp64", "unit": "TFLOP/s", "peak_source": FP64_PEAK.get("source")}
        per = k["alg_flops_per_span"]
    else:
        ach, peak = k["achieved_gbs"], float(pk["hbm_gbs"])
        out = {"bound": "hbm", "unit": "GB/s",
               "peak_source": f"{pk['_source']} HBM copy bandwidth (hbm_gbs)"}
        per = k["alg_bytes_per_span"]
    ratio = NCU_TRAFFIC_PER_ALG_BYTE.get(cls)
    out.update({"kernel": KERNEL_NAMES[cls], "class": cls, "achieved": ach, "peak": peak,
                "frac": round(ach / peak, 4) if peak else None,
                "traffic": (k["alg_bytes_per_span"] * ratio) if ratio else None,
                "alg_per_launch": per, "ms_per_launch": k["ms_per_span"],
                "share_of_step": k["share_of_step"]})
    if cls == "panel":
        # a panel launch is a chain of nb pivot decisions (FP32 register
        # panel 64 columns wide, FP64 32), each a cluster-wide argmax and a
        # pivot-row exchange: latency, not bandwidth or tensor throughput
        cols = 64 if mixed else 32
        out["limiter"] = (f"latency: {cols} sequential pivot decisions per launch, "
                          f"{k['ms_per_span'] * 1e3 / cols:.2f} us each")
    return out


def e2e_host(args, Acm, B, n, nrhs, mixed=False) -> dict:
    import ctypes as C

    import torch

    from tmv_gb300 import linalg

    hA = torch.empty((n, n), dtype=torch.float64, pin_memory=True)
    hA.copy_(Acm.t())  # row-major storage of A^T == column-major storage of A
    hB = torch.empty((n, nrhs), dtype=torch.float64, pin_memory=True)
    hB.copy_(B)
    hX = torch.empty((nrhs, n), dtype=torch.float64, pin_memory=True)
    h = linalg.handle(Acm.device.index)
    from tmv_gb300 import _lib

    info = _lib.IRInfo()

    def call():
        if mixed:
            h.check(h.call("tmvg_lu_solve_mixed_f64_host", n, C.c_void_p(hA.data_ptr()), nrhs,
                           C.c_void_p(hB.data_ptr()), C.c_void_p(hX.data_ptr()), 10, 1e-12,
                           C.byref(info)))
        else:
            h.check(h.call("tmvg_divide_f64_host", n, C.c_void_p(hA.data_ptr()), nrhs,
                           C.c_void_p(hB.data_ptr()), C.c_void_p(hX.data_ptr()), None, None))
    call()
    steps = max(3, min(args.steps, 7))
    per_call = []
    t0 = time.perf_counter()
    for _ in range(steps):
        t1 = time.perf_counter()
        call()  # synchronous: returns after X is back in host memory
        per_call.append((time.perf_counter() - t1) * 1e3)
    # the median call: one synchronous call is one step, and a host-side
    # stall in one call (seen as a single 4x outlier) says nothing of the path
    dt = float(np.median(per_call)) * 1e-3
    return {"value": round(lu_solve_flops(n, nrhs) / dt / 1e12, 4), "unit": "TFLOP/s",
            "h2d_bytes_per_step": 8 * n * n + 8 * n * nrhs, "d2h_bytes_per_step": 8 * n * nrhs,
            "ms_per_step": round(dt * 1e3, 3), "steps": steps, "statistic": "median call",
            "ms_mean": round((time.perf_counter() - t0) / steps * 1e3, 3),
            "ms_per_call": [round(t, 3) for t in per_call]}


def other_workloads(dev, with_cpu: bool) -> dict:
    """The other measured workloads, each timed with CUDA events over device-
    resident inputs (seeded synthetic data with the shapes and distributions
    of the workloads): FP64 product C = A*B at M=N=K=1024 (A, B ~ U[-1,1]);
    FP64 LU factor + solve at n = 4096 (A ~ N(0,1) + 4 sqrt(n) I, 8 right-hand
    sides); the solve adjoint at n = 2048 (64 right-hand sides): forward
    X = A^-1 B, backward gB = A^-T G and gA = -gB X^T."""
    import torch

    from tmv_gb300 import adjoint, linalg

    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MiB > L2

    def ev_time(fn, reps=5, warm=3):
        for _ in range(warm):
            fn()
        best = float("inf")
        for i in range(reps):
            flush.fill_(float(i))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        return best

    out = {}
    g = torch.Generator(device=dev)
    g.manual_seed(1)
    m = 1024
    A = (torch.rand((m, m), dtype=torch.float64, device=dev, generator=g) * 2 - 1).t()
    Bm = (torch.rand((m, m), dtype=torch.float64, device=dev, generator=g) * 2 - 1).t()
    C = torch.empty((m, m), dtype=torch.float64, device=dev).t()
    ms = ev_time(lambda: linalg.multmm(False, 1.0, A, Bm, C))
    tf = 2.0 * m ** 3 / (ms * 1e-3) / 1e12
    out["fp64_gemm_1024"] = {"value": round(tf, 4), "unit": "TFLOP/s", "ms": round(ms, 4),
                             "roofline": fp64_roofline(tf),
                             "kernel": "gemm_simt_kernel<double> (MultMM, column-major operands)",
                             "flush": "256 MiB written between runs"}
    if with_cpu:
        orc, kind, what = cpu_reference()
        orc.set_threads(os.cpu_count() or 1)
        Ah, Bh = np.asfortranarray(A.cpu().numpy()), np.asfortranarray(Bm.cpu().numpy())
        Ch = np.zeros((m, m), order="F")
        t0 = time.perf_counter()
        orc.multmm(False, 1.0, Ah, Bh, Ch)
        dt = time.perf_counter() - t0
        out["fp64_gemm_1024"]["cpu_baseline"] = {
            "value": round(2.0 * m ** 3 / dt / 1e12, 5), "unit": "TFLOP/s", "cores": os.cpu_count() or 1,
            "kind": kind, "sample": f"one 1024^3 MultMM (OpenMP block product, {dt:.2f} s); {what}"}
    n = 4096
    A4 = torch.randn((n, n), dtype=torch.float64, device=dev, generator=g)
    A4 += 4.0 * np.sqrt(n) * torch.eye(n, dtype=torch.float64, device=dev)
    A4 = linalg.colmajor(A4)
    B4 = linalg.colmajor(torch.randn((n, 8), dtype=torch.float64, device=dev, generator=g))
    ms = ev_time(lambda: linalg.divide(A4, B4), reps=3, warm=1)
    fl = lu_solve_flops(n, 8)
    tf = fl / (ms * 1e-3) / 1e12
    out["fp64_lu_solve_4096"] = {"value": round(tf, 4), "unit": "TFLOP/s", "ms": round(ms, 3),
                                 "roofline": fp64_roofline(tf),
                                 "workload": "X = B/A, n = 4096, 8 right-hand sides, A ~ N(0,1) + 4 sqrt(n) I"}
    n = 2048
    A5 = torch.randn((n, n), dtype=torch.float64, device=dev, generator=g)
    A5 += 3.0 * np.sqrt(n) * torch.eye(n, dtype=torch.float64, device=dev)
    A5 = linalg.colmajor(A5)
    B5 = linalg.colmajor(torch.randn((n, 64), dtype=torch.float64, device=dev, generator=g))
    G5 = linalg.colmajor(torch.randn((n, 64), dtype=torch.float64, device=dev, generator=g))
    X5, LU5, P5 = adjoint.solve_fwd(A5, B5)
    fwd_ms = ev_time(lambda: adjoint.solve_fwd(A5, B5), reps=3, warm=1)
    bwd_ms = ev_time(lambda: adjoint.solve_bwd(LU5, P5, X5, G5), reps=3, warm=1)
    out["adjoint_2048x64"] = {
        "forward_ms": round(fwd_ms, 3), "backward_ms": round(bwd_ms, 3),
        "forward_tflops": round(lu_solve_flops(n, 64) / (fwd_ms * 1e-3) / 1e12, 4),
        "backward_tflops": round(4.0 * n * n * 64 / (bwd_ms * 1e-3) / 1e12, 4),
        "forward_roofline": fp64_roofline(lu_solve_flops(n, 64) / (fwd_ms * 1e-3) / 1e12),
        "backward_roofline": fp64_roofline(4.0 * n * n * 64 / (bwd_ms * 1e-3) / 1e12),
        "workload": "X = A^-1 B (n = 2048, 64 right-hand sides), backward gB = A^-T G and gA = -gB X^T "
                    "from the stored factors"}
    del flush
    out["complex_lu_solve_4096"] = complex_workload(dev, with_cpu)
    out["band_lu_65536x1024"] = band_workloads(dev, with_cpu)
    return out


def complex_workload(dev, with_cpu: bool) -> dict:
    """complex<double> X = B/A at n = 4096 with 8 right-hand sides (A, B with
    N(0,1) real and imaginary parts, 4 sqrt(n) added to A's diagonal, seeded),
    timed with CUDA events (best of three after one warm-up), the two device
    copies of A and B inside each timed call."""
    import torch

    from tmv_gb300 import linalg

    stream = torch.cuda.current_stream(dev)

    def ev_time(fn, reps=3, warm=1):
        for _ in range(warm):
            fn()
        best = float("inf")
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        return best

    g = torch.Generator(device=dev)
    g.manual_seed(7)
    # complex<double> LU + solve at n = 4096 (8 right-hand sides): A, B with
    # N(0,1) real and imaginary parts, 4 sqrt(n) added to the diagonal
    n = 4096
    Az = torch.complex(torch.randn((n, n), dtype=torch.float64, device=dev, generator=g),
                       torch.randn((n, n), dtype=torch.float64, device=dev, generator=g))
    Az += 4.0 * np.sqrt(n) * torch.eye(n, dtype=torch.complex128, device=dev)
    Az = Az.t().contiguous().t()
    Bz = torch.complex(torch.randn((n, 8), dtype=torch.float64, device=dev, generator=g),
                       torch.randn((n, 8), dtype=torch.float64, device=dev, generator=g)).t().contiguous().t()
    LUz, Xz = torch.empty_like(Az), torch.empty_like(Bz)

    def zsolve():
        LUz.copy_(Az)
        Xz.copy_(Bz)
        Pz = linalg.lu_decompose_z(LUz)
        linalg.lu_ldiveq_z(LUz, Pz, Xz)

    ms = ev_time(zsolve, reps=3, warm=1)
    zfl = 8.0 * n ** 3 / 3.0 + 8.0 * n * n * 8  # real flops: 4 real FMAs per complex FMA
    tf = zfl / (ms * 1e-3) / 1e12
    res = (Az @ Xz - Bz).abs().max().item() / (Az.abs().sum(dim=1).max().item() * Xz.abs().max().item())
    out = {
        "value": round(tf, 4), "unit": "TFLOP/s", "ms": round(ms, 3), "roofline": fp64_roofline(tf),
        "normwise_backward_error": res,
        "workload": "complex<double> X = B/A, n = 4096, 8 right-hand sides, A ~ CN(0,1) + 4 sqrt(n) I; "
                    "flops 8n^3/3 + 8 n^2 nrhs (timed region includes the two device copies of A and B)"}
    if with_cpu:
        orc, kind, what = cpu_reference()
        nc = 2048
        ah = (Az[:nc, :nc]).cpu().numpy().copy(order="F")
        t0 = time.perf_counter()
        orc.lu_decompose_z(ah)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {
            "value": round(8.0 * nc ** 3 / 3.0 / dt / 1e12, 5), "unit": "TFLOP/s", "cores": 1, "kind": kind,
            "sample": f"one complex LU_Decompose at n = {nc} ({dt:.2f} s, one core); {what}"}
    del Az, Bz, LUz, Xz
    return out


def band_workloads(dev, with_cpu: bool, count: int = 65536) -> dict:
    """The batched band LU (x = b / A per system, TMV's LU_Decompose and
    LU_LDivEq on band storage, one thread per system): 65536 systems of
    n = 1024 with one right-hand side, entries N(0,1) with lo + hi + 2 added to
    the diagonal, seeded; tridiagonal (lo = hi = 1, TMV's tridiagonal
    algorithm) and pentadiagonal (lo = hi = 2, the general algorithm).  The
    factorisation is in place, so every timed launch gets a fresh copy of the
    inputs (copied before its events); the band and right-hand sides (2.1 and
    3.8 GB) exceed L2.  Rooflines: the FP64 pipe, counting one pipe slot per
    product, difference and reciprocal (division) -- half the DFMA TFLOP/s
    rate in operations -- and HBM for the bytes read and written once."""
    import torch

    from tmv_gb300.band import band_divide, band_layout, band_lu_rdiveq, band_lu_solve, band_lu_solve_count

    def timed(fn, reset) -> float:
        ts = []
        for rep in range(6):
            reset()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            if rep >= 2:
                ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))

    n = 1024
    stream = torch.cuda.current_stream(dev)
    hbm = peaks()["hbm_gbs"]
    out = {}
    for lo, hi, algo in [(1, 1, "tridiag"), (2, 2, "general")]:
        lay = band_layout(n, lo, hi)
        g = torch.Generator(device=dev).manual_seed(11)
        ab0 = torch.randn(count * lay.stride_ab, dtype=torch.float64, device=dev, generator=g)
        i = torch.arange(n, device=dev)
        ab0.view(count, lay.stride_ab)[:, i * (lay.ldab + 1)] += lo + hi + 2.0
        b0 = torch.randn(count * n, dtype=torch.float64, device=dev, generator=g)
        ab, X = torch.empty_like(ab0), torch.empty_like(b0)
        P = torch.empty(count * n, dtype=torch.int64, device=dev)
        st = torch.empty(count, dtype=torch.int32, device=dev)
        times = []
        for rep in range(6):
            ab.copy_(ab0)
            X.copy_(b0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            band_lu_solve(ab, count, lay, X, 1, algo=algo, P=P, status=st)
            e1.record(stream)
            torch.cuda.synchronize()
            if rep >= 2:
                times.append(e0.elapsed_time(e1))
        ms = float(np.median(times))
        assert int(st.abs().sum().item()) == 0
        work = band_lu_solve_count(count, lay, 1)
        ops = work["flops"] / (ms * 1e-3) / 1e12  # T operations / s
        pipe = FP64_PEAK["tflops"] / 2 if FP64_PEAK["tflops"] else None
        gbs = work["bytes"] / (ms * 1e-3) / 1e9
        key = f"{'tridiag' if algo == 'tridiag' else 'general'}_lo{lo}_hi{hi}"
        out[key] = {
            "value": round(count / (ms * 1e-3), 1), "unit": "systems/s", "ms": round(ms, 4),
            "kernel": f"band_lu_kernel<{lo},{2 * lo},{'true' if algo == 'tridiag' else 'false'}>",
            "fp64_ops_per_launch": work["flops"], "bytes_per_launch": work["bytes"],
            "roofline_fp64_pipe": {"bound": "fp64", "achieved": round(ops, 4), "unit": "Top/s",
                                   "peak": round(pipe, 4) if pipe else None,
                                   "frac": round(ops / pipe, 4) if pipe else None,
                                   "peak_source": "DFMA rate / 2 (one pipe slot per op)"},
            "roofline_hbm": {"bound": "hbm", "achieved": round(gbs, 1), "peak": hbm, "unit": "GB/s",
                             "frac": round(gbs / hbm, 4)},
            "workload": f"{count} systems, n = {n}, lo = {lo}, hi = {hi}, 1 right-hand side, "
                        f"algorithm {algo}"}
        # x A = b from the same factors (LU_RDivEq), one row per system
        X2 = torch.empty_like(b0)
        ms_r = timed(lambda: band_lu_rdiveq(ab, count, lay, P, X2, 1, algo=algo, status=st),
                     lambda: X2.copy_(b0))
        assert int(st.abs().sum().item()) == 0
        out[key]["rdiveq"] = {"value": round(count / (ms_r * 1e-3), 1), "unit": "systems/s",
                              "ms": round(ms_r, 4),
                              "what": "x A = b per system from the factors above (LU_RDivEq)"}
        if with_cpu:
            orc, kind, what = cpu_reference()
            cores = os.cpu_count() or 1
            orc.set_threads(cores)
            sample = count  # the whole batch: about a second on 16 cores
            hab = ab0[:sample * lay.stride_ab].cpu().numpy().copy()
            hb = b0[:sample * n].cpu().numpy().copy()
            t0 = time.perf_counter()
            Ph, sth = orc.band_batched_solve(sample, n, lo, hi, 1 if algo == "tridiag" else 0, hab,
                                             lay.ldab, lay.stride_ab, 1, hb, n, n)
            dt = time.perf_counter() - t0
            gx = X[:sample * n].cpu().numpy()
            ok = bool(np.array_equal(hb.view(np.int64), gx.view(np.int64)))
            # normwise per system: max_s ||x_cpu - x_gpu||_inf / ||x_gpu||_inf
            dv = np.abs(hb - gx).reshape(sample, n).max(axis=1)
            diff = float(np.max(dv / np.maximum(np.abs(gx).reshape(sample, n).max(axis=1), 1e-300)))
            out[key]["cpu_baseline"] = {
                "value": round(sample / dt, 1), "unit": "systems/s", "cores": cores, "kind": kind,
                "sample": f"all {sample} systems ({dt:.2f} s, OpenMP over systems); {what}",
                "solutions_vs_gpu": {
                    "bitwise_equal": ok, "max_normwise_rel_diff": diff,
                    "note": "the GPU rounds every product and difference separately, as TMV's "
                            "source reads and as its x86-64 build runs it (bit for bit in the "
                            "tests); g++ -O2 on aarch64 contracts a - b*c into fused "
                            "multiply-adds by default, so TMV built there differs by rounding"}}
        del ab0, b0, ab, X, P, st
    lo, hi = 2, 1
    lay = band_layout(n, lo, hi)
    g = torch.Generator(device=dev).manual_seed(12)
    ab0 = torch.randn(count * lay.stride_ab, dtype=torch.float64, device=dev, generator=g)
    i = torch.arange(n, device=dev)
    ab0.view(count, lay.stride_ab)[:, i * (lay.ldab + 1)] += lo + hi + 2.0
    b0 = torch.randn(count * n, dtype=torch.float64, device=dev, generator=g)
    X = torch.empty_like(b0)
    lay_lu = band_layout(n, min(lo, hi), lo)
    lu = torch.empty(count * lay_lu.stride_ab, dtype=torch.float64, device=dev)
    P = torch.empty(count * n, dtype=torch.int64, device=dev)
    st = torch.empty(count, dtype=torch.int32, device=dev)
    ms_d = timed(lambda: band_divide(ab0, count, lay, X, 1, lu=lu, P=P, status=st), lambda: X.copy_(b0))
    assert int(st.abs().sum().item()) == 0
    out["divide_lo2_hi1"] = {
        "value": round(count / (ms_d * 1e-3), 1), "unit": "systems/s", "ms": round(ms_d, 4),
        "workload": f"{count} systems, n = {n}, lo = 2, hi = 1, 1 right-hand side: B /= A as "
                    "BandLUDiv runs it (A^T copied and factored, then LU_RDivEq), A not modified"}
    return out


def cpu_reference():
    """The CPU implementation timed beside the GPU: TMV 0.76 itself where its
    library was compiled on this machine (oracle/_ref, built from TMV's
    sources by the build step: NOBLAS/NOLAP, OpenMP MultMM), else the
    oracle's C restatement of the same algorithm.  Returns (backend, kind,
    description)."""
    import oracle

    if oracle.ref_available():
        return (oracle.ref(), "reference",
                "TMV 0.76 compiled from its sources on this machine (NOBLAS/NOLAP, OpenMP MultMM)")
    return oracle.port(), "port", "the oracle's C restatement of TMV's algorithm"


def cpu_baseline(A: np.ndarray, B: np.ndarray, n: int, cond: float) -> dict:
    """TMV's FP64 LU + solve (m.divideUsing(tmv::LU); X = B/m) on the host
    cores: one solve of the same workload (same A and b)."""
    orc, kind, what = cpu_reference()
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    t0 = time.perf_counter()
    X, LU, P = orc.divide(A, B)
    dt = time.perf_counter() - t0
    return {"value": round(lu_solve_flops(n, 1) / dt / 1e12, 5), "unit": "TFLOP/s",
            "cores": cores, "kind": kind,
            "sample": f"one FP64 LU factor + solve at n={n}, cond={cond:g} ({dt:.1f} s); {what}"}


def run_reference(args) -> dict | None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    orc, kind, what = cpu_reference()
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    n = args.n
    A, b = haar_matrix_numpy(n, args.cond, seed=3)
    B = b.reshape(n, 1)
    for _ in range(min(args.warmup, 1)):
        orc.divide(A, B)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        orc.divide(A, B)
    dt = (time.perf_counter() - t0) / args.steps
    v = lu_solve_flops(n, 1) / dt / 1e12
    return {"metric": METRIC, "value": round(v, 5), "unit": "TFLOP/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": f"dense LU solve n={n}, 1 RHS, cond={args.cond:g}",
                       "n": n, "nrhs": 1, "cond": args.cond},
            "cpu_baseline": {"value": round(v, 5), "unit": "TFLOP/s", "cores": cores,
                             "kind": kind,
                             "sample": f"{args.steps} FP64 LU solves at n={n} ({what}; "
                                       "warm-up capped at 1)"},
            "e2e": {"value": round(v, 5), "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=8192)
    ap.add_argument("--cond", type=float, default=1e6)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--path", default="mixed", choices=["mixed", "fp64", "batched", "band", "complex"],
                    help="mixed: the headline solve; fp64: the FP64 LU solve alone; batched: "
                         "only the batched uneven solver; band: only the batched band LU "
                         "workloads; complex: only the complex<double> LU solve (the last "
                         "three for profiling them)")
    ap.add_argument("--matrix-cache", default=None,
                    help="load the workload matrix from this file if present, else save it "
                         "there (lets a profiler run skip the QR-based generation)")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-sweep", action="store_true",
                    help="skip the condition-number / equal-accuracy sweep")
    ap.add_argument("--batch-count", type=int, default=20000)
    ap.add_argument("--band-count", type=int, default=65536,
                    help="systems of the band workload with --path band (smaller for a profiler)")
    ap.add_argument("--batch-cpu-sample", type=int, default=20000)
    ap.add_argument("--no-extras", action="store_true",
                    help="time the step only (no FP64 comparison, e2e, roofline or CPU leg)")
    args = ap.parse_args()
    if args.impl == "reference":
        out = run_reference(args)
    else:
        out = run_gpu(args)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
