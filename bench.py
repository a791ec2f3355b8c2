#!/usr/bin/env python
"""Benchmark of the SHLL Euler hot path on one GB300 (or N replicas under torchrun).

Metric: cell-updates/s of the FP32-flux / FP64-accumulate solver (SHLL_PREC_MIXED_F64), next to
the plain FP64 one-launch-per-step path, with the L1 error against the FP64 path and the
fraction of the HBM roofline (48 algorithmic bytes per 1D cell-update: 3 FP64 conserved values
read and written once).

Default workload (one "step" of this benchmark = one full run of it): 1D Sod shock tube,
second-order SHLL as the x sweep of base-c/2nd_order_base_shll.c, 65536 cells on [0,1],
diaphragm at 0.5, rho 10/1, T 1/1, gas at rest, gamma 1.4, R 1, CFL 0.25, to t = 0.2
(104858 time steps); synthetic initial data generated on the host.

--impl reference times the reference's CPU implementation of the same path on the host cores
(the bit-exact CPU port of base-c in its published FP32 arithmetic: the reference's own sources
are not present on the GPU host), on a bounded sample of the same tube.
"""
import argparse
import importlib.util
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "shll-sve-cfd_gb300")
PROFILES = os.path.join(ROOT, "profiles")


def load_pkg():
    name = "shll_gb300"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, os.path.join(PKG, "shll_gb300.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.stop = threading.Event()
        self.t = threading.Thread(target=self._run, daemon=True)

    def _run(self):
        while not self.stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                vals = [v.strip() for v in out.stdout.strip().split(",")]
                if len(vals) >= 7:
                    self.samples.append(vals)
            except Exception:
                pass
            self.stop.wait(0.2)

    def __enter__(self):
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop.set()
        self.t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def profile_traffic(kernel):
    """Per-launch DRAM bytes of `kernel` recorded in profiles/*.md ('traffic_bytes_per_launch:')."""
    try:
        for fn in sorted(os.listdir(PROFILES)):
            if not fn.endswith(".md"):
                continue
            txt = open(os.path.join(PROFILES, fn)).read()
            if f"kernel: {kernel}" in txt:
                for line in txt.splitlines():
                    if line.startswith("traffic_bytes_per_launch:"):
                        return float(line.split(":")[1])
    except Exception:
        pass
    return None


def sod_params(shll, n, order, precision, **kw):
    return shll.params(1, order, nx=n, precision=precision, t_end=0.2, **kw)


def cpu_sample(n, order, steps, bits):
    """Times the CPU port of the reference (bit-exact FP32/FP64 port of base-c) on a sample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.lib()
    cfg = O.make_cfg(order=order, nx=n, real_bits=bits, n_steps=steps)
    prim = O.ic_sod(n)
    t0 = time.perf_counter()
    O.run(cfg, prim)
    dt = time.perf_counter() - t0
    return n * steps / dt, dt


def l2_flush(torch, buf):
    buf.add_(1.0)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cells", type=int, default=65536)
    ap.add_argument("--order", type=int, default=2)
    ap.add_argument("--fold", type=int, default=0, help="fold interval of the mixed path (0 = library default)")
    ap.add_argument("--precision", default="mixed_f64")
    ap.add_argument("--no-extras", action="store_true", help="skip the FP64 comparison runs and CPU baseline")
    args = ap.parse_args()
    W = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    n, order = args.cells, args.order
    steps_per_run = None
    workload = (f"1D Sod shock tube, {'second' if order == 2 else 'first'}-order SHLL, {n} cells, "
                f"rho 10/1, T 1/1, t=0.2")

    if args.impl == "reference":
        if rank != 0:
            return
        # each step: a bounded sample of the same tube (all its cells, a slice of its time steps)
        sample_steps = max(50, int(3.0e8 / n))
        vals = []
        for i in range(W + args.steps):
            v, dt = cpu_sample(n, order, sample_steps, 32)
            if i >= W:
                vals.append((v, dt))
        value = sum(v for v, _ in vals) / len(vals)
        ms = 1000 * sum(dt for _, dt in vals) / len(vals)
        sample = f"{n} cells x {sample_steps} of the run's time steps per step, FP32 as published, 1 thread"
        print(json.dumps({
            "impl": "reference", "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": W, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": workload, "cells": n, "order": order},
            "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": 1, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }))
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    shll = load_pkg()
    stream = torch.cuda.Stream()
    p = sod_params(shll, n, order, args.precision, fold_steps=args.fold)
    steps_per_run = shll.steps_for(p)
    cu_per_run = steps_per_run * n
    ctx = shll.Context(p)
    ctx.set_stream(stream.cuda_stream)
    ctx.init_state()
    ctx.checkpoint()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2
    for _ in range(W):
        ctx.restore()
        ctx.run()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    l0 = shll.kernel_launches()
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                l2_flush(torch, flush)
            ctx.restore()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.run()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1000.0)
    torch.cuda.synchronize()
    launches = shll.kernel_launches() - l0
    t_total = sum(times)
    if dist:
        t = torch.tensor([t_total], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_total = float(t.item())
        dist.barrier()
    value = world * cu_per_run * args.steps / t_total
    ms_per_step = 1000 * t_total / args.steps
    mixed_out = ctx.primitives()

    # roofline of the dominant kernel (the sweep kernel: fold_steps time steps per launch)
    fold = args.fold if args.fold > 0 else 16
    fold = min(fold, 32)
    sweeps = math.ceil(steps_per_run / fold)
    bytes_per_launch = 48.0 * n * fold
    avg_launch = t_total / (args.steps * sweeps)  # upper bound: includes launch gaps
    hbm, peak_kind = peaks()
    achieved = bytes_per_launch / avg_launch / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "traffic": profile_traffic("k_sweep1d"), "peak_kind": peak_kind,
                "kernel": "k_sweep1d", "algorithmic_bytes_per_launch": bytes_per_launch,
                "launch_duration_s": avg_launch}

    # end to end through the C-ABI with host buffers: upload primitives, run, download
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    x = np.arange(n)
    rho = np.where(x < 0.5 * n, 10.0, 1.0)
    u = np.zeros(n)
    T = np.ones(n)
    pe = sod_params(shll, n, order, args.precision, fold_steps=args.fold, ic_kind=shll.IC_USER)
    ectx = shll.Context(pe)
    ectx.set_primitives(rho, u, T)
    ectx.run()  # warm
    torch.cuda.synchronize()
    e_times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        ectx.set_primitives(rho, u, T)
        ectx.run()
        out = ectx.primitives()
        e_times.append(time.perf_counter() - t0)
    e2e_value = world * cu_per_run * args.steps / sum(e_times)
    ectx.close()

    extras = {}
    if not args.no_extras and rank == 0:
        # plain FP64 path, one launch per step (bit-exact to the FP64 reference): throughput + L1
        pf = sod_params(shll, n, order, "f64_exact")
        fctx = shll.Context(pf)
        fctx.set_stream(stream.cuda_stream)
        fctx.init_state()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fctx.run()
        e1.record(stream)
        e1.synchronize()
        t64 = e0.elapsed_time(e1) / 1000.0
        f64_out = fctx.primitives()
        fctx.close()
        l1 = np.mean(np.abs(mixed_out - f64_out), axis=1)
        import oracle as O
        O.lib()
        ex = O.riemann_exact(n, steps_per_run * (0.125 / n))
        extras = {
            "fp64_plain": {"value": cu_per_run / t64, "unit": "cell-updates/s", "schedule": "one launch per step",
                           "precision": "f64_exact"},
            "speedup_vs_fp64_plain": (cu_per_run / (t_total / args.steps)) / (cu_per_run / t64),
            "l1_vs_fp64": {"rho": l1[0], "u": l1[1], "T": l1[2]},
            "l1_rho_vs_exact_riemann": {"mixed": float(np.mean(np.abs(mixed_out[0] - ex[0]))),
                                        "fp64": float(np.mean(np.abs(f64_out[0] - ex[0])))},
        }
        cpu_v, cpu_dt = cpu_sample(n, order, max(50, int(3.0e8 / n)), 32)
        extras["cpu_baseline"] = {"value": cpu_v, "unit": "cell-updates/s", "cores": 1, "kind": "port",
                                  "sample": f"{n} cells x {max(50, int(3.0e8 / n))} time steps, FP32 as "
                                            f"published, {cpu_dt:.1f} s"}
    if rank == 0:
        line = {
            "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": W, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32-flux+f64-acc", "data": "synthetic",
            "config": {"workload": workload, "cells": n, "order": order, "time_steps_per_run": steps_per_run,
                       "precision": args.precision, "fold_steps": fold, "parallelism": f"replicas{world}",
                       "l2": "flushed between runs (256 MB write)"},
            "roofline": roofline,
            "e2e": {"value": e2e_value, "unit": "cell-updates/s", "h2d_bytes_per_step": 3 * n * 8,
                    "d2h_bytes_per_step": 3 * n * 8},
            "gpu_launches": launches,
            "clocks": clk.summary(),
        }
        line.update(extras)
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
