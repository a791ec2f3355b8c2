#!/usr/bin/env python
"""Benchmark of the SHLL Euler hot path on one GB300 (or N independent replicas under torchrun).

Metric: cell-updates/s of the FP32-flux / FP64-accumulate solver (SHLL_PREC_MIXED_F64), next to
the plain FP64 path (one launch per time step), with the L1 error against FP64 and the fraction of
the HBM roofline (algorithmic bytes per cell-update: 48 in 1D = 3 FP64 conserved values read and
written once, 64 in 2D).

Workloads (all inputs are seeded synthetic initial data generated on the host; gamma 1.4, R 1,
kinetic CFL 0.25):
  sod1d    (default) 1D Sod tube, second-order SHLL (the x sweep of base-c/2nd_order_base_shll.c),
           65536 cells, diaphragm 0.5, rho 10/1, T 1/1, at rest, to t = 0.2 (104858 steps).
  circle2d 2D first-order SHLL (base-c/base_shll_2d.c), 4096 x 4096, circular diaphragm r = 0.25
           at (0.5, 0.5), rho 10 inside / 1 outside, T 1, at rest, 500 steps.
  batch1d  4096 tubes, seed 0: cells log-uniform in [256, 16384], density ratio U(2,100), temperature
           ratio U(0.5,2), diaphragm U(0.3,0.7); first order for the first 2048, second order after;
           each to t = 0.2.
  batch2d  256 first-order domains, seed 1: side uniform in {128, 256, 512, 1024}, radius U(0.1,0.35),
           density ratio U(2,50), temperature ratio U(0.5,2), at rest, 400 steps each.
One benchmark "step" is one full run of the workload.

--impl reference times the reference's CPU implementation of the path on the host cores (the
bit-exact CPU port of base-c in its published FP32 arithmetic, test infrastructure of this
repository: the reference's own sources are not present on the GPU host), on a bounded sample.
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


def oracle_mod():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.lib()
    return O


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

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [v for v in (num(s[0]) for s in self.samples) if v is not None]
        mx = [v for v in (num(s[1]) for s in self.samples) if v is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def profile_traffic(kernel, workload):
    """Per-launch DRAM bytes of `kernel` on `workload` from profiles/*.md
    ('kernel: <name>', 'workload: <name>', 'traffic_bytes_per_launch: <bytes>')."""
    try:
        for fn in sorted(os.listdir(PROFILES)):
            if not fn.endswith(".md"):
                continue
            txt = open(os.path.join(PROFILES, fn)).read()
            if f"kernel: {kernel}\n" in txt and f"workload: {workload}\n" in txt:
                for line in txt.splitlines():
                    if line.startswith("traffic_bytes_per_launch:"):
                        return float(line.split(":")[1])
    except Exception:
        pass
    return None


# ---------------------------------------------------------------------------------------------
# workloads


def items_batch1d(shll, precision, count=4096, seed=0, fold=0):
    rng = np.random.default_rng(seed)
    out = []
    for t in range(count):
        n = int(round(math.exp(rng.uniform(math.log(256), math.log(16384)))))
        ratio = float(rng.uniform(2, 100))
        tr = float(rng.uniform(0.5, 2))
        xd = float(rng.uniform(0.3, 0.7))
        order = 1 if t < count // 2 else 2
        out.append(shll.params(1, order, nx=n, precision=precision, t_end=0.2, fold_steps=fold, ic_x_d=xd,
                               ic_rho_l=ratio, ic_T_l=tr, ic_rho_r=1.0, ic_T_r=1.0, ic_u_l=0.0, ic_u_r=0.0))
    return out


def items_batch2d(shll, precision, count=256, seed=1, fold=0):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.choice([128, 256, 512, 1024]))
        r = float(rng.uniform(0.1, 0.35))
        ratio = float(rng.uniform(2, 50))
        tr = float(rng.uniform(0.5, 2))
        out.append(shll.params(2, 1, nx=n, ny=n, precision=precision, n_steps=400, fold_steps=fold,
                               ic_kind=shll.IC_CIRCLE2D, ic_cx=0.5, ic_cy=0.5, ic_radius=r, ic_rho_l=ratio,
                               ic_T_l=tr, ic_rho_r=1.0, ic_T_r=1.0))
    return out


# --run-steps: a fixed step count for the single-domain workloads (short runs of the same kernels,
# for profiling); 0 keeps each workload's own end time or step count
RUN_STEPS = 0


def params_single(shll, workload, precision, cells, order, fold):
    if workload == "omp2d":   # base-omp/2nd_order_base_shll.c:30-44, 147-172 (MC limiter, "Configuration 6")
        p = shll.params(2, 2, nx=cells, ny=cells, precision=precision, t_end=0.3, limiter=1, mc_alpha=1.25,
                        ic_kind=shll.IC_QUADRANTS2D, fold_steps=fold)
    elif workload == "sod1d":
        p = shll.params(1, order, nx=cells, precision=precision, t_end=0.2, fold_steps=fold)
    else:
        p = shll.params(2, 1, nx=cells, ny=cells, precision=precision, n_steps=500, fold_steps=fold,
                        ic_kind=shll.IC_CIRCLE2D, ic_cx=0.5, ic_cy=0.5, ic_radius=0.25, ic_rho_l=10.0,
                        ic_T_l=1.0, ic_rho_r=1.0, ic_T_r=1.0)
    if RUN_STEPS > 0:
        p.n_steps = RUN_STEPS
    return p


def describe(workload, cells, order):
    return {
        "sod1d": f"1D Sod shock tube, {'second' if order == 2 else 'first'}-order SHLL, {cells} cells, rho 10/1, "
                 f"T 1/1, t=0.2",
        "circle2d": f"2D first-order SHLL, {cells}x{cells}, circular diaphragm r=0.25, rho 10/1, T 1, 500 steps",
        "batch1d": "4096 independent 1D tubes (seed 0), 256..16384 cells log-uniform, half first / half second "
                   "order, each to t=0.2",
        "batch2d": "256 independent 2D first-order domains (seed 1), 128^2..1024^2, circular diaphragms, 400 steps",
        "omp2d": f"2D second-order SHLL with the MC limiter (alpha 1.25), {cells}x{cells}, four-quadrant initial data "
                 f"of base-omp, t=0.3",
    }[workload]


class Problem:
    """One workload instance on the GPU: single context or batch, with reset + timed run."""

    def __init__(self, shll, workload, precision, cells, order, fold, stream, tune=True):
        self.shll, self.workload, self.stream = shll, workload, stream
        self.precision, self.tune, self.tuned = precision, tune and not fold, False
        self.batch = workload.startswith("batch")
        self.dim = 2 if workload in ("circle2d", "batch2d", "omp2d") else 1
        if self.batch:
            gen = items_batch1d if workload == "batch1d" else items_batch2d
            self.items = gen(shll, precision, fold=fold)
            self.cu = sum(p.nx * (p.ny if p.dim == 2 else 1) * shll.steps_for(p) for p in self.items)
        else:
            self.p = params_single(shll, workload, precision, cells, order, fold)
            self.cu = self.p.nx * (self.p.ny if self.p.dim == 2 else 1) * shll.steps_for(self.p)
        self.obj = None

    def reset(self):
        """Brings the initial state onto the device (untimed).  Mixed-precision problems are built
        once (and autotuned) and reset by a device-side restore of the initial state, so repeated
        runs replay their captured launch sequence; plain FP64 2D problems are rebuilt."""
        if self.obj is not None and (self.dim == 1 or self.precision.startswith("mixed")):
            self.obj.restore()
            return
        if self.obj is not None:
            self.obj.close()
        if self.batch:
            self.obj = self.shll.Batch(self.items)
        else:
            self.obj = self.shll.Context(self.p)
            self.obj.init_state()
        self.obj.set_stream(self.stream.cuda_stream)
        if self.dim == 1 or self.precision.startswith("mixed"):
            if self.tune and self.precision.startswith("mixed") and not self.tuned:
                self.obj.autotune()   # untimed: 1D sweep length and fold window per size class, 2D fold window
                self.tuned = True
            self.obj.checkpoint()

    def tuning(self):
        """The autotuner's choices: {"sweep steps/fold steps/chunk cells": items}."""
        if not self.precision.startswith("mixed"):
            return None
        if not self.batch:
            return {"%d/%d/%d" % self.obj.tuning(): 1}
        out = {}
        for i in range(len(self.items)):
            key = "%d/%d/%d" % self.obj.tuning(i)
            out[key] = out.get(key, 0) + 1
        return out

    def host_buffers(self, torch):
        """Pinned host memory for the end-to-end leg: every item's initial primitives (its
        descriptor's, as the library loads them) and room for its results."""
        plist = self.items if self.batch else [self.p]
        shapes = [(4 if p.dim == 2 else 3, p.nx * (p.ny if p.dim == 2 else 1)) for p in plist]
        total = sum(nv * n for nv, n in shapes)
        pin_in = torch.empty(total, dtype=torch.float64, pin_memory=True).numpy()
        pin_out = torch.empty(total, dtype=torch.float64, pin_memory=True).numpy()
        ins, outs, off = [], [], 0
        for p, (nv, n) in zip(plist, shapes):
            ins.append(pin_in[off:off + nv * n].reshape(nv, n))
            outs.append(pin_out[off:off + nv * n].reshape(nv, n))
            self.shll.initial_primitives(p, out=ins[-1])
            off += nv * n
        self.pin_in, self.pin_out = pin_in, pin_out   # (batches: the packed layout, item after item)
        return ins, outs

    def upload(self, ins):
        """The initial state from host memory through the public API (copied as given, converted on
        the device)."""
        if self.batch:   # one packed upload for every item
            self.obj.set_all_primitives(self.pin_in)
            return
        b = ins[0]
        args, kw = ((b[0], b[1], b[2]), {}) if self.dim == 1 else ((b[0], b[1], b[3]), {"v": b[2]})
        self.obj.set_primitives(*args, **kw)

    def download(self, outs):
        if self.batch:
            self.obj.get_all_primitives(self.pin_out)
        else:
            self.obj.primitives(out=outs[0])

    def run(self):
        if self.batch:
            self.obj.run(allow_numeric=True)
        else:
            self.obj.run()

    def failed(self):
        """Items whose run reached a non-positive or NaN state (the reference's own scheme breaks down
        on some of the strongest randomly drawn shock tubes)."""
        if not self.batch:
            return []
        return [i for i in range(len(self.items)) if self.obj.item_status(i) != 0]

    def close(self):
        if self.obj is not None:
            self.obj.close()
            self.obj = None

    def result(self):
        if self.batch:
            return [self.obj.primitives(i) for i in range(len(self.items))]
        return self.obj.primitives()


def cpu_sample(n, order, steps, bits):
    """Times the CPU port of the reference (bit-exact to base-c) on all n cells x `steps` steps."""
    O = oracle_mod()
    cfg = O.make_cfg(order=order, nx=n, real_bits=bits, n_steps=steps)
    prim = O.ic_sod(n)
    t0 = time.perf_counter()
    O.run(cfg, prim)
    dt = time.perf_counter() - t0
    return n * steps / dt, dt


def cpu_sample_2d(n, steps, bits):
    O = oracle_mod()
    cfg = O.make_cfg(dim=2, order=1, nx=n, ny=n, real_bits=bits, n_steps=steps)
    prim = O.ic_circle2d(n, n, r=0.25)
    t0 = time.perf_counter()
    O.run(cfg, prim)
    dt = time.perf_counter() - t0
    return n * n * steps / dt, dt


def cpu_batch_sample(workload, budget_cells):
    """Times the CPU port on a sample of the seeded batch with every host thread: items in seed
    order, each for a capped number of steps, until about `budget_cells` cell-updates; one item per
    thread at a time (the oracle's C code runs outside the GIL).  Returns (cell-updates/s, seconds,
    threads, description)."""
    import concurrent.futures
    O = oracle_mod()
    rng = np.random.default_rng(0 if workload == "batch1d" else 1)
    jobs, total = [], 0
    while total < budget_cells:
        if workload == "batch1d":
            n = int(round(math.exp(rng.uniform(math.log(256), math.log(16384)))))
            ratio, tr, xd = float(rng.uniform(2, 100)), float(rng.uniform(0.5, 2)), float(rng.uniform(0.3, 0.7))
            order = 1 if len(jobs) % 2 == 0 else 2
            steps = min(int(math.ceil(1.6 * n)), max(20, int(2e7 / n)))
            jobs.append(("1d", n, order, steps, ratio, tr, xd))
            total += n * steps
        else:
            n = int(rng.choice([128, 256, 512, 1024]))
            r = float(rng.uniform(0.1, 0.35))
            ratio, tr = float(rng.uniform(2, 50)), float(rng.uniform(0.5, 2))
            steps = min(400, max(10, int(1e7 / (n * n))))
            jobs.append(("2d", n, 1, steps, ratio, tr, r))
            total += n * n * steps

    def one(job):
        kind, n, order, steps, a, b, c = job
        if kind == "1d":
            cfg = O.make_cfg(order=order, nx=n, real_bits=32, n_steps=steps)
            prim = O.ic_sod(n, x_d=c, rhoL=a, TL=b)
        else:
            cfg = O.make_cfg(dim=2, order=1, nx=n, ny=n, real_bits=32, n_steps=steps)
            prim = O.ic_circle2d(n, n, r=c, rho_in=a, T_in=b)
        try:
            O.run(cfg, prim)
        except ValueError:
            pass   # a tube that breaks down still did its work
        return (n if kind == "1d" else n * n) * steps

    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    with concurrent.futures.ThreadPoolExecutor(max_workers=threads) as ex:
        done = sum(ex.map(one, jobs))
    dt = time.perf_counter() - t0
    desc = (f"{len(jobs)} items of the seeded batch in seed order, steps capped, {done:.3g} cell-updates, "
            f"FP32 as published, {threads} threads")
    return done / dt, dt, threads, desc


def reference_arm(args, workload, W):
    """CPU reference timing (rank 0 only): the single-domain cases on one thread (base-c is serial;
    base-omp parallelises only its 2D second-order solver), the batches with every host thread."""
    vals = []
    cores = 1
    for i in range(W + args.steps):
        if workload in ("batch1d", "batch2d"):
            v, dt, cores, sample = cpu_batch_sample(workload, 4e9 if workload == "batch1d" else 2e9)
        elif workload == "omp2d":
            v, dt, cores = cpu_sample_omp2d(args.cells, 200)
            sample = f"{args.cells}x{args.cells} cells x 200 time steps per step, FP32 as published, {cores} threads"
        elif workload == "sod1d":
            n = args.cells
            steps = max(50, int(3.0e8 / n))
            v, dt = cpu_sample(n, args.order, steps, 32)
            sample = f"{n} cells x {steps} time steps per step, FP32 as published, 1 thread"
        else:
            n = 512
            steps = max(20, int(2.0e8 / (n * n)))
            v, dt = cpu_sample_2d(n, steps, 32)
            sample = f"{n}x{n} cells x {steps} time steps per step, FP32 as published, 1 thread"
        if i >= W:
            vals.append((v, dt))
    value = sum(v for v, _ in vals) / len(vals)
    ms = 1000 * sum(dt for _, dt in vals) / len(vals)
    return value, ms, sample, cores


def max_over_ranks(x, dist, device):
    """The slowest rank's figure (replicas: the job ends when the last rank ends)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def job_value(world, cell_updates_per_run, runs, seconds):
    """Whole-job cell-updates/s: every rank runs its own replica of the workload (weak scaling)."""
    return world * cell_updates_per_run * runs / seconds


DEFAULT_CELLS = {"sod1d": 65536, "circle2d": 4096, "omp2d": 1024}
# the arithmetic each workload is measured in, where it is not --precision
PRECISION = {}


def measure(shll, torch, stream, workload, cells, order, args, steps, W, dist, world, rank, local, extras,
            precision=None):
    """One workload on this rank's GPU: W untimed runs, then `steps` timed runs (CUDA events on the
    launching stream, L2 flushed before each), the end-to-end leg through the public API with host
    buffers, and (rank 0, extras) the FP64 comparison and the CPU baseline.  Returns the JSON fields."""
    precision = precision or PRECISION.get(workload, args.precision)
    prob = Problem(shll, workload, precision, cells, order, args.fold, stream, tune=not args.no_tune)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2
    for _ in range(W):
        prob.reset()
        prob.run()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches = 0
    times = []
    with ClockSampler(local) as clk:
        for _ in range(steps):
            prob.reset()
            with torch.cuda.stream(stream):
                flush.add_(1.0)
            torch.cuda.synchronize()
            la = shll.kernel_launches()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            prob.run()
            e1.record(stream)
            e1.synchronize()
            launches += shll.kernel_launches() - la
            times.append(e0.elapsed_time(e1) / 1000.0)
    torch.cuda.synchronize()
    t_total = max_over_ranks(sum(times), dist, "cuda")
    value = job_value(world, prob.cu, steps, t_total)
    mixed_out = prob.result()

    # roofline: algorithmic bytes (48 per 1D, 64 per 2D cell-update) of the timed runs over their
    # CUDA-event time, i.e. per launch of the run's kernels over their average launch duration
    hbm, peak_kind = peaks()
    bytes_per_cu = 64.0 if prob.dim == 2 else 48.0
    kernel = {"sod1d": "k_tube1d" if launches <= 3 * steps else "k_sweep1d", "batch1d": "k_sweep1d",
              "circle2d": "k_step2d", "batch2d": "k_step2d",
              "omp2d": "k_step2d_o2" if precision.startswith("mixed") else "k_step2"}[workload]
    achieved = bytes_per_cu * prob.cu * steps / t_total / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "traffic": profile_traffic(kernel, workload), "peak_kind": peak_kind, "kernel": kernel,
                "algorithmic_bytes_per_run": bytes_per_cu * prob.cu, "launches_per_run": launches / steps,
                "launch_duration_s": t_total / max(1, launches),
                "note": "algorithmic bytes of the timed runs / their CUDA-event time (effective: the state is "
                        "read and written once per fold window)"}

    # end to end through the C-ABI with host buffers: every step uploads every item's initial
    # primitives from pinned host memory, runs, and downloads the result primitives
    host_in, host_out = prob.host_buffers(torch)
    e_times = []
    for _ in range(max(1, min(steps, 3))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        prob.upload(host_in)
        prob.run()
        prob.download(host_out)
        torch.cuda.synchronize()
        e_times.append(time.perf_counter() - t0)
    e2e_identical = all(np.array_equal(a, b, equal_nan=True)
                        for a, b in zip(host_out, mixed_out if prob.batch else [mixed_out]))
    h2d = d2h = sum(b.nbytes for b in host_in)
    e2e_value = world * prob.cu * len(e_times) / sum(e_times)
    out = {
        "value": value, "unit": "cell-updates/s", "steps": steps, "warmup": W, "ms_per_step": 1000 * t_total / steps,
        "dtype": {"mixed_f64": "f32-flux+f64-acc", "mixed_kahan": "f32-flux+f32x2-acc"}.get(precision, precision),
        "config": {"workload": describe(workload, cells, order), "name": workload, "cells": cells or None,
                   "order": order if workload == "sod1d" else None, "cell_updates_per_run": prob.cu,
                   "precision": precision, "fold_steps": args.fold or ("autotuned" if prob.tuning() else 64),
                   "tuning": prob.tuning(), "parallelism": f"replicas{world}",
                   "l2": "flushed between runs (256 MB write)"},
        "roofline": roofline,
        "e2e": {"value": e2e_value, "unit": "cell-updates/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "host_memory": "pinned", "result_identical_to_device_run": e2e_identical},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if extras and rank == 0 and not precision.startswith("mixed"):
        out["cpu_baseline"] = cpu_baseline(workload, cells, order)
    elif extras and rank == 0:
        out.update(fp64_comparison(shll, torch, stream, prob, args, cells, order, mixed_out, t_total / steps))
    prob.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="sod1d", choices=["sod1d", "circle2d", "batch1d", "batch2d", "omp2d"])
    ap.add_argument("--cells", type=int, default=0, help="cells (1D) or side (2D); default per workload")
    ap.add_argument("--order", type=int, default=2)
    ap.add_argument("--fold", type=int, default=0, help="fold interval of the mixed path (0 = library default)")
    ap.add_argument("--precision", default="mixed_f64")
    ap.add_argument("--no-extras", action="store_true", help="skip the FP64 comparison runs and CPU baseline")
    ap.add_argument("--no-tune", action="store_true", help="1D mixed: skip the autotuner (library defaults)")
    ap.add_argument("--no-other-workloads", action="store_true",
                    help="measure only --workload (by default the sod1d line also carries batch1d, circle2d "
                         "and batch2d under 'workloads')")
    ap.add_argument("--other-steps", type=int, default=3, help="timed runs of each other workload")
    ap.add_argument("--run-steps", type=int, default=0,
                    help="single-domain workloads: a fixed number of time steps per run (small profiling cases)")
    args = ap.parse_args()
    global RUN_STEPS
    RUN_STEPS = args.run_steps
    workload = args.workload
    if args.cells == 0:
        args.cells = DEFAULT_CELLS.get(workload, 0)
    W = max(args.warmup, 3)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return
        config = {"workload": describe(workload, args.cells, args.order), "name": workload,
                  "cells": args.cells or None, "order": args.order if workload == "sod1d" else None}
        value, ms, sample, cores = reference_arm(args, workload, args.warmup)
        print(json.dumps({
            "impl": "reference", "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": config,
            "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": cores, "kind": "port", "sample": sample},
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
    head = measure(shll, torch, stream, workload, args.cells, args.order, args, args.steps, W, dist, world, rank,
                   local, not args.no_extras)
    others = {}
    if workload == "sod1d" and not args.no_other_workloads:
        for w in ("batch1d", "circle2d", "batch2d", "omp2d"):
            others[w] = measure(shll, torch, stream, w, DEFAULT_CELLS.get(w, 0), 1, args, args.other_steps, 3, dist,
                                world, rank, local, not args.no_extras)
    if rank == 0:
        head.pop("dtype")
        line = {"metric": "cell-updates/s", "value": head.pop("value"), "unit": head.pop("unit"), "n_gpus": world,
                "steps": head.pop("steps"), "warmup": head.pop("warmup"), "ms_per_step": head.pop("ms_per_step"),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": {"mixed_f64": "f32-flux+f64-acc", "mixed_kahan": "f32-flux+f32x2-acc"}.get(
                    head["config"]["precision"], head["config"]["precision"]),
                "data": "synthetic"}
        line.update(head)
        if others:
            line["workloads"] = others
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def host_cpu():
    """The host CPU model and its processor count."""
    model = ""
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                model = line.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    try:
        lscpu = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=5).stdout
        for line in lscpu.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
    except Exception:
        pass
    return f"{model or 'unknown CPU'}, nproc {os.cpu_count()}"


def cpu_sample_omp2d(n, steps):
    """base-omp's own problem on every host thread (the oracle's stages with an OpenMP team, FP32 as
    published): cell-updates/s, seconds, threads."""
    O = oracle_mod()
    threads = O.set_threads(0)
    try:
        cfg = O.make_cfg(dim=2, order=2, nx=n, ny=n, real_bits=32, limiter=1, mc_alpha=1.25, n_steps=steps)
        prim = O.ic_quadrants2d(n, n, 32)
        t0 = time.perf_counter()
        O.run(cfg, prim)
        dt = time.perf_counter() - t0
    finally:
        O.set_threads(1)
    return n * n * steps / dt, dt, threads


def cpu_baseline(workload, cells, order):
    """The CPU port of the reference timed on a bounded sample of the workload (1 thread; base-omp's
    problem on every host thread)."""
    if workload == "omp2d":
        steps = 200
        v, dt, threads = cpu_sample_omp2d(cells, steps)
        return {"value": v, "unit": "cell-updates/s", "cores": threads, "kind": "port",
                "sample": f"{cells}x{cells} cells x {steps} time steps, FP32 as published, {threads} threads "
                          f"(base-omp's OpenMP stages), {dt:.1f} s; host {host_cpu()}"}
    if workload in ("sod1d", "batch1d"):
        n = cells if workload == "sod1d" else 4096
        order = order if workload == "sod1d" else 2
        steps = max(50, int(3.0e8 / n))
        v, dt = cpu_sample(n, order, steps, 32)
        sample = f"{n} cells x {steps} time steps ({'order ' + str(order)}), FP32 as published, {dt:.1f} s"
    else:
        n = 512
        steps = max(20, int(2.0e8 / (n * n)))
        v, dt = cpu_sample_2d(n, steps, 32)
        sample = f"{n}x{n} cells x {steps} time steps, FP32 as published, {dt:.1f} s"
    return {"value": v, "unit": "cell-updates/s", "cores": 1, "kind": "port", "sample": sample}


def batch_results(shll, stream, items):
    b = shll.Batch(items)
    b.set_stream(stream.cuda_stream)
    b.run(allow_numeric=True)
    out = [(b.primitives(i), b.item_status(i)) for i in range(len(items))]
    b.close()
    return out


def pair_flux_run(shll, torch, stream, prob, f64_out, t_run, runs=3):
    """The same single-tube workload with every chunk in double-FP32 arithmetic
    (shll_set_pair_flux(2)): throughput (CUDA events, L2 flushed before each run), effective HBM
    fraction and L1 against the bit-exact FP64 run."""
    hbm, _ = peaks()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    shll.set_pair_flux(2)
    try:
        ctx = shll.Context(prob.p)
        ctx.set_stream(stream.cuda_stream)
        ctx.init_state()
        ctx.checkpoint()
        times = []
        for _ in range(runs + 1):
            ctx.restore()
            with torch.cuda.stream(stream):
                flush.add_(1.0)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.run()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1000.0)
        out = ctx.primitives()
        ctx.close()
    finally:
        shll.set_pair_flux(1)
    t = sum(times[1:]) / runs   # (the first run is a warm-up)
    value = prob.cu / t
    names = ["rho", "u", "v", "T"] if prob.dim == 2 else ["rho", "u", "T"]
    bpc = 64.0 if prob.dim == 2 else 48.0
    return {"value": value, "unit": "cell-updates/s", "ms_per_step": 1000 * t, "runs": runs,
            "roofline_frac": bpc * value / 1e9 / hbm, "speed_relative_to_fp32_flux": t_run / t,
            "l1_vs_fp64": dict(zip(names, [float(x) for x in np.mean(np.abs(out - f64_out), axis=1)])),
            "note": "fluxes, slopes and increments in double-FP32 arithmetic in every chunk"}


def fp64_comparison(shll, torch, stream, prob, args, cells, order, mixed_out, t_run):
    """Plain FP64 path (one launch per step) on the same workload (or a seeded subsample for the
    batches): throughput, L1 of the mixed result against it, CPU baseline."""
    out = {}
    if prob.batch:
        sub = 16 if prob.workload == "batch1d" else 8
        gen = items_batch1d if prob.workload == "batch1d" else items_batch2d
        items64 = gen(shll, "f64")[::sub]
        idx = list(range(0, len(prob.items), sub))
        b = shll.Batch(items64)
        b.set_stream(stream.cuda_stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.run(allow_numeric=True)
        e1.record(stream)
        e1.synchronize()
        t64 = e0.elapsed_time(e1) / 1000.0
        fused = [(b.primitives(j), b.item_status(j)) for j in range(len(items64))]
        b.close()
        # the bit-exact FP64 path (the oracle's arithmetic): the reference of the L1 figures; the
        # plain path's distance to it (fused multiply-add the only difference) measures how far the
        # FP64 result of an item is reproducible at all
        exact = batch_results(shll, stream, gen(shll, "f64_exact")[::sub])
        cu64 = sum(p.nx * (p.ny if p.dim == 2 else 1) * shll.steps_for(p) for p in items64)
        failed_mixed = set(prob.failed())
        names = ["rho", "u", "v", "T"] if prob.dim == 2 else ["rho", "u", "T"]
        by_order, l1s, worst, fail64 = {}, [], 0.0, 0
        for j, i in enumerate(idx):
            (pe, se), (pf, sf) = exact[j], fused[j]
            if se != 0 or sf != 0:
                fail64 += 1
                continue
            if i in failed_mixed:
                by_order.setdefault(prob.items[i].order, []).append((np.inf, 0.0))
                continue
            e = np.mean(np.abs(mixed_out[i] - pe), axis=1)
            floor = float(np.max(np.mean(np.abs(pf - pe), axis=1)))
            l1s.append(e)
            worst = max(worst, float(e[0]))
            by_order.setdefault(prob.items[i].order, []).append((float(np.max(e)), floor))
        summary = {}
        for o, v in sorted(by_order.items()):
            errs = np.array([x for x, _ in v])
            rep = [x for x, f in v if f <= 1e-8]
            other = [(x, f) for x, f in v if f > 1e-8]
            summary[f"order{o}"] = {
                "items": len(v), "median": float(np.median(errs)), "max": float(np.max(errs)),
                "items_at_or_below_1e-6": int(np.sum(errs <= 1e-6)),
                "fp64_reproducible_items": len(rep),
                "fp64_reproducible_at_or_below_1e-6": int(sum(x <= 1e-6 for x in rep)),
                "fp64_reproducible_max": float(max(rep)) if rep else None,
                "others_max_ratio_to_fp64_floor": float(max(x / f for x, f in other)) if other else None}
        out["l1_vs_fp64_by_order"] = summary
        out["l1_note"] = ("max over rho, u, [v,] T of L1 against the bit-exact FP64 path on the sampled items; an "
                          "item is FP64-reproducible when FP64 with and without fused multiply-add agree to 1e-8 "
                          "(on the others the reference scheme amplifies rounding beyond that)")
        out["items_broken_down"] = {"mixed_all_items": len(failed_mixed), "fp64_sampled_items": fail64,
                                    "mixed_sampled_items": len([i for i in idx if i in failed_mixed]),
                                    "note": "items whose density/energy went non-positive, overflowed or NaN "
                                            "(the reference scheme's own breakdown on strong tubes)"}
        out["fp64_plain"] = {"value": cu64 / t64, "unit": "cell-updates/s", "schedule": "one launch per step",
                             "precision": "f64", "sample": f"every {sub}th item ({len(items64)} items)"}
        out["speedup_vs_fp64_plain"] = (prob.cu / t_run) / (cu64 / t64)
        if l1s:
            out["l1_vs_fp64"] = dict(zip(names, [float(x) for x in np.mean(l1s, axis=0)]), rho_worst_item=worst)
        out["cpu_baseline"] = cpu_baseline(prob.workload, cells, order)
        return out
    prec64 = "f64_exact" if prob.workload == "sod1d" else "f64"
    p64 = params_single(shll, prob.workload, prec64, cells, order, 0)
    ctx = shll.Context(p64)
    ctx.set_stream(stream.cuda_stream)
    ctx.init_state()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ctx.run()
    e1.record(stream)
    e1.synchronize()
    t64 = e0.elapsed_time(e1) / 1000.0
    f64_out = ctx.primitives()
    ctx.close()
    l1 = np.mean(np.abs(mixed_out - f64_out), axis=1)
    names = ["rho", "u", "v", "T"] if prob.dim == 2 else ["rho", "u", "T"]
    out["fp64_plain"] = {"value": prob.cu / t64, "unit": "cell-updates/s", "schedule": "one launch per step",
                         "precision": prec64}
    out["speedup_vs_fp64_plain"] = (prob.cu / t_run) / (prob.cu / t64)
    out["l1_vs_fp64"] = dict(zip(names, [float(x) for x in l1]))
    if prec64 == "f64":
        # how far the FP64 result is reproducible at all: the same run without fused multiply-add
        ctx = shll.Context(params_single(shll, prob.workload, "f64_exact", cells, order, 0))
        ctx.set_stream(stream.cuda_stream)
        ctx.init_state()
        ctx.run()
        floor = np.mean(np.abs(ctx.primitives() - f64_out), axis=1)
        ctx.close()
        out["l1_fp64_fma_vs_exact"] = dict(zip(names, [float(x) for x in floor]))
    if prob.workload == "omp2d":
        # the second-order scheme's sensitivity at this size: FP64 from the initial state with density
        # and temperature perturbed by 6e-8 relative (FP32 rounding scale)
        p0 = params_single(shll, prob.workload, "f64", cells, order, 0)
        prim = shll.initial_primitives(p0)
        r = np.random.default_rng(0)
        prim[0] *= 1.0 + 6e-8 * r.uniform(-1.0, 1.0, prim.shape[1])
        prim[3] *= 1.0 + 6e-8 * r.uniform(-1.0, 1.0, prim.shape[1])
        p0.ic.kind = shll.IC_USER
        ctx = shll.Context(p0)
        ctx.set_stream(stream.cuda_stream)
        ctx.set_primitives(prim[0], prim[1], prim[3], v=prim[2])
        ctx.run()
        pert = np.mean(np.abs(ctx.primitives() - f64_out), axis=1)
        ctx.close()
        out["l1_fp64_perturbed_6e-8"] = dict(zip(names, [float(x) for x in pert]))
        out["l1_note"] = ("second order amplifies rounding at this size: FP64 from initial data perturbed by 6e-8 "
                          "relative moves by l1_fp64_perturbed_6e-8 (oracle/noise_floor.py spread2d on the CPU)")
    if prob.workload == "sod1d":
        O = oracle_mod()
        ex = O.riemann_exact(cells, shll.steps_for(prob.p) * (0.125 / cells))
        out["l1_rho_vs_exact_riemann"] = {"mixed": float(np.mean(np.abs(mixed_out[0] - ex[0]))),
                                          "fp64": float(np.mean(np.abs(f64_out[0] - ex[0])))}
        if order == 2:
            out["l1_note"] = ("second order amplifies rounding at this size: the FP64 run from initial data "
                              "perturbed by 6e-8 relative moves by L1(rho) 5.05e-5 (oracle/noise_floor.py); the "
                              "pair flux everywhere meets FP64 to 1e-6 (pair_flux_everywhere)")
        out["pair_flux_everywhere"] = pair_flux_run(shll, torch, stream, prob, f64_out, t_run)
    out["cpu_baseline"] = cpu_baseline(prob.workload, cells, order)
    return out


if __name__ == "__main__":
    main()
