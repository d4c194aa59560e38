#!/usr/bin/env python3
"""Benchmark of the GB300 prism path: Mcell*station/s of forward + adjoint.

Workloads (synthetic, seeded; see jif3d_gb300/workloads.py):
  plain   -- FP64 matrix-free forward + adjoint (LQDerivative) of one model,
             box terms recomputed on every call, on the 64x64x32 mesh with
             32x32 stations, g_z + FTG (joint, 10 raw values per station).

A step = one forward and one adjoint over the whole survey.  `value` counts
cells x stations per second with inputs resident in HBM; `e2e` is the same
through the public C ABI with host buffers (copies inside the timed region).

--impl reference times the CPU oracle (the C restatement of the reference's
OpenMP implementation, run with all host threads) on a bounded station
sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mcell*station/s fwd+adjoint"
UNIT = "Mcell*station/s"
L2_FLUSH_BYTES = 512 << 20  # > 129 MB L2

# FP64 flop-equivalents per node evaluation of the joint (g_z + 6 FTG) node
# terms: 21 add/mul + 1 sqrt + 3 ln + 4 atan2 with the per-call weights
# measured by ncu FP64 instruction counters (sqrt 13, ln 44, atan2 59.5;
# profiles/fp64_weights.md), plus 7 accumulation FMA.
FP64_FLOP_PER_NODE = {"joint": 418.0}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--workload", choices=["plain"], default="plain")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-i", str(self.index), "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def workload(name):
    from jif3d_gb300 import workloads as W
    if name == "plain":
        s = W.config4(nmodels=1)
        s.models = None
        return s
    raise ValueError(name)


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_ours(args, rank, world, local):
    import torch
    from jif3d_gb300 import capi, workloads as W
    torch.cuda.set_device(local)
    s = workload(args.workload)
    ctx = capi.Context(local)
    # a dedicated (non-default) stream: the engine and the CUDA events share it
    stream = torch.cuda.Stream(device=local)
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    W.setup_context(ctx, s)
    n = s.stations.shape[0]
    units = s.ngrid * n  # cells x stations per step
    dev = torch.device("cuda", local)
    d_model = torch.tensor(s.model, dtype=torch.float64, device=dev)
    d_data = torch.zeros(n * s.dpm, dtype=torch.float64, device=dev)
    d_grad = torch.zeros(s.nparm, dtype=torch.float64, device=dev)
    rng = np.random.default_rng(1)
    misfit_h = rng.normal(size=n * s.dpm)
    d_misfit = torch.tensor(misfit_h, dtype=torch.float64, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def step():
        ctx.forward_device(d_model.data_ptr(), d_data.data_ptr())
        ctx.lqderivative_device(d_model.data_ptr(), d_misfit.data_ptr(), d_grad.data_ptr())

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    l0 = ctx.launch_count()
    times = []
    for _ in range(args.steps):
        flush.zero_()  # L2 flush between timed steps (outside the events)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        step()
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
    torch.cuda.synchronize()
    launches = ctx.launch_count() - l0
    clk = clocks.stop()
    barrier(world)
    total_ms = max_over_ranks(sum(times), world)
    ms_per_step = total_ms / args.steps
    value = units * world * args.steps / (total_ms * 1e-3) / 1e6

    # end to end through the C ABI with host buffers (copies in the timed region)
    model_h = s.model.copy()
    for _ in range(2):
        ctx.forward(model_h)
        ctx.lqderivative(model_h, misfit_h)
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        data_h = ctx.forward(model_h)
        grad_h = ctx.lqderivative(model_h, misfit_h)
    t1 = time.perf_counter()
    e2e_s = max_over_ranks(t1 - t0, world)
    e2e = {"value": units * world * args.steps / e2e_s / 1e6, "unit": UNIT,
           "h2d_bytes_per_step": 8 * (2 * s.nparm + misfit_h.size),
           "d2h_bytes_per_step": 8 * (data_h.size + grad_h.size)}

    # FP64 roofline of the node kernels
    peak = ctx.probe_fp64()
    nodes = (s.shape[0] + 1) * (s.shape[1] + 1) * (s.shape[2] + 1)
    fpn = FP64_FLOP_PER_NODE["joint"]
    roof = None
    if fpn:
        achieved = 2 * nodes * n * fpn / (ms_per_step * 1e-3) / 1e9
        roof = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "GFLOP/s",
                "frac": achieved / peak, "traffic": None,
                "peak_source": "measured FP64 FMA probe (MEASURED_PEAKS.json has no FP64 entry)"}
    ctx.close()
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": s.name + "_plain_fp64_joint", "cells": s.ngrid, "stations": n,
                   "models": 1, "l2": "flushed between timed steps (512 MiB write)",
                   "parallelism": f"replicas{world}"},
        "e2e": e2e, "gpu_launches": launches, "roofline": roof, "clocks": clk,
    }


def cpu_sample_time(s, nthreads, budget_s=12.0):
    """Time the oracle's forward + LQDerivative on a station sample sized to
    about budget_s seconds of CPU work; returns (cell*station/s, sample text)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle import oracle as O
    from helpers import oracle_forward, oracle_lqderivative
    O.build()
    n = s.stations.shape[0]

    def run(k):
        sub = s.subset(np.arange(k) * max(1, n // k))
        t0 = time.perf_counter()
        d = oracle_forward(O, sub)
        oracle_lqderivative(O, sub, np.ones(d.size))
        return time.perf_counter() - t0, sub

    t1, _ = run(1)
    k = int(max(1, min(n, budget_s / max(t1, 1e-3))))
    t, sub = run(k)
    return s.ngrid * k / t / 1e6, f"{k} of {n} stations x all {s.ngrid} cells, fwd+adjoint"


def run_reference(args, rank, world):
    if rank != 0:
        return None
    s = workload(args.workload)
    nthreads = os.cpu_count() or 1
    vals, sample = [], ""
    for _ in range(max(1, args.steps if args.steps <= 3 else 3)):
        v, sample = cpu_sample_time(s, nthreads, budget_s=10.0)
        vals.append(v)
    v = statistics.median(vals)
    return {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": len(vals),
        "warmup": 0, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": {"workload": s.name + "_plain_fp64_joint", "cells": s.ngrid,
                   "stations": s.stations.shape[0], "models": 1},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    args = parse()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend=backend)
    if args.impl == "reference":
        res = run_reference(args, rank, world)
    else:
        res = run_ours(args, rank, world, local)
        if rank == 0:
            v, sample = cpu_sample_time(workload(args.workload), os.cpu_count() or 1)
            res["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": os.cpu_count() or 1,
                                   "kind": "port", "sample": sample}
    if rank == 0 and res is not None:
        print(json.dumps(res))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
