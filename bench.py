#!/usr/bin/env python3
"""Benchmark of the GB300 prism path: Mcell*station/s of forward + adjoint.

Workloads (synthetic, seeded; jif3d_gb300/workloads.py):
  batched (default) -- 64x64x32 cells (50 m, layers 25 m x1.05), 32x32
      stations at z = -50 m, joint g_z + FTG, 256 density models (Gaussian
      blobs + N(0, 0.05) g/cm^3).  The sensitivity is built once per geometry
      from the FP64 box terms and kept in HBM as fp16 hi + lo with a
      power-of-two row scale (as FullSensitivityGravMagCalculator keeps J
      between calls).  A step = batched forward of the 256 models, the
      weighted misfit (d - d_obs)/sigma^2, and the batched adjoint 2 J^T r,
      products on the tensor cores.
  plain -- the FP64 matrix-free forward + adjoint of one model on the same
      survey (box terms recomputed every call).

`value` counts cells x stations x models per second with inputs resident in
HBM; `e2e` is the same through the C ABI with host buffers (copies inside
the timed region).  Beside the headline the batched run reports the other
workloads (g_z 30x30x15, FTG 64x64x32 through the FP32 stored J, joint
96x96x48, total-field anomaly 128x128x64 over its 32 uneven station subsets),
each next to the oracle's OpenMP forward and adjoint on the host cores.
`--impl reference` times the CPU oracle (the C restatement of the reference's
implementation) on a bounded sample.

`--case` runs one small, self-contained case of a kernel family and exits
(for profiler captures that must end by themselves):
  node    -- FP64 node-term forward + adjoint, `--stations` of `--config`
  gemm    -- tensor-core batched products, `--stations` of the 64x64x32 survey
  stream  -- FP32 stored-J products, `--stations` of the FTG survey
  refine  -- projection / combination to a 2x2x2 refinement, `--models` models
  batched -- `--steps` batched steps (256 models, all stations), no timing
  reference-gpu -- the reference's own CUDA layer (Gravity/gravcuda.cu, built
      from the staged sources) on `--stations` stations of `--config` (1: g_z,
      2: FTG); prints one JSON line (run as a child process: the reference
      exits the process on a CUDA error)
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
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
SIGMA_GZ, SIGMA_U = 1e-8, 1e-9
# Nominal FP64 (non-tensor) rate of a GB300, for a second FP64 roofline
# denominator beside the library's own measured FMA rate.
FP64_NOMINAL_GFLOPS = 1250.0

# FP64 flops per joint node evaluation (an FMA counts 2): 21 add/mul + sqrt +
# 3 flog + 2 fatan2 + 1 fatan2_pair + 7 accumulation FMA, with the FP64
# instruction weights of the device functions counted by ncu on
# microkernels of each function (sqrt 13, flog 21, fatan2 36, fatan2_pair 42);
# the node kernels' own counters give 223 (forward) and 214 (adjoint).
FP64_FLOP_PER_JOINT_NODE = 225.0
# FP64 flops per node evaluation of the other kinds, counted by ncu
# (DFMA = 2, DADD, DMUL) on the node kernels, mean of forward and adjoint
FP64_FLOP_PER_NODE = {1: 110.0, 2: 210.0, 3: 208.0, 4: FP64_FLOP_PER_JOINT_NODE}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--workload", choices=["batched", "plain"], default="batched")
    p.add_argument("--models", type=int, default=256)
    p.add_argument("--sections", choices=["all", "headline"], default="all",
                   help="headline: only the batched step and its e2e / roofline (no other "
                        "workloads, no CPU baselines)")
    p.add_argument("--case", choices=["node", "gemm", "stream", "refine", "batched",
                                      "reference-gpu"])
    p.add_argument("--stations", type=int, default=64)
    p.add_argument("--config", type=int, default=4, choices=[1, 2, 3, 4, 5])
    return p.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region:
    start() returns once nvidia-smi is printing (so sampling covers the region
    from its first step), samples come every 10 ms and only those read between
    start() and stop() count."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index, period_ms=10):
        self.index = index
        self.period_ms = period_ms
        self.proc = None
        self.lines = []
        self.counting = False

    def _reader(self):
        for line in self.proc.stdout:
            if self.counting:
                self.lines.append(line)
            else:
                self.first.set()

    def start(self):
        import threading
        self.first = threading.Event()
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-i", str(self.index), "-lms", str(self.period_ms)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._reader, daemon=True)
        self.thread.start()
        self.first.wait(timeout=15)
        self.counting = True

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.counting = False
        lines = list(self.lines)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=10)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "power_w_max": max(power) if power else None, "samples": len(sm),
                "period_ms": self.period_ms}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, \
            "fallback"


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# DRAM traffic of one tensor-core product launch on the 64x64x32 survey with
# 1024 stations and 256 models: one-pass dram__bytes_read.sum +
# dram__bytes_write.sum of the full-size launches, mean of the forward and
# the adjoint, from the capture
#   ncu --metrics gpu__time_duration.sum,dram__bytes_read.sum,dram__bytes_write.sum
#       --clock-control none --csv python bench.py --case batched --steps 2
# (forward 3934.5 + 219.2 MB, adjoint 3813.1 + 257.6 MB).
GEMM_DRAM_BYTES_PER_LAUNCH = 0.5 * ((3940.2 + 117.7) + (3809.6 + 119.6)) * 1e6
GEMM_TRAFFIC_SOURCE = ("ncu one-pass dram__bytes_read.sum + dram__bytes_write.sum of the "
                       "full-size launches (mean of forward and adjoint, fixed-rule plans of "
                       "17 and 1 K splits) of `python bench.py --case batched --steps 2`, not "
                       "measured in this run")


def sigma_vector(s):
    n = s.stations.shape[0]
    return np.tile(np.array([SIGMA_GZ] + [SIGMA_U] * 9), n)


def timed_steps(step, nsteps, stream, flush):
    import torch
    times = []
    for _ in range(nsteps):
        flush.zero_()  # L2 flush between timed steps (outside the events)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        step()
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
    return times


def host_link(h_in, h_out, load):
    """Host link speed from page-locked buffers (best of 5): the input
    buffer copied in, the output buffer copied out, both at once on two
    streams, and both at once while `load` (device steps queued on the
    compute stream, longer than the copies) runs (GB/s of all bytes moved)."""
    import torch
    d_in = torch.empty_like(h_in, device="cuda")
    d_out = torch.empty_like(h_out, device="cuda")
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
    nb_in, nb_out = h_in.numel() * 8, h_out.numel() * 8

    def best(fn, nbytes, busy=None):
        t = []
        for _ in range(5):
            torch.cuda.synchronize()
            if busy:
                busy()
            t0 = time.perf_counter()
            fn()
            s_in.synchronize()
            s_out.synchronize()
            t.append(time.perf_counter() - t0)
            torch.cuda.synchronize()
        return nbytes / min(t) / 1e9

    def h2d():
        with torch.cuda.stream(s_in):
            d_in.copy_(h_in, non_blocking=True)

    def d2h():
        with torch.cuda.stream(s_out):
            h_out.copy_(d_out, non_blocking=True)

    def both():
        h2d()
        d2h()
    r = {"h2d_gbs": best(h2d, nb_in), "d2h_gbs": best(d2h, nb_out),
         "both_gbs": best(both, nb_in + nb_out),
         "both_under_load_gbs": best(both, nb_in + nb_out, load),
         "how": "torch copies of the pinned step buffers (models in, gradients out), "
                "alone and on two streams at once, idle and with three batched steps "
                "queued on the compute stream; best of 5"}
    del d_in, d_out
    return r


def measure_refinement(s, nmod, steps, stream, flush, local, peaks):
    """ProjectValues and CombineGradient of the batch between the inversion
    grid of the workload (coarse) and a forward grid refined 2 x 2 x 2; each
    pass is timed alone with CUDA events, L2 flushed in between.  Algorithmic
    bytes: project reads the coarse models and writes the refined ones,
    combine the reverse (8 bytes a value each way)."""
    import torch
    from jif3d_gb300 import capi
    half = [np.sort(np.concatenate([c, c[:-1] + 0.5 * np.diff(c)]))
            for c in (s.coords(0), s.coords(1), s.coords(2))]
    fine = [capi.refine_axis(s.coords(a), (s.xsize, s.ysize, s.zsize)[a], half[a])
            for a in range(3)]
    rctx = capi.Context(local)
    rctx.set_stream(stream.cuda_stream)
    corner = [np.concatenate([[o], o + np.cumsum(f)[:-1]]) for o, f in zip(s.origin, fine)]
    rctx.set_mesh(corner[0], corner[1], corner[2], *fine)
    rctx.set_background(s.bg_thick)
    rctx.set_refinement(s.xsize, s.ysize, s.zsize)
    nf = int(np.prod([f.size for f in fine])) + s.bg_thick.size
    coarse = torch.tensor(s.models, dtype=torch.float64, device=f"cuda:{local}")
    refined = torch.zeros((nmod, nf), dtype=torch.float64, device=coarse.device)
    back = torch.zeros_like(coarse)
    project = lambda: rctx.refine_project_device(nmod, coarse.data_ptr(), refined.data_ptr())
    combine = lambda: rctx.refine_combine_device(nmod, refined.data_ptr(), back.data_ptr())
    for _ in range(3):
        project()
        combine()
    torch.cuda.synchronize()
    t_p = statistics.median(timed_steps(project, steps, stream, flush))
    t_c = statistics.median(timed_steps(combine, steps, stream, flush))
    nbytes = 8 * (coarse.numel() + refined.numel())
    out = {"coarse_cells": s.ngrid, "refined_cells": nf - s.bg_thick.size, "models": nmod,
           "refined_shape": [f.size for f in fine], "bytes_per_pass": nbytes,
           "project_ms": t_p, "combine_ms": t_c,
           "project_gbs": nbytes / (t_p * 1e-3) / 1e9, "combine_gbs": nbytes / (t_c * 1e-3) / 1e9,
           "hbm_peak_gbs": peaks["hbm_gbs"]}
    out["project_frac"] = out["project_gbs"] / peaks["hbm_gbs"]
    out["combine_frac"] = out["combine_gbs"] / peaks["hbm_gbs"]
    rctx.close()
    return out


def cpu_oracle_config(s, nst, seed):
    """The oracle's OpenMP forward (Calculate) and LQDerivative of one model
    on the host cores, on `nst` seeded stations of the survey (all of them
    when it has no more): Mcell*station/s of each and of their sum (the
    throughput of a (cell, station) pair does not depend on the station)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle import oracle as O
    from helpers import oracle_forward, oracle_lqderivative
    O.build()
    n = s.stations.shape[0]
    if nst >= n:
        idx, what = np.arange(n), f"all {n} stations"
    else:
        idx = np.sort(np.random.default_rng(seed).choice(n, nst, replace=False))
        what = f"{nst} of {n} stations (seeded sample, seed {seed})"
    sub = s.subset(idx)
    sub.subsets = None
    misfit = np.random.default_rng(seed + 1).normal(size=idx.size * sub.dpm)
    t0 = time.perf_counter()
    oracle_forward(O, sub)
    t1 = time.perf_counter()
    oracle_lqderivative(O, sub, misfit)
    t2 = time.perf_counter()
    pairs = s.ngrid * idx.size / 1e6
    return {"value": pairs / (t2 - t0), "forward": pairs / (t1 - t0),
            "adjoint": pairs / (t2 - t1), "unit": UNIT, "cores": os.cpu_count() or 1,
            "kind": "port", "seconds": t2 - t0,
            "sample": f"oracle OpenMP forward + LQDerivative, one model, {what} x all "
                      f"{s.ngrid} cells"}


def measure_stream(steps, stream, flush, local, peaks, cpu):
    """The FTG survey on the 64 x 64 x 32 mesh with 40 x 40 stations: the
    forward and adjoint of one model through the FP32 device-resident J (six
    stored rows per station: 9600 x 131072, 5.03 GB), each streaming J once
    (k_gemv_f32 / k_gemv_t_f32), timed alone with CUDA events, L2 flushed in
    between; next to the FP64 matrix-free path on the same survey, the FP32
    products' errors against it, and the oracle on the host cores."""
    import torch
    from jif3d_gb300 import capi, workloads as W
    s = W.config2()
    ctx = capi.Context(local)
    ctx.set_stream(stream.cuda_stream)
    W.setup_context(ctx, s)
    dev = f"cuda:{local}"
    n = s.stations.shape[0]
    nd = n * s.dpm
    m = torch.tensor(s.model, dtype=torch.float64, device=dev)
    r = torch.tensor(np.random.default_rng(12).normal(size=nd), dtype=torch.float64, device=dev)
    d64, d32 = (torch.zeros(nd, dtype=torch.float64, device=dev) for _ in range(2))
    g64, g32 = (torch.zeros(s.nparm, dtype=torch.float64, device=dev) for _ in range(2))

    fwd64 = lambda: ctx.forward_device(m.data_ptr(), d64.data_ptr())
    adj64 = lambda: ctx.lqderivative_device(m.data_ptr(), r.data_ptr(), g64.data_ptr())
    fwd64()
    adj64()
    t_pf = statistics.median(timed_steps(fwd64, 2, stream, flush))
    t_pa = statistics.median(timed_steps(adj64, 2, stream, flush))
    ctx.build_sensitivity(capi.STORE_FP32)
    info = ctx.sensitivity_info()
    fwd = lambda: ctx.stored_forward_device(m.data_ptr(), d32.data_ptr())
    adj = lambda: ctx.stored_lqderivative_device(m.data_ptr(), r.data_ptr(), g32.data_ptr())
    for _ in range(3):
        fwd()
        adj()
    torch.cuda.synchronize()
    t_f = statistics.median(timed_steps(fwd, steps, stream, flush))
    t_a = statistics.median(timed_steps(adj, steps, stream, flush))
    jb = info["bytes"]
    relerr = lambda x, y: float(torch.linalg.norm(x - y) / torch.linalg.norm(y))
    pairs = s.ngrid * n / 1e6
    out = {"workload": s.name + "_fp32_stored", "cells": s.ngrid, "stations": n,
           "stored_rows": info["rows"], "j_bytes": jb,
           "value": pairs / ((t_f + t_a) * 1e-3), "unit": UNIT,
           "forward_ms": t_f, "adjoint_ms": t_a,
           "forward_gbs": jb / (t_f * 1e-3) / 1e9, "adjoint_gbs": jb / (t_a * 1e-3) / 1e9,
           "hbm_peak_gbs": peaks["hbm_gbs"],
           "plain_fp64": {"value": pairs / ((t_pf + t_pa) * 1e-3),
                          "forward": pairs / (t_pf * 1e-3), "adjoint": pairs / (t_pa * 1e-3),
                          "ms_per_step": t_pf + t_pa},
           "err_vs_fp64": {"data": relerr(d32, d64), "grad": relerr(g32, g64)},
           "how": "J streamed once per direction (algorithmic bytes = J bytes); times include "
                  "the model conversion, the chunk sums and the assembly / weights kernels"}
    out["forward_frac"] = out["forward_gbs"] / peaks["hbm_gbs"]
    out["adjoint_frac"] = out["adjoint_gbs"] / peaks["hbm_gbs"]
    out["speedup_vs_plain_fp64"] = out["value"] / out["plain_fp64"]["value"]
    ctx.close()
    if cpu:
        out["cpu_baseline"] = cpu_oracle_config(s, 64, 202)
        out["speedup_vs_cpu"] = out["value"] / out["cpu_baseline"]["value"]
        out["plain_fp64"]["speedup_vs_cpu"] = (out["plain_fp64"]["value"] /
                                               out["cpu_baseline"]["value"])
    return out


def measure_fp64_configs(stream, flush, local, cpu):
    """The FP64 matrix-free forward and adjoint of one model on the other
    workloads, each timed with CUDA events (L2 flushed in between): g_z on
    the 30 x 30 x 15 mesh (400 stations, 3 background layers), joint g_z +
    FTG on 96 x 96 x 48 (2500 stations), and the total-field anomaly on
    128 x 128 x 64 over all 32 uneven station subsets (74,753 stations in one
    subsets forward and one subsets adjoint call; no warm-up, one call each,
    ~40 s).  FP64 roofline: node evaluations x FP64 flops per node of the
    kind / time, against the library's measured FP64 FMA rate and against the
    nominal rate.  Beside each, the oracle's OpenMP forward and LQDerivative
    on the host cores (all stations of the g_z survey, 64 seeded stations of
    the others)."""
    import torch
    from jif3d_gb300 import capi, workloads as W
    dev = f"cuda:{local}"
    out = {}
    peak = None
    for cfg, full_batch, nsteps, cpu_nst in ((1, False, 5, 400), (3, False, 2, 64),
                                             (5, True, 1, 64)):
        s = W.CONFIGS[cfg]()
        ctx = capi.Context(local)
        ctx.set_stream(stream.cuda_stream)
        W.setup_context(ctx, s)
        peak = peak or ctx.probe_fp64()
        m = torch.tensor(s.model, dtype=torch.float64, device=dev)
        rng = np.random.default_rng(cfg)
        if full_batch:
            subs = s.subsets
            nst = sum(len(x) for x in subs)
            nd = nst * s.dpm
            d = torch.zeros(nd, dtype=torch.float64, device=dev)
            r = torch.tensor(rng.normal(size=nd), dtype=torch.float64, device=dev)
            g = torch.zeros((len(subs), s.nparm), dtype=torch.float64, device=dev)
            fwd = lambda: ctx.subsets_forward_device(subs, m.data_ptr(), d.data_ptr())
            adj = lambda: ctx.subsets_lqderivative_device(subs, m.data_ptr(), r.data_ptr(),
                                                          g.data_ptr())
        else:
            nst = s.stations.shape[0]
            nd = nst * s.dpm
            d = torch.zeros(nd, dtype=torch.float64, device=dev)
            r = torch.tensor(rng.normal(size=nd), dtype=torch.float64, device=dev)
            g = torch.zeros(s.nparm, dtype=torch.float64, device=dev)
            fwd = lambda: ctx.forward_device(m.data_ptr(), d.data_ptr())
            adj = lambda: ctx.lqderivative_device(m.data_ptr(), r.data_ptr(), g.data_ptr())
            fwd()
            adj()
            torch.cuda.synchronize()
        t_f = statistics.median(timed_steps(fwd, nsteps, stream, flush))
        t_a = statistics.median(timed_steps(adj, nsteps, stream, flush))
        t = t_f + t_a
        nodes = (s.shape[0] + 1) * (s.shape[1] + 1) * (s.shape[2] + 1)
        kind = s.kind  # scalar 1, tensor 2, magnetic 3, joint 4
        gflops = 2 * nodes * nst * FP64_FLOP_PER_NODE[kind] / (t * 1e-3) / 1e9
        pairs = s.ngrid * nst / 1e6
        e = {"cells": s.ngrid, "stations": nst, "ms_per_step": t,
             "forward_ms": t_f, "adjoint_ms": t_a,
             "value": pairs / (t * 1e-3), "forward": pairs / (t_f * 1e-3),
             "adjoint": pairs / (t_a * 1e-3), "unit": UNIT,
             "fp64_gflops": gflops, "fp64_frac": gflops / peak,
             "fp64_frac_of_nominal": gflops / FP64_NOMINAL_GFLOPS,
             "flop_per_node": FP64_FLOP_PER_NODE[kind]}
        if full_batch:
            e["subsets"] = len(subs)
            e["subset_sizes"] = [int(min(len(x) for x in subs)), int(max(len(x) for x in subs))]
            e["how"] = "one subsets forward + one subsets adjoint call over all 32 subsets"
        ctx.close()
        del d, r, g
        if cpu:
            e["cpu_baseline"] = cpu_oracle_config(s, cpu_nst, 200 + cfg)
            e["speedup_vs_cpu"] = e["value"] / e["cpu_baseline"]["value"]
        out[s.name] = e
    out["fp64_peak_gflops"] = peak
    out["fp64_peak_source"] = ("j3g_probe_fp64: this library's FMA-chain probe kernel "
                               "(no FP64 figure in MEASURED_PEAKS.json); fp64_frac_of_nominal "
                               f"uses the nominal {FP64_NOMINAL_GFLOPS:.0f} GFLOP/s")
    out["how"] = ("forward and adjoint of one model, each timed on its own; fp64_frac counts "
                  "node evaluations only (the background, reductions and assembly are in the "
                  "time)")
    return out


def measure_netcdf(s, data):
    """Host throughput of the library's NetCDF writer and reader on the
    workload's files: the density model (131,072 cells) and the FTG data of
    the 1024 stations, written as CDF-2 and read back (MB/s of file bytes)."""
    import tempfile
    from jif3d_gb300 import gravmag as G, netcdf as N
    M = G.ThreeDGravityModel()
    M.SetMeshSize(*s.shape)
    M.SetXCellSizes(s.xsize)
    M.SetYCellSizes(s.ysize)
    M.SetZCellSizes(s.zsize)
    M.SetData()[...] = s.model[:s.ngrid].reshape(s.shape)
    st = s.stations
    with tempfile.TemporaryDirectory() as tmp:
        out = {}
        for name, write, read in (
                ("model", lambda f: M.WriteNetCDF(f), lambda f: G.ThreeDGravityModel().ReadNetCDF(f)),
                ("ftg_data", lambda f: N.SaveTensorGravityMeasurements(
                    f, data, st[:, 0], st[:, 1], st[:, 2], np.ones_like(data)),
                 lambda f: N.ReadTensorGravityMeasurements(f))):
            f = os.path.join(tmp, name + ".nc")
            t0 = time.perf_counter()
            write(f)
            t1 = time.perf_counter()
            read(f)
            t2 = time.perf_counter()
            mb = os.path.getsize(f) / 1e6
            out[name] = {"file_mb": mb, "write_mbs": mb / (t1 - t0), "read_mbs": mb / (t2 - t1)}
    return out


def pipelined_steps(ctx, sets, nsteps, misfit, nsets=3, back=2):
    """The end-to-end loop over the pipelined host-buffer calls
    (j3g_batched_forward_async / _lqderivative_async / j3g_batched_wait).

    Step i waits for its own data, forms the misfit on the host (``misfit(st)``
    reads st["data"] and writes st["mis"]), queues its derivative and then the
    forward of step i + 2 (the batches' models are known ahead, as for
    independent batches); the gradient of step i - ``back`` is taken (waited
    for) last, before its host buffers come round again (``nsets`` sets of
    arrays "models", "data", "mis", "grads").  With back = 1 the host waited
    there until that gradient (268 MB) had come back, so the forward of step
    i + 3 was queued late and waited for its models; back = 2 needs three
    sets, or the misfit of step i + 1 overwrites what the derivative of step
    i - 1 may still be reading.  The library's ring holds four calls (a fifth
    waits for the oldest)."""
    fwd, adj = {}, {}

    def queue_fwd(i):
        st = sets[i % nsets]
        fwd[i] = ctx.batched_forward_async(st["models"], out=st["data"])
    for i in range(min(2, nsteps)):
        queue_fwd(i)
    for i in range(nsteps):
        st = sets[i % nsets]
        ctx.batched_wait(fwd[i])
        misfit(st)
        adj[i] = ctx.batched_lqderivative_async(st["models"], st["mis"], out=st["grads"])
        if i + 2 < nsteps:
            queue_fwd(i + 2)
        if i >= back:
            ctx.batched_wait(adj[i - back])
    for i in range(max(0, nsteps - back), nsteps):
        ctx.batched_wait(adj[i])


def run_batched(args, rank, world, local):
    import torch
    from jif3d_gb300 import capi, workloads as W
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    s = W.config4(nmodels=args.models)
    nmod = s.models.shape[0]
    ctx = capi.Context(local)
    stream = torch.cuda.Stream(device=local)
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    W.setup_context(ctx, s)
    n = s.stations.shape[0]
    R, K = n * 7, s.ngrid
    units = s.ngrid * n * nmod

    # observed data: FP64 matrix-free response of the base model + noise
    sig = sigma_vector(s)
    d_base = torch.tensor(s.model, dtype=torch.float64, device=dev)
    d_obs = torch.zeros(n * 10, dtype=torch.float64, device=dev)
    ctx.forward_device(d_base.data_ptr(), d_obs.data_ptr())
    ctx.synchronize()
    rng = np.random.default_rng(44)
    d_obs += torch.tensor(sig * rng.normal(size=n * 10), dtype=torch.float64, device=dev)
    w = torch.tensor(1.0 / sig ** 2, dtype=torch.float64, device=dev)
    # the weighted misfit (d - d_obs) w as one elementwise pass: d w - d_obs w
    neg_obs_w = -(d_obs * w)

    # sensitivity build (once per geometry, outside the timed steps)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ctx.build_sensitivity(capi.STORE_F16X2)
    e1.record(stream)
    e1.synchronize()
    build_ms = e0.elapsed_time(e1)
    info = ctx.sensitivity_info()

    ctx.set_autotune(True)  # first products of each shape pick their plan (warm-up)
    models = torch.tensor(s.models, dtype=torch.float64, device=dev)
    data = torch.zeros((nmod, n * 10), dtype=torch.float64, device=dev)
    misfit = torch.zeros_like(data)
    grads = torch.zeros_like(models)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def step():
        ctx.batched_forward_device(nmod, models.data_ptr(), data.data_ptr())
        torch.addcmul(neg_obs_w, data, w, out=misfit)
        ctx.batched_lqderivative_device(nmod, models.data_ptr(), misfit.data_ptr(),
                                        grads.data_ptr())

    for _ in range(args.warmup):
        step()
    ctx.synchronize()
    torch.cuda.synchronize()
    # the whole step (library kernels and the torch misfit) in one CUDA graph;
    # the warm-up calls made every allocation, so capture sees stream work only
    graph = torch.cuda.CUDAGraph()
    l0 = ctx.launch_count()
    with torch.cuda.graph(graph, stream=stream):
        step()
    launches_per_step = ctx.launch_count() - l0
    for _ in range(args.warmup):
        graph.replay()
    torch.cuda.synchronize()
    barrier(world)
    clocks = ClockSampler(local)
    clocks.start()
    times = timed_steps(graph.replay, args.steps, stream, flush)
    clk = clocks.stop()
    launches = launches_per_step * args.steps
    # eager steps with the per-phase CUDA-event timers (breakdown and roofline)
    ctx.set_timing(True)
    eager_times = timed_steps(step, args.steps, stream, flush)
    gf_ms, gf_n = ctx.get_timing(capi.TIMER_GEMM_FORWARD)
    ga_ms, ga_n = ctx.get_timing(capi.TIMER_GEMM_ADJOINT)
    phase_ms = {name: ctx.get_timing(t)[0] / args.steps
                for name, t in (("split", capi.TIMER_SPLIT), ("split_sums", capi.TIMER_REDUCE),
                                ("epilogue", capi.TIMER_EPILOGUE))}
    phase_ms["gemm"] = (gf_ms + ga_ms) / args.steps
    phase_ms["eager_step"] = sum(eager_times) / args.steps
    ctx.set_timing(False)
    ctx.synchronize()
    barrier(world)
    total_ms = max_over_ranks(sum(times), world)
    ms_per_step = total_ms / args.steps
    value = units * world * args.steps / (total_ms * 1e-3) / 1e6

    # accuracy of the mixed path against the FP64 matrix-free path: four
    # models at all stations (data and gradient of the step's misfit), and
    # the data of all models at every eighth station
    errs = {"data_gz": 0.0, "data_ftg": 0.0, "grad": 0.0,
            "max_abs_data_gz": 0.0, "max_abs_data_ftg": 0.0, "max_abs_grad": 0.0}
    ref = torch.zeros(n * 10, dtype=torch.float64, device=dev)
    gref = torch.zeros(s.nparm, dtype=torch.float64, device=dev)
    rel = lambda x, y: float(torch.linalg.norm(x - y) / torch.linalg.norm(y))
    for i in (0, nmod // 3, (2 * nmod) // 3, nmod - 1):
        ctx.forward_device(models[i].data_ptr(), ref.data_ptr())
        ctx.lqderivative_device(models[i].data_ptr(), misfit[i].data_ptr(), gref.data_ptr())
        ctx.synchronize()
        a, r = data[i].view(n, 10), ref.view(n, 10)
        for key, x, y in (("data_gz", a[:, 0], r[:, 0]), ("data_ftg", a[:, 1:], r[:, 1:]),
                          ("grad", grads[i], gref)):
            errs[key] = max(errs[key], rel(x, y))
            errs["max_abs_" + key] = max(errs["max_abs_" + key], float((x - y).abs().max()))
    sub_idx = np.arange(0, n, 8)
    sctx = capi.Context(local)
    sctx.set_stream(stream.cuda_stream)
    W.setup_context(sctx, s.subset(sub_idx))
    sref = torch.zeros(sub_idx.size * 10, dtype=torch.float64, device=dev)
    sub_t = torch.tensor(sub_idx, device=dev)
    sub_worst = {"data_gz": 0.0, "data_ftg": 0.0}
    for i in range(nmod):
        sctx.forward_device(models[i].data_ptr(), sref.data_ptr())
        a, r = data[i].view(n, 10)[sub_t], sref.view(-1, 10)
        sub_worst["data_gz"] = max(sub_worst["data_gz"], rel(a[:, 0], r[:, 0]))
        sub_worst["data_ftg"] = max(sub_worst["data_ftg"], rel(a[:, 1:], r[:, 1:]))
    sctx.close()
    errs["all_models_on_station_subset"] = sub_worst
    errs["how"] = ("relative norm errors (max over models) and max absolute errors (SI) "
                   "against the FP64 matrix-free path: 4 models at all 1024 stations (data and "
                   "gradient); all models' data at 128 stations (every eighth)")

    # plain FP64 matrix-free path, one model, same survey (for the ratio)
    plain_t = []
    for it in range(3):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ctx.forward_device(models[0].data_ptr(), data[0].data_ptr())
        ctx.lqderivative_device(models[0].data_ptr(), misfit[0].data_ptr(), grads[0].data_ptr())
        b.record(stream)
        b.synchronize()
        if it > 0:
            plain_t.append(a.elapsed_time(b))
    plain_ms = statistics.median(plain_t)
    plain_value = s.ngrid * n / (plain_ms * 1e-3) / 1e6

    # end to end through the C ABI with host buffers in pinned memory: every
    # step copies the models and the misfits in, the data and the gradients
    # out (the linear adjoint does not read the models); the weighted misfit
    # is computed on the host between the two calls
    def pinned(shape):
        return torch.empty(shape, dtype=torch.float64, pin_memory=True)
    sets = []
    for _ in range(3):  # host buffers of three steps in flight
        st = {k: pinned(shape) for k, shape in (("models", s.models.shape), ("data", data.shape),
                                                 ("mis", data.shape), ("grads", s.models.shape))}
        st["models"].copy_(torch.from_numpy(s.models))
        sets.append(st)
    neg_obs_w_t, w_t = neg_obs_w.cpu(), torch.from_numpy(1.0 / sig ** 2)

    def host_misfit(st):
        torch.addcmul(neg_obs_w_t, st["data"], w_t, out=st["mis"])

    def e2e_blocking(nsteps):
        st = sets[0]
        for _ in range(nsteps):
            ctx.batched_forward(st["models"].numpy(), out=st["data"].numpy())
            host_misfit(st)
            ctx.batched_lqderivative(st["models"].numpy(), st["mis"].numpy(),
                                     out=st["grads"].numpy())

    # the same buffers as numpy arrays for the pipelined calls, with their
    # torch views for the misfit
    np_sets = [dict({k: v.numpy() for k, v in st.items()}, torch=st) for st in sets]

    def e2e_pipelined(nsteps):
        pipelined_steps(ctx, np_sets, nsteps, lambda st: host_misfit(st["torch"]))

    # warm-up: each ring slot replays its product from a CUDA graph once the
    # same shape has run there twice; a run of K steps takes 2K tickets of the
    # four-slot ring, so two runs warm both phases of the ring (no graph is
    # captured inside the timed runs)
    for _ in range(2):
        e2e_pipelined(args.steps)
    e2e_blocking(2)
    barrier(world)
    # five timed runs of K steps each way: the median is reported, all listed
    # (the host link is shared with the machine's other work, and single runs
    # of a few tens of ms now and then take twice as long)
    sync_runs, pipe_runs = [], []
    for _ in range(5):
        t0 = time.perf_counter()
        e2e_blocking(args.steps)
        t1 = time.perf_counter()
        e2e_pipelined(args.steps)
        t2 = time.perf_counter()
        sync_runs.append(max_over_ranks(t1 - t0, world))
        pipe_runs.append(max_over_ranks(t2 - t1, world))
    sync_s = statistics.median(sync_runs)
    e2e_s = statistics.median(pipe_runs)
    nbytes_in = 8 * (s.models.size + data.numel())
    nbytes_out = 8 * (data.numel() + s.models.size)
    def load():
        for _ in range(3):
            step()
    link = host_link(sets[0]["models"], sets[1]["grads"], load)
    link["bound_ms_per_step"] = (nbytes_in + nbytes_out) / (link["both_gbs"] * 1e6)
    link["bound_under_load_ms_per_step"] = ((nbytes_in + nbytes_out) /
                                            (link["both_under_load_gbs"] * 1e6))
    # the host's misfit alone (it sits between the two calls of a step)
    mis_t = []
    for _ in range(7):
        a0 = time.perf_counter()
        host_misfit(sets[0])
        mis_t.append((time.perf_counter() - a0) * 1e3)
    e2e = {"value": units * world * args.steps / e2e_s / 1e6, "unit": UNIT,
           "h2d_bytes_per_step": nbytes_in, "host_buffers": "pinned",
           "d2h_bytes_per_step": nbytes_out, "ms_per_step": e2e_s * 1e3 / args.steps,
           "link": link,
           "host_misfit_ms": statistics.median(mis_t), "host_threads": torch.get_num_threads(),
           "runs_ms_per_step": [x * 1e3 / args.steps for x in pipe_runs],
           "how": "pipelined calls (j3g_batched_*_async): each step's forward is queued two "
                  "steps ahead, the gradient two steps back is waited for (three host buffer "
                  "sets); copies on their own streams (in and out per direction) overlap the "
                  "products; median of five timed runs of K steps",
           "blocking": {"value": units * world * args.steps / sync_s / 1e6,
                        "runs_ms_per_step": [x * 1e3 / args.steps for x in sync_runs],
                        "how": "j3g_batched_forward / j3g_batched_lqderivative, one at a time"}}

    peaks, src = measured_peaks()
    flops_alg = 2.0 * R * nmod * K  # per product launch, either direction
    gemm_ms = (gf_ms + ga_ms) / max(1, gf_n + ga_n)
    achieved = flops_alg / (gemm_ms * 1e-3) / 1e12
    j_bytes = 2 * R * info["cols"] * 2  # hi + lo read once per launch
    # fp16 and bf16 MMA (kind::f16) share one dense rate; the measured cuBLAS
    # bf16 figure is the denominator
    roof = {"bound": "tensor", "achieved": achieved, "peak": peaks["bf16_tflops"],
            "unit": "TFLOP/s", "frac": achieved / peaks["bf16_tflops"],
            "traffic": GEMM_DRAM_BYTES_PER_LAUNCH,
            "flops_per_launch": flops_alg,
            "flops_how": "2 x rows x cells x models per product launch (7 stored rows per "
                         "station), the algorithmic work of one J M or J^T R",
            "traffic_unit": "DRAM bytes per launch", "traffic_source": GEMM_TRAFFIC_SOURCE,
            # J hi + lo and the forward's model hi + lo, read once; the
            # per-split partial sums come on top
            "algorithmic_bytes_per_launch": j_bytes + 4 * nmod * K,
            "peak_source": f"{src} bf16_tflops (burst; fp16 MMA runs at the bf16 rate)",
            "kernel": "k_gemm_pair<fp16> (CTA pair, 256 x 256 tiles, 3 fp16 products per launch)",
            "ms_per_launch": {"forward": gf_ms / max(1, gf_n), "adjoint": ga_ms / max(1, ga_n)},
            "plans": {"forward": ctx.gemm_plan(0), "adjoint": ctx.gemm_plan(1),
                      "how": "autotuned on the first call of each shape (K splits, N tile)"},
            "executed_frac": 3 * achieved / peaks["bf16_tflops"],
            "executed_how": "tensor-pipe work actually issued (hi*hi + hi*lo + lo*hi: 3 x the "
                            "algorithmic flops) over the same peak",
            "j_stream_gbs": j_bytes / (gemm_ms * 1e-3) / 1e9,
            "j_stream_hbm_frac": j_bytes / (gemm_ms * 1e-3) / 1e9 / peaks["hbm_gbs"],
            "hbm_peak_gbs": peaks["hbm_gbs"]}
    ctx.close()
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "fp16x2 (hi+lo) J and models, fp32 accumulators drained every 32 cells, "
                 "fp64 split sums",
        "data": "synthetic",
        "config": {"workload": s.name + "_f16x2_256models", "cells": s.ngrid, "stations": n,
                   "models": nmod, "rows": R, "kind": "joint g_z + FTG",
                   "l2": "flushed between timed steps (512 MiB write); J (3.8 GB per direction) "
                         "exceeds L2",
                   "parallelism": f"replicas{world}"},
        "sensitivity_build_ms": build_ms, "sensitivity_bytes": info["bytes"],
        "gpu_launches": launches, "clocks": clk,
        "step": "one CUDA graph per step (batched forward, weighted misfit, batched "
                "adjoint: %d library kernels + 1 torch kernel), replayed" % launches_per_step,
        "ms_per_step_by_phase": phase_ms,
        "plain_fp64": {"value": plain_value, "unit": UNIT, "ms_per_step": plain_ms,
                       "what": "FP64 matrix-free fwd+adjoint of one model, same survey"},
    }
    if args.sections == "all":
        cpu = rank == 0
        out["refinement"] = measure_refinement(s, nmod, args.steps, stream, flush, local, peaks)
        out["stream_fp32"] = measure_stream(args.steps, stream, flush, local, peaks, cpu)
        out["fp64_configs"] = measure_fp64_configs(stream, flush, local, cpu)
        if rank == 0:
            out["reference_gpu"] = measure_reference_gpu(
                local, {1: lambda idx: our_gridded(local, 1, idx),
                        2: lambda idx: our_gridded(local, 2, idx)})
        ftg = data[0].view(n, 10)[:, 1:].reshape(-1).cpu().numpy()
        out["netcdf"] = measure_netcdf(s, ftg) if rank == 0 else None
    out["e2e"] = e2e
    out["roofline"] = roof
    out["speedup_vs_plain_fp64"] = value / plain_value
    out["err_vs_fp64"] = errs
    return out


def run_plain(args, rank, world, local):
    import torch
    from jif3d_gb300 import capi, workloads as W
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    s = W.config4(nmodels=1)
    ctx = capi.Context(local)
    stream = torch.cuda.Stream(device=local)
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    W.setup_context(ctx, s)
    n = s.stations.shape[0]
    units = s.ngrid * n
    d_model = torch.tensor(s.model, dtype=torch.float64, device=dev)
    d_data = torch.zeros(n * 10, dtype=torch.float64, device=dev)
    d_grad = torch.zeros(s.nparm, dtype=torch.float64, device=dev)
    misfit_h = np.random.default_rng(1).normal(size=n * 10)
    d_misfit = torch.tensor(misfit_h, dtype=torch.float64, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def step():
        ctx.forward_device(d_model.data_ptr(), d_data.data_ptr())
        ctx.lqderivative_device(d_model.data_ptr(), d_misfit.data_ptr(), d_grad.data_ptr())

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(world)
    clocks = ClockSampler(local)
    clocks.start()
    ctx.set_timing(True)
    l0 = ctx.launch_count()
    times = timed_steps(step, args.steps, stream, flush)
    launches = ctx.launch_count() - l0
    nf_ms, nf_n = ctx.get_timing(capi.TIMER_NODE_FORWARD)
    na_ms, na_n = ctx.get_timing(capi.TIMER_NODE_ADJOINT)
    ctx.set_timing(False)
    clk = clocks.stop()
    barrier(world)
    total_ms = max_over_ranks(sum(times), world)
    ms_per_step = total_ms / args.steps
    value = units * world * args.steps / (total_ms * 1e-3) / 1e6
    model_h = s.model.copy()
    for _ in range(2):
        ctx.forward(model_h)
        ctx.lqderivative(model_h, misfit_h)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        dh = ctx.forward(model_h)
        gh = ctx.lqderivative(model_h, misfit_h)
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e = {"value": units * world * args.steps / e2e_s / 1e6, "unit": UNIT,
           "h2d_bytes_per_step": 8 * (2 * s.nparm + misfit_h.size),
           "d2h_bytes_per_step": 8 * (dh.size + gh.size)}
    peak = ctx.probe_fp64()
    nodes = (s.shape[0] + 1) * (s.shape[1] + 1) * (s.shape[2] + 1)
    node_ms = (nf_ms + na_ms) / max(1, nf_n + na_n)
    achieved = nodes * n * FP64_FLOP_PER_JOINT_NODE / (node_ms * 1e-3) / 1e9
    ctx.close()
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": s.name + "_plain_fp64_joint", "cells": s.ngrid, "stations": n,
                   "models": 1, "l2": "flushed between timed steps (512 MiB write)",
                   "parallelism": f"replicas{world}"},
        "e2e": e2e, "gpu_launches": launches,
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "GFLOP/s",
                     "frac": achieved / peak, "traffic": None,
                     "kernel": "k_node_forward<JOINT> / k_node_adjoint<JOINT>",
                     "peak_source": "measured FP64 FMA probe (MEASURED_PEAKS.json has no FP64 "
                                    "entry)"},
        "clocks": clk,
    }


# ---------------------------------------------------------------------------
# CPU baselines (the oracle: the C restatement of the reference's algorithm)

class CachedProductsSample:
    """The reference's cached-sensitivity path on the host
    (FullSensitivityGravMagCalculator: d = J m, g = 2 J^T r per model, FP64)
    on the batched workload: the FP64 sensitivity rows of a station sample
    (32 of the 1024 stations, 320 rows x 131072 cells = 336 MB, more than a
    host's last-level cache) are built once, untimed; each sample then runs
    the products of as many models as fit in `budget_s`, spread over all
    host threads."""
    NST = 32

    def __init__(self):
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        from oracle import oracle as O
        from helpers import oracle_forward
        from jif3d_gb300 import workloads as W
        O.build()
        self.O = O
        self.s = s = W.config4()
        n = s.stations.shape[0]
        sub = s.subset(np.arange(self.NST) * (n // self.NST))
        _, J = oracle_forward(O, sub, want_sens=True)
        self.J = np.ascontiguousarray(J)
        self.r = np.random.default_rng(7).normal(size=self.J.shape[0])
        self.cores = os.cpu_count() or 1
        self.per_model_s = None

    def one(self, m):
        self.O.sens_matvec(self.J, m)
        self.O.sens_rmatvec2(self.J, self.r)

    def sample(self, budget_s):
        """Returns (Mcell*station*model/s, seconds, models) of one sample."""
        s = self.s
        if self.per_model_s is None:
            t0 = time.perf_counter()
            self.one(s.models[0])
            self.per_model_s = time.perf_counter() - t0
        nm = int(max(self.cores, min(4 * s.models.shape[0],
                                     budget_s * self.cores / max(self.per_model_s, 1e-4))))
        models = [s.models[i % s.models.shape[0]] for i in range(nm)]
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(max_workers=self.cores) as ex:
            list(ex.map(self.one, models))
        t = time.perf_counter() - t0
        return s.ngrid * self.NST * nm / t / 1e6, t, nm

    def describe(self, nm):
        n = self.s.stations.shape[0]
        return (f"cached-J products (J m and 2 J^T r, FP64) of {nm} models on {self.NST} of "
                f"{n} stations (J {self.J.nbytes / 1e6:.0f} MB, built once) x all "
                f"{self.s.ngrid} cells, models spread over {self.cores} threads")


class MatrixFreeSample:
    """The reference's OpenMP matrix-free forward + LQDerivative (one model,
    FP64) on the batched workload's survey, on a station sample sized to
    `budget_s`; all host threads."""

    def __init__(self):
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        from oracle import oracle as O
        from helpers import oracle_forward, oracle_lqderivative
        from jif3d_gb300 import workloads as W
        O.build()
        self.O, self.fwd, self.lqd = O, oracle_forward, oracle_lqderivative
        self.s = W.config4(nmodels=1)
        self.per_station_s = None
        self.cores = os.cpu_count() or 1

    def _run(self, k):
        n = self.s.stations.shape[0]
        sub = self.s.subset(np.arange(k) * max(1, n // k))
        t0 = time.perf_counter()
        d = self.fwd(self.O, sub)
        self.lqd(self.O, sub, np.ones(d.size))
        return time.perf_counter() - t0

    def sample(self, budget_s):
        if self.per_station_s is None:
            self.per_station_s = self._run(1)
        n = self.s.stations.shape[0]
        k = int(max(1, min(n, budget_s / max(self.per_station_s, 1e-3))))
        t = self._run(k)
        return self.s.ngrid * k / t / 1e6, t, k

    def describe(self, k):
        n = self.s.stations.shape[0]
        return (f"OpenMP matrix-free fwd+adjoint, {k} of {n} stations x all {self.s.ngrid} "
                f"cells, {self.cores} threads")


def run_reference(args, rank, world):
    """The reference arm: the oracle (the C restatement of the reference's
    implementation) on the host cores, on the same workload, metric and unit
    as our arm.  Each of the `--steps` steps is one bounded sample (about
    150 s / steps of host work, 2 to 10 s each), after up to three untimed
    warm-up samples of one second on the same sampler (thread pool, pages of
    the built rows)."""
    if rank != 0:
        return None
    sampler = CachedProductsSample() if args.workload == "batched" else MatrixFreeSample()
    budget = max(2.0, min(10.0, 150.0 / max(1, args.steps)))
    nwarm = min(args.warmup, 3)
    for _ in range(nwarm):
        sampler.sample(1.0)
    vals, secs, size = [], [], 0
    for _ in range(max(1, args.steps)):
        v, t, size = sampler.sample(budget)
        vals.append(v)
        secs.append(t)
    v = statistics.median(vals)
    full_units = 131072 * 1024 * (256 if args.workload == "batched" else 1) / 1e6
    return {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": len(vals),
        "warmup": nwarm, "ms_per_step": 1e3 * statistics.median(secs),
        "ms_per_full_step": 1e3 * full_units / v,
        "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": {"workload": "config4_batched_64x64x32_" +
                               ("f16x2_256models" if args.workload == "batched"
                                else "plain_fp64_joint"),
                   "cells": 131072, "stations": 1024,
                   "models": 256 if args.workload == "batched" else 1},
        "step": "one bounded sample of the workload on the host cores (ms_per_step is its "
                "time; ms_per_full_step the whole workload at the sample's rate)",
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": sampler.cores, "kind": "port",
                         "sample": sampler.describe(size)},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def reference_gpu_case(args):
    """The reference GPU forward (per-station kernels, row copies to the
    host, host inner products) on the first `--stations` stations of a
    workload, after one untimed station; prints a JSON line."""
    from oracle import refgpu
    from jif3d_gb300 import workloads as W
    if refgpu.build() is None:
        print(json.dumps({"unavailable": "reference CUDA sources not staged in baseline/_ref "
                                         "(staged by __graft_entry__.build() where the jif3D "
                                         "tree exists)"}))
        return
    s = W.CONFIGS[args.config]()
    tensor = args.config == 2
    n = min(args.stations, s.stations.shape[0])
    step = s.stations.shape[0] // n
    idx = np.arange(0, step * n, step)
    corner = [s.coords(a)[:-1] for a in range(3)]
    refgpu.run(*corner, s.xsize, s.ysize, s.zsize, s.stations[idx[:1]], s.model, tensor)
    data, _, t_loop, t_prep = refgpu.run(*corner, s.xsize, s.ysize, s.zsize, s.stations[idx],
                                         s.model, tensor)
    pairs = s.ngrid * n / 1e6
    print(json.dumps({"workload": s.name, "stations": n, "station_index": idx.tolist(),
                      "cells": s.ngrid, "forward_s": t_loop, "prepare_free_s": t_prep,
                      "forward": pairs / t_loop, "unit": UNIT,
                      "data": data.ravel().tolist()}))


def our_gridded(local, cfg, idx):
    """Our FP64 matrix-free gridded response (background values zero) at the
    stations `idx` of a workload, in the reference GPU layer's order: g_z, or
    Uxx Uxy Uxz Uyy Uyz Uzz."""
    from jif3d_gb300 import capi, workloads as W
    s = W.CONFIGS[cfg]()
    sub = s.subset(idx)
    ctx = capi.Context(local)
    W.setup_context(ctx, sub)
    m = s.model.copy()
    m[s.ngrid:] = 0.0
    d = ctx.forward(m)
    ctx.close()
    return d if cfg == 1 else d.reshape(-1, 9)[:, [0, 1, 2, 4, 5, 8]].ravel()


def measure_reference_gpu(local, ours):
    """The reference's own CUDA layer beside ours: its forward on the g_z
    workload (all 400 stations) and on the FTG workload (64 of 1600
    stations), each in a child process; throughput in Mcell*station/s and
    its data against our FP64 matrix-free data at the same stations."""
    out = {}
    for cfg, nst in ((1, 400), (2, 64)):
        env = dict(os.environ, CUDA_VISIBLE_DEVICES=os.environ.get("CUDA_VISIBLE_DEVICES",
                                                                   str(local)))
        r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--case",
                            "reference-gpu", "--config", str(cfg), "--stations", str(nst)],
                           capture_output=True, text=True, env=env, timeout=600)
        line = r.stdout.strip().splitlines()[-1] if r.stdout.strip() else ""
        try:
            res = json.loads(line)
        except ValueError:
            res = {"unavailable": f"reference GPU run failed (rc {r.returncode}): "
                                  f"{r.stderr.strip()[-300:]}"}
        if "data" in res and cfg in ours:
            got = np.array(res.pop("data"))
            ref = ours[cfg](np.array(res.pop("station_index")))
            res["rel_err_vs_ours"] = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
        res.pop("data", None)
        res.pop("station_index", None)
        out[f"config{cfg}"] = res
    out["how"] = ("jif3D Gravity/gravcuda.cu built unmodified for sm_103a (block size 128): one "
                  "kernel per station (six for FTG), each row copied to page-locked host memory "
                  "and multiplied by the densities on the host, as Scalar/TensorCudaGravityImp "
                  "do; forward only (the reference GPU path has no adjoint)")
    return out


def run_case(args):
    """One small, self-contained case of a kernel family (see the module
    docstring); it runs a few launches and prints one line."""
    if args.case == "reference-gpu":
        reference_gpu_case(args)
        return
    import torch
    from jif3d_gb300 import capi, workloads as W
    ctx = capi.Context(0)
    dev = "cuda:0"

    def thin(s, k):
        s.subsets = None
        step = max(1, s.stations.shape[0] // k)
        return s.subset(np.arange(0, s.stations.shape[0], step)[:k])

    if args.case == "node":
        s = thin(W.config4(nmodels=1) if args.config == 4 else W.CONFIGS[args.config](),
                 args.stations)
        W.setup_context(ctx, s)
        d = ctx.forward(s.model)
        g = ctx.lqderivative(s.model, np.ones(d.size))
        print("node case ok", s.name, s.stations.shape[0], "stations", float(d[0]), float(g[0]))
    elif args.case == "gemm":
        s = thin(W.config4(nmodels=args.models), args.stations)
        W.setup_context(ctx, s)
        ctx.build_sensitivity(capi.STORE_F16X2)
        d = ctx.batched_forward(s.models)
        g = ctx.batched_lqderivative(s.models, np.ones_like(d))
        print("gemm case ok", s.stations.shape[0], "stations", args.models, "models",
              float(d[0, 0]), float(g[0, 0]))
    elif args.case == "stream":
        s = thin(W.config2(), args.stations)
        W.setup_context(ctx, s)
        ctx.build_sensitivity(capi.STORE_FP32)
        n = s.stations.shape[0]
        dm = torch.tensor(s.model, dtype=torch.float64, device=dev)
        dd = torch.zeros(n * 9, dtype=torch.float64, device=dev)
        dg = torch.zeros(s.nparm, dtype=torch.float64, device=dev)
        ctx.stored_forward_device(dm.data_ptr(), dd.data_ptr())
        ctx.stored_lqderivative_device(dm.data_ptr(), dd.data_ptr(), dg.data_ptr())
        ctx.synchronize()
        print("stream case ok", n, "stations", float(dd[0]), float(dg[0]))
    elif args.case == "refine":
        s = W.config4(nmodels=args.models)
        half = [np.sort(np.concatenate([c, c[:-1] + 0.5 * np.diff(c)]))
                for c in (s.coords(0), s.coords(1), s.coords(2))]
        fine = [capi.refine_axis(s.coords(a), (s.xsize, s.ysize, s.zsize)[a], half[a])
                for a in range(3)]
        corner = [np.concatenate([[o], o + np.cumsum(f)[:-1]]) for o, f in zip(s.origin, fine)]
        ctx.set_mesh(corner[0], corner[1], corner[2], *fine)
        ctx.set_refinement(s.xsize, s.ysize, s.zsize)
        coarse = torch.tensor(s.models, dtype=torch.float64, device=dev)
        refined = torch.zeros((args.models, ctx.sizes()["nparm"]), dtype=torch.float64,
                              device=dev)
        back = torch.zeros_like(coarse)
        ctx.refine_project_device(args.models, coarse.data_ptr(), refined.data_ptr())
        ctx.refine_combine_device(args.models, refined.data_ptr(), back.data_ptr())
        ctx.synchronize()
        print("refine case ok", [f.size for f in fine], args.models, "models",
              float(back[0, 0]))
    elif args.case == "batched":
        s = W.config4(nmodels=args.models)
        W.setup_context(ctx, s)
        n = s.stations.shape[0]
        ctx.build_sensitivity(capi.STORE_F16X2)
        models = torch.tensor(s.models, dtype=torch.float64, device=dev)
        nmod = models.shape[0]
        data = torch.zeros((nmod, n * 10), dtype=torch.float64, device=dev)
        obs = torch.zeros(n * 10, dtype=torch.float64, device=dev)
        misfit = torch.zeros_like(data)
        grads = torch.zeros_like(models)
        for _ in range(args.steps):
            ctx.batched_forward_device(nmod, models.data_ptr(), data.data_ptr())
            torch.sub(data, obs, out=misfit)
            ctx.batched_lqderivative_device(nmod, models.data_ptr(), misfit.data_ptr(),
                                            grads.data_ptr())
        ctx.synchronize()
        print("batched case ok", n, "stations", nmod, "models", float(grads[0, 0]))
    ctx.close()


def main():
    args = parse()
    args.warmup = max(3, args.warmup)
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="nccl" if args.impl == "ours" else "gloo")
    if args.case:
        run_case(args)
        res = None
    elif args.impl == "reference":
        res = run_reference(args, rank, world)
    else:
        run = run_batched if args.workload == "batched" else run_plain
        res = run(args, rank, world, local)
        if rank == 0:
            smp = CachedProductsSample() if args.workload == "batched" else MatrixFreeSample()
            v, _, size = smp.sample(12.0)
            base = {"cpu_baseline": {"value": v, "unit": UNIT, "cores": smp.cores,
                                     "kind": "port", "sample": smp.describe(size)}}
            if args.workload == "batched" and args.sections == "all":
                mf = MatrixFreeSample()
                v2, _, k = mf.sample(10.0)
                base["cpu_baseline_matrix_free"] = {"value": v2, "unit": UNIT,
                                                    "cores": mf.cores, "sample": mf.describe(k)}
            # the CPU baselines go before the roofline, the speed-up and the
            # errors, which stay last in the line
            tail = {k: res.pop(k) for k in ("e2e", "roofline", "speedup_vs_plain_fp64",
                                            "err_vs_fp64") if k in res}
            res.update(base)
            res.update(tail)
    if rank == 0 and res is not None:
        print(json.dumps(res))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
