"""Small, self-contained cases for profiling the kernels with ncu.

    python -m jif3d_gb300.profiling node [--stations 64] [--config 4]  # node-term fwd + adjoint
    python -m jif3d_gb300.profiling fp64-weights           # libm FP64 weight probes
    python -m jif3d_gb300.profiling gemm [--stations 128]  # tensor-core batched products
    python -m jif3d_gb300.profiling stream [--stations 400] # FP32 streaming products
    python -m jif3d_gb300.profiling batched [--steps 2]     # full config-4 batched steps
    python -m jif3d_gb300.profiling refine [--models 32]    # model refinement passes

Each case runs a few launches on a few-MB problem so that an ncu capture of
it ends by itself; ``batched`` runs the full 256-model config-4 step (7.5 GB of
stored J) for a launch list with one-pass metrics only.
"""
from __future__ import annotations

import argparse
import sys

import numpy as np


def case_node(stations: int, config: int = 4) -> None:
    """Node-term forward and adjoint of one model on a workload's mesh and
    kind (1 scalar, 2 tensor, 3 or 4 joint, 5 magnetic TFA) with every k-th
    station, `stations` of them."""
    from . import capi, workloads as W
    s = W.config4(nmodels=1) if config == 4 else W.CONFIGS[config]()
    s.subsets = None
    step = max(1, s.stations.shape[0] // stations)
    s = s.subset(np.arange(0, s.stations.shape[0], step)[:stations])
    ctx = capi.Context(0)
    W.setup_context(ctx, s)
    d = ctx.forward(s.model)
    g = ctx.lqderivative(s.model, np.ones(d.size))
    print("node case ok", s.stations.shape[0], "stations", float(d[0]), float(g[0]))
    ctx.close()


def case_gemm(stations: int, models: int) -> None:
    """Tensor-core batched products on the config-4 mesh with a station
    subset: one batched forward and one batched adjoint (~0.5 GB of J)."""
    from . import capi, workloads as W
    s = W.config4(nmodels=models)
    step = max(1, s.stations.shape[0] // stations)
    s = s.subset(np.arange(0, s.stations.shape[0], step)[:stations])
    ctx = capi.Context(0)
    W.setup_context(ctx, s)
    ctx.build_sensitivity(capi.STORE_F16X2)
    d = ctx.batched_forward(s.models)
    g = ctx.batched_lqderivative(s.models, np.ones_like(d))
    print("gemm case ok", s.stations.shape[0], "stations", models, "models", float(d[0, 0]),
          float(g[0, 0]))
    ctx.close()


def case_stream(stations: int) -> None:
    """FP32 streaming products on the config-2 mesh with a station subset."""
    import torch
    from . import capi, workloads as W
    s = W.config2()
    step = max(1, s.stations.shape[0] // stations)
    s = s.subset(np.arange(0, s.stations.shape[0], step)[:stations])
    ctx = capi.Context(0)
    W.setup_context(ctx, s)
    ctx.build_sensitivity(capi.STORE_FP32)
    n = s.stations.shape[0]
    dm = torch.tensor(s.model, dtype=torch.float64, device="cuda")
    dd = torch.zeros(n * 9, dtype=torch.float64, device="cuda")
    dg = torch.zeros(s.nparm, dtype=torch.float64, device="cuda")
    ctx.stored_forward_device(dm.data_ptr(), dd.data_ptr())
    ctx.stored_lqderivative_device(dm.data_ptr(), dd.data_ptr(), dg.data_ptr())
    ctx.synchronize()
    print("stream case ok", n, "stations", float(dd[0]), float(dg[0]))
    ctx.close()


def case_batched(steps: int) -> None:
    """The batched benchmark step on config 4 (256 models): batched forward,
    weighted misfit, batched adjoint, after the sensitivity build."""
    import torch
    from . import capi, workloads as W
    s = W.config4()
    ctx = capi.Context(0)
    W.setup_context(ctx, s)
    n = s.stations.shape[0]
    ctx.build_sensitivity(capi.STORE_F16X2)
    models = torch.tensor(s.models, dtype=torch.float64, device="cuda")
    nmod = models.shape[0]
    data = torch.zeros((nmod, n * 10), dtype=torch.float64, device="cuda")
    obs = torch.zeros(n * 10, dtype=torch.float64, device="cuda")
    grads = torch.zeros_like(models)
    for _ in range(steps):
        ctx.batched_forward_device(nmod, models.data_ptr(), data.data_ptr())
        misfit = (data - obs).contiguous()
        ctx.batched_lqderivative_device(nmod, models.data_ptr(), misfit.data_ptr(),
                                        grads.data_ptr())
    ctx.synchronize()
    print("batched case ok", n, "stations", nmod, "models", float(grads[0, 0]))
    ctx.close()


def case_refine(models: int) -> None:
    """Projection and combination between the config-4 grid (coarse) and a
    grid refined 2 x 2 x 2 (128 x 128 x 64), for ``models`` models: one launch
    of each (32 models: 268 MB of refined values, larger than L2)."""
    import torch
    from . import capi, workloads as W
    s = W.config4(nmodels=models)
    half = [np.sort(np.concatenate([c, c[:-1] + 0.5 * np.diff(c)]))
            for c in (s.coords(0), s.coords(1), s.coords(2))]
    fine = [capi.refine_axis(s.coords(a), (s.xsize, s.ysize, s.zsize)[a], half[a])
            for a in range(3)]
    ctx = capi.Context(0)
    corner = [np.concatenate([[o], o + np.cumsum(f)[:-1]]) for o, f in zip(s.origin, fine)]
    ctx.set_mesh(corner[0], corner[1], corner[2], *fine)
    ctx.set_refinement(s.xsize, s.ysize, s.zsize)
    coarse = torch.tensor(s.models, dtype=torch.float64, device="cuda")
    refined = torch.zeros((models, ctx.sizes()["nparm"]), dtype=torch.float64, device="cuda")
    back = torch.zeros_like(coarse)
    ctx.refine_project_device(models, coarse.data_ptr(), refined.data_ptr())
    ctx.refine_combine_device(models, refined.data_ptr(), back.data_ptr())
    ctx.synchronize()
    print("refine case ok", [f.size for f in fine], models, "models", float(back[0, 0]))
    ctx.close()


def case_fp64_weights(n_iter: int) -> None:
    from . import capi
    lib = capi.load()
    rc = lib.j3g_probe_math(0, n_iter)
    if rc != 0:
        raise SystemExit(f"probe failed: {rc}")
    print("fp64 weight probes ok")


def main(argv=None) -> None:
    p = argparse.ArgumentParser()
    sub = p.add_subparsers(dest="case", required=True)
    n = sub.add_parser("node")
    n.add_argument("--stations", type=int, default=64)
    n.add_argument("--config", type=int, default=4, choices=[1, 2, 3, 4, 5])
    w = sub.add_parser("fp64-weights")
    w.add_argument("--iters", type=int, default=1000)
    g = sub.add_parser("gemm")
    g.add_argument("--stations", type=int, default=128)
    g.add_argument("--models", type=int, default=256)
    st = sub.add_parser("stream")
    st.add_argument("--stations", type=int, default=400)
    b = sub.add_parser("batched")
    b.add_argument("--steps", type=int, default=2)
    r = sub.add_parser("refine")
    r.add_argument("--models", type=int, default=32)
    a = p.parse_args(argv)
    if a.case == "node":
        case_node(a.stations, a.config)
    elif a.case == "gemm":
        case_gemm(a.stations, a.models)
    elif a.case == "stream":
        case_stream(a.stations)
    elif a.case == "batched":
        case_batched(a.steps)
    elif a.case == "refine":
        case_refine(a.models)
    elif a.case == "fp64-weights":
        case_fp64_weights(a.iters)


if __name__ == "__main__":
    main(sys.argv[1:])
