"""Small, self-contained cases for profiling the kernels with ncu.

    python -m jif3d_gb300.profiling node [--stations 64]   # node-term fwd + adjoint
    python -m jif3d_gb300.profiling fp64-weights           # libm FP64 weight probes

Each case runs a few launches on a few-MB problem so that an ncu capture of
it ends by itself.
"""
from __future__ import annotations

import argparse
import sys

import numpy as np


def case_node(stations: int) -> None:
    from . import capi, workloads as W
    s = W.config4(nmodels=1)
    step = max(1, s.stations.shape[0] // stations)
    s = s.subset(np.arange(0, s.stations.shape[0], step)[:stations])
    ctx = capi.Context(0)
    W.setup_context(ctx, s)
    d = ctx.forward(s.model)
    g = ctx.lqderivative(s.model, np.ones(d.size))
    print("node case ok", s.stations.shape[0], "stations", float(d[0]), float(g[0]))
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
    w = sub.add_parser("fp64-weights")
    w.add_argument("--iters", type=int, default=1000)
    a = p.parse_args(argv)
    if a.case == "node":
        case_node(a.stations)
    elif a.case == "fp64-weights":
        case_fp64_weights(a.iters)


if __name__ == "__main__":
    main(sys.argv[1:])
