"""GPU paths at sizes where a kernel grid would pass the 65535-block limit of
its y dimension: batches of more than one product pass of models, station
sets whose blocks, rows or row chunks exceed 65535, and meshes whose cell
count exceeds 65535 product tiles of 128 rows.

Large station sets repeat a small set of distinct positions, so the
results are checked against the small set (whose own parity with the
oracle is tested elsewhere): tiled data, and gradients that are the copy
count times the small gradient.  Tolerances: FP64 path 1e-10, mixed path
1e-6 (relative norm error).
"""
import dataclasses

import numpy as np
import pytest

from helpers import oracle_forward, oracle_lqderivative, relerr, small_survey
from jif3d_gb300 import capi, workloads as W

pytestmark = pytest.mark.gpu
TOL64, TOL = 1e-10, 1e-6


def rowwise_max_relerr(x, ref):
    num = np.linalg.norm(np.asarray(x) - ref, axis=1)
    return float(np.max(num / np.linalg.norm(ref, axis=1)))


def tiled(s, copies):
    return dataclasses.replace(s, stations=np.tile(s.stations, (copies, 1)))


def test_batch_of_more_models_than_one_pass(ctx, oracle_lib):
    """32805 models: two passes of the batched products (32768 + 37)."""
    s = small_survey(W.SCALAR, seed=300, nx=4, ny=3, nz=2, nmeas=6)
    W.setup_context(ctx, s)
    ctx.build_sensitivity(capi.STORE_F16X2)
    d0, J = oracle_forward(oracle_lib, s, want_sens=True)
    assert relerr(J @ s.model, d0) <= 1e-12  # the scalar forward is J m
    rng = np.random.default_rng(5)
    nmod = 32768 + 37
    models = s.model[None, :] * (1 + 0.1 * rng.normal(size=(nmod, s.nparm)))
    assert rowwise_max_relerr(ctx.batched_forward(models), models @ J.T) <= TOL
    mis = rng.normal(size=(nmod, s.stations.shape[0]))
    assert relerr(oracle_lqderivative(oracle_lib, s, mis[0]), 2.0 * mis[0] @ J) <= 1e-12
    g = ctx.batched_lqderivative(models, mis)
    assert rowwise_max_relerr(g, 2.0 * mis @ J) <= TOL


def test_fp64_path_more_than_262140_stations(ctx):
    """270000 joint stations: more station blocks of the node forward than
    65535 at four stations per block."""
    s = small_survey(W.JOINT, seed=301, nx=3, ny=3, nz=2, nmeas=1000)
    copies = 270
    W.setup_context(ctx, s)
    d1 = ctx.forward(s.model)
    mis1 = np.random.default_rng(6).normal(size=d1.size)
    g1 = ctx.lqderivative(s.model, mis1)
    big = tiled(s, copies)
    W.setup_context(ctx, big)
    assert relerr(ctx.forward(big.model), np.tile(d1, copies)) <= TOL64
    assert relerr(ctx.lqderivative(big.model, np.tile(mis1, copies)), copies * g1) <= TOL64


@pytest.mark.parametrize("storage,copies", [(capi.STORE_F16X2, 2200), (capi.STORE_FP32, 8389)])
def test_stored_more_rows_than_grid_y(ctx, storage, copies):
    """2.2 million rows (the transposed fp16 copy has more than 65535 row
    blocks of 32) and 8.389 million rows (more than 65535 chunks of 128 rows
    in the FP32 transposed product)."""
    s = small_survey(W.SCALAR, seed=302, nx=3, ny=3, nz=2, nmeas=1000)
    W.setup_context(ctx, s)
    d1 = ctx.forward(s.model)
    mis1 = np.random.default_rng(7).normal(size=d1.size)
    g1 = ctx.lqderivative(s.model, mis1)
    big = tiled(s, copies)
    W.setup_context(ctx, big)
    ctx.build_sensitivity(storage)
    try:
        d = ctx.batched_forward(big.model[None, :])[0]
        assert relerr(d, np.tile(d1, copies)) <= TOL
        g = ctx.batched_lqderivative(big.model[None, :], np.tile(mis1, copies)[None, :])[0]
        assert relerr(g, copies * g1) <= TOL
    finally:
        ctx.drop_sensitivity()


def test_stored_adjoint_more_cells_than_grid_y(ctx):
    """256 x 256 x 129 cells (8.45 million): the adjoint product has more
    than 65535 tiles of 128 cells."""
    rng = np.random.default_rng(8)
    nx, ny, nz = 256, 256, 129
    st = np.array([[1280.0, 1280.0, -50.0], [300.0, 2000.0, -20.0]])
    s = W.Survey("big-mesh", np.full(nx, 10.0), np.full(ny, 10.0), np.full(nz, 10.0),
                 (0.0, 0.0, 0.0), st, W.SCALAR,
                 np.concatenate([rng.uniform(1, 11, nx * ny * nz), [2.0]]),
                 bg_thick=np.array([3000.0]))
    W.setup_context(ctx, s)
    d64 = ctx.forward(s.model)
    mis = np.array([0.7, -1.3])
    g64 = ctx.lqderivative(s.model, mis)
    ctx.build_sensitivity(capi.STORE_F16X2)
    try:
        assert relerr(ctx.batched_forward(s.model[None, :])[0], d64) <= TOL
        assert relerr(ctx.batched_lqderivative(s.model[None, :], mis[None, :])[0], g64) <= TOL
    finally:
        ctx.drop_sensitivity()
