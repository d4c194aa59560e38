"""GPU parity of the stored-sensitivity (mixed precision) paths.

Tolerance (mixed path): relative norm error <= 1e-6 per output group against
the FP64 oracle, the bound stated for the mixed-precision path.  J is stored
in FP32 (streaming products) or as fp16 hi + lo with a power-of-two row
scale (tensor-core products); the FP64 matrix-free path serves as the
reference at full sizes (its own parity with the oracle is <= 1e-10).
"""
import numpy as np
import pytest

from helpers import oracle_forward, oracle_lqderivative, relerr, small_survey
from jif3d_gb300 import capi, workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-6


def groups(s, v):
    """Split a data vector into the output groups of its kind (joint: g_z, tensor)."""
    v = np.asarray(v)
    if s.kind == W.JOINT and s.transform == W.T_NONE:
        r = v.reshape(-1, 10)
        return [r[:, 0], r[:, 1:]]
    return [v]


def check_groups(s, got, ref, tol=TOL):
    for g, r in zip(groups(s, got), groups(s, ref)):
        e = relerr(g, r)
        assert e <= tol, e


def dev(a):
    import torch
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


@pytest.mark.parametrize("storage", [capi.STORE_FP32, capi.STORE_F16X2])
@pytest.mark.parametrize("kind", [W.SCALAR, W.TENSOR, W.MAGNETIC, W.JOINT])
def test_stored_single_model(ctx, oracle_lib, storage, kind):
    import torch
    s = small_survey(kind, seed=200 + kind, nx=9, ny=8, nz=6, nmeas=12)
    W.setup_context(ctx, s)
    ctx.build_sensitivity(storage)
    info = ctx.sensitivity_info()
    assert info["storage"] == storage and info["cols"] == s.ngrid
    n = s.stations.shape[0]
    d = torch.zeros(n * s.dpm, dtype=torch.float64, device="cuda")
    ctx.stored_forward_device(dev(s.model).data_ptr(), d.data_ptr())
    ctx.synchronize()
    check_groups(s, d.cpu().numpy(), oracle_forward(oracle_lib, s))
    misfit = np.random.default_rng(kind).normal(size=n * s.dpm)
    g = torch.zeros(s.nparm, dtype=torch.float64, device="cuda")
    dm, dr = dev(s.model), dev(misfit)
    ctx.stored_lqderivative_device(dm.data_ptr(), dr.data_ptr(), g.data_ptr())
    ctx.synchronize()
    gref = oracle_lqderivative(oracle_lib, s, misfit)
    assert relerr(g.cpu().numpy(), gref) <= TOL


@pytest.mark.parametrize("kind,transform", [(W.TENSOR, W.T_FTG_INVARIANT),
                                            (W.MAGNETIC, W.T_TOTAL_FIELD),
                                            (W.MAGNETIC, W.T_TFA)])
def test_batched_transforms(ctx, oracle_lib, kind, transform):
    s = small_survey(kind, seed=230 + transform, transform=transform, nx=8, ny=7, nz=5)
    W.setup_context(ctx, s)
    ctx.build_sensitivity(capi.STORE_F16X2)
    rng = np.random.default_rng(3)
    models = s.model[None, :] * (1 + 0.1 * rng.normal(size=(3, s.nparm)))
    d = ctx.batched_forward(models)
    n = s.stations.shape[0]
    mis = rng.normal(size=(3, n))
    g = ctx.batched_lqderivative(models, mis)
    for i in range(3):
        assert relerr(d[i], oracle_forward(oracle_lib, s, models[i])) <= TOL
        assert relerr(g[i], oracle_lqderivative(oracle_lib, s, mis[i], models[i])) <= TOL


@pytest.mark.parametrize("nmodels", [1, 5, 70, 130])
def test_batched_joint_many_models(ctx, oracle_lib, nmodels):
    """Batched products for N-tile sizes 64 / 128 / 256 against the oracle on
    a few models and against the single-model stored product on all."""
    import torch
    s = small_survey(W.JOINT, seed=250, nx=12, ny=10, nz=7, nmeas=15)
    W.setup_context(ctx, s)
    ctx.build_sensitivity(capi.STORE_F16X2)
    rng = np.random.default_rng(nmodels)
    models = s.model[None, :] + 2.0 * rng.normal(size=(nmodels, s.nparm))
    n = s.stations.shape[0]
    d = ctx.batched_forward(models)
    mis = rng.normal(size=(nmodels, n * 10))
    g = ctx.batched_lqderivative(models, mis)
    for i in sorted({0, nmodels // 2, nmodels - 1}):
        check_groups(s, d[i], oracle_forward(oracle_lib, s, models[i]))
        assert relerr(g[i], oracle_lqderivative(oracle_lib, s, mis[i], models[i])) <= TOL


def test_batched_host_pinned_outputs(ctx):
    """The host-buffer batched calls write into caller arrays in pinned memory
    (what an inversion loop reuses each iteration) with the same result as
    into fresh pageable arrays; a wrong output array is an argument error."""
    import torch
    s = small_survey(W.JOINT, seed=260, nx=10, ny=8, nz=6, nmeas=14)
    W.setup_context(ctx, s)
    ctx.build_sensitivity(capi.STORE_F16X2)
    rng = np.random.default_rng(9)
    models = s.model[None, :] + rng.normal(size=(4, s.nparm))
    n = s.stations.shape[0]

    def pinned(shape):
        return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    mh, dh, rh, gh = pinned(models.shape), pinned((4, n * 10)), pinned((4, n * 10)), \
        pinned(models.shape)
    mh[...] = models
    rh[...] = rng.normal(size=rh.shape)
    assert ctx.batched_forward(mh, out=dh) is dh
    assert ctx.batched_lqderivative(mh, rh, out=gh) is gh
    assert np.array_equal(dh, ctx.batched_forward(models))
    assert np.array_equal(gh, ctx.batched_lqderivative(models, np.array(rh)))
    with pytest.raises(capi.J3GError):
        ctx.batched_forward(mh, out=np.zeros((4, n * 10), dtype=np.float32))
    with pytest.raises(capi.J3GError):
        ctx.batched_lqderivative(mh, rh, out=np.zeros((3, s.nparm)))
    # the linear derivative does not read the models
    assert np.array_equal(ctx.batched_lqderivative(None, rh), gh)
    t = small_survey(W.TENSOR, seed=261, transform=W.T_FTG_INVARIANT, nx=6, ny=5, nz=4)
    W.setup_context(ctx, t)
    ctx.build_sensitivity(capi.STORE_F16X2)
    with pytest.raises(capi.J3GError):  # the invariant's derivative needs the data
        ctx.batched_lqderivative(None, np.zeros((2, t.stations.shape[0])))


@pytest.mark.parametrize("kind,transform", [(W.JOINT, W.T_NONE), (W.TENSOR, W.T_FTG_INVARIANT)])
def test_pipelined_batched_calls(ctx, kind, transform):
    """The pipelined host-buffer calls give, bit for bit, what the blocking
    calls give: five forwards in flight (the ring holds four), waits out of
    order, derivatives with and without the models (the FTG invariant needs
    them), page-locked and pageable buffers."""
    import torch
    s = small_survey(kind, seed=270 + transform, transform=transform, nx=9, ny=8, nz=6,
                     nmeas=12)
    W.setup_context(ctx, s)
    ctx.build_sensitivity(capi.STORE_F16X2)
    rng = np.random.default_rng(11)
    n = s.stations.shape[0]
    nd = n * s.dpm

    def pinned(shape):
        return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    batches = [s.model[None, :] * rng.uniform(0.5, 1.5, (3, s.nparm)) for _ in range(5)]
    outs = [pinned((3, nd)) for _ in batches]
    tickets = [ctx.batched_forward_async(b, out=o) for b, o in zip(batches, outs)]
    for t in reversed(tickets):
        ctx.batched_wait(t)
    for b, o in zip(batches, outs):
        assert np.array_equal(o, ctx.batched_forward(b))
    mis = [rng.normal(size=(3, nd)) for _ in batches]
    grads = [np.zeros((3, s.nparm)) for _ in batches]  # pageable
    models = [b if transform != W.T_NONE else None for b in batches]
    tickets = [ctx.batched_lqderivative_async(m, r, out=g)
               for m, r, g in zip(models, mis, grads)]
    t_fwd = ctx.batched_forward_async(batches[0], out=outs[0])
    ctx.batched_wait(tickets[1])
    ctx.batched_wait(t_fwd)
    ctx.batched_wait(tickets[3])
    ctx.batched_wait(tickets[4])
    ctx.batched_wait(tickets[0])  # its slot was reused: already complete
    for b, r, g in zip(batches, mis, grads):
        assert np.array_equal(g, ctx.batched_lqderivative(b, r))
    with pytest.raises(capi.J3GError):
        ctx.batched_wait(10 ** 9)


def test_pipelined_calls_replay_graphs(ctx):
    """Pipelined calls replay their products from per-slot CUDA graphs once a
    shape is warm.  Many calls per slot (eager, captured, replayed), then a
    pinned plan, another model count and a new geometry -- each of which
    must retire the graphs -- all give, bit for bit, what the blocking calls
    give."""
    import torch

    def pinned(shape):
        return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()

    def run(s, models, mis, ncalls=10):
        nd = mis.shape[1]
        outs = [pinned((models.shape[0], nd)) for _ in range(ncalls)]
        grads = [pinned(models.shape) for _ in range(ncalls)]
        tf = [ctx.batched_forward_async(models * (1 + 0.01 * k), out=outs[k])
              for k in range(ncalls)]
        for t in tf:
            ctx.batched_wait(t)
        ta = [ctx.batched_lqderivative_async(None, mis * (k + 1), out=grads[k])
              for k in range(ncalls)]
        for t in ta:
            ctx.batched_wait(t)
        for k in range(ncalls):
            assert np.array_equal(outs[k], ctx.batched_forward(models * (1 + 0.01 * k)))
            assert np.array_equal(grads[k], ctx.batched_lqderivative(models, mis * (k + 1)))

    rng = np.random.default_rng(31)
    s = small_survey(W.JOINT, seed=291, nx=12, ny=10, nz=8, nmeas=30)
    W.setup_context(ctx, s)
    ctx.build_sensitivity(capi.STORE_F16X2)
    models = s.model[None, :] * rng.uniform(0.5, 1.5, (260, s.nparm))
    mis = rng.normal(size=(260, s.stations.shape[0] * 10))
    run(s, models, mis)
    try:
        ctx.set_gemm_plan(0, 6, 256)
        ctx.set_gemm_plan(1, 3, 128)
        run(s, models, mis)
    finally:
        ctx.set_gemm_plan(0, 0)
        ctx.set_gemm_plan(1, 0)
    run(s, models[:70], mis[:70])
    s2 = small_survey(W.TENSOR, seed=292, nx=9, ny=11, nz=7, nmeas=25)
    W.setup_context(ctx, s2)
    ctx.build_sensitivity(capi.STORE_F16X2)
    m2 = s2.model[None, :] * rng.uniform(0.5, 1.5, (200, s2.nparm))
    run(s2, m2, rng.normal(size=(200, s2.stations.shape[0] * 9)))


@pytest.mark.parametrize("transform", [W.T_NONE, W.T_FTG_INVARIANT])
def test_pipelined_step_loop(ctx, transform):
    """The inversion-step loop over pipelined calls -- each forward queued two
    steps ahead, the misfit formed on the host from the step's data, its
    derivative queued, the gradient of two steps back waited for, three
    sets of page-locked buffers -- gives every step's data and gradient bit
    for bit as the blocking calls do.  A forward's data and a derivative's
    misfits travel on copy streams of their own direction while the other
    direction's copies are in flight."""
    import torch
    kind = W.JOINT if transform == W.T_NONE else W.TENSOR
    s = small_survey(kind, seed=296 + transform, transform=transform, nx=12, ny=10, nz=8,
                     nmeas=30)
    W.setup_context(ctx, s)
    ctx.build_sensitivity(capi.STORE_F16X2)
    rng = np.random.default_rng(37)
    nmod, nd, nsteps = 40, s.stations.shape[0] * s.dpm, 9
    batches = [s.model[None, :] * rng.uniform(0.5, 1.5, (nmod, s.nparm)) for _ in range(nsteps)]
    obs = rng.normal(size=nd) * 1e-5
    w = rng.uniform(0.5, 2.0, size=nd)

    def pinned(shape):
        return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    # each step's models stay as they are until its derivative is waited for
    # (the FTG invariant's derivative reads them): one page-locked array each
    models = [pinned((nmod, s.nparm)) for _ in range(nsteps)]
    for m, b in zip(models, batches):
        m[:] = b
    sets = [dict(data=pinned((nmod, nd)), mis=pinned((nmod, nd)), grads=pinned((nmod, s.nparm)))
            for _ in range(3)]
    got_data, got_grads, mis_of = {}, {}, {}
    fwd, adj = {}, {}

    def queue_fwd(i):
        fwd[i] = ctx.batched_forward_async(models[i], out=sets[i % 3]["data"])

    def take_grad(i):
        ctx.batched_wait(adj[i])
        got_grads[i] = sets[i % 3]["grads"].copy()
    for i in range(2):
        queue_fwd(i)
    for i in range(nsteps):
        st = sets[i % 3]
        ctx.batched_wait(fwd[i])
        got_data[i] = st["data"].copy()
        np.multiply(st["data"] - obs, w, out=st["mis"])
        mis_of[i] = st["mis"].copy()
        adj[i] = ctx.batched_lqderivative_async(models[i], st["mis"], out=st["grads"])
        if i + 2 < nsteps:
            queue_fwd(i + 2)
        if i >= 2:
            take_grad(i - 2)
    for i in range(nsteps - 2, nsteps):
        take_grad(i)
    for i in range(nsteps):
        assert np.array_equal(got_data[i], ctx.batched_forward(batches[i])), i
        assert np.array_equal(got_grads[i], ctx.batched_lqderivative(batches[i], mis_of[i])), i


def test_pinned_gemm_plans(ctx, oracle_lib):
    """Pinned plans (j3g_set_gemm_plan) are used as given -- the CTA pair with
    many K splits, one-SM 128-wide tiles -- and agree with the oracle; a tile
    the batch does not fill falls back to the automatic plan; unpinning
    restores the fixed rule."""
    s = small_survey(W.JOINT, seed=290, nx=16, ny=14, nz=10, nmeas=40)
    W.setup_context(ctx, s)
    ctx.build_sensitivity(capi.STORE_F16X2)
    rng = np.random.default_rng(29)
    models = s.model[None, :] + 2.0 * rng.normal(size=(300, s.nparm))
    mis = rng.normal(size=(300, s.stations.shape[0] * 10))
    try:
        for plan_f, plan_a in (((50, 256), (5, 256)), ((8, 128), (3, 128))):
            ctx.set_gemm_plan(0, *plan_f)
            ctx.set_gemm_plan(1, *plan_a)
            d = ctx.batched_forward(models)
            g = ctx.batched_lqderivative(models, mis)
            assert ctx.gemm_plan(0) == dict(nsplit=plan_f[0], tile=plan_f[1], tuned_ms=0.0)
            assert ctx.gemm_plan(1) == dict(nsplit=plan_a[0], tile=plan_a[1], tuned_ms=0.0)
            for i in (0, 299):
                check_groups(s, d[i], oracle_forward(oracle_lib, s, models[i]))
                assert relerr(g[i], oracle_lqderivative(oracle_lib, s, mis[i], models[i])) <= TOL
        ctx.set_gemm_plan(0, 4, 256)
        ctx.batched_forward(models[:10])  # 10 models: the 256 tile does not fit
        assert ctx.gemm_plan(0)["tile"] == 64
    finally:
        ctx.set_gemm_plan(0, 0)
        ctx.set_gemm_plan(1, 0)
    ctx.batched_forward(models)
    assert ctx.gemm_plan(0)["nsplit"] != 50
    with pytest.raises(capi.J3GError):
        ctx.set_gemm_plan(0, 4, 96)


def test_models_split_over_pinned_splits(ctx, oracle_lib):
    """Plans pinned to one K split (4320 cells, 68 k-blocks in one block of
    the models' split) and to three: each split's scale and the split sums
    follow the plan, and the products match the oracle."""
    s = small_survey(W.JOINT, seed=310, nx=20, ny=18, nz=12, nmeas=24)
    W.setup_context(ctx, s)
    ctx.build_sensitivity(capi.STORE_F16X2)
    rng = np.random.default_rng(31)
    models = s.model[None, :] * (1 + 0.1 * rng.normal(size=(260, s.nparm)))
    mis = rng.normal(size=(260, s.stations.shape[0] * 10))
    try:
        for nsplit in (1, 3):
            ctx.set_gemm_plan(0, nsplit, 0)
            d = ctx.batched_forward(models)
            g = ctx.batched_lqderivative(models, mis)
            for i in (0, 259):
                check_groups(s, d[i], oracle_forward(oracle_lib, s, models[i]))
                assert relerr(g[i], oracle_lqderivative(oracle_lib, s, mis[i], models[i])) <= TOL
    finally:
        ctx.set_gemm_plan(0, 0)


def test_models_with_uneven_magnitudes(ctx, oracle_lib):
    """Models whose K splits differ in magnitude by many binades (a near-zero
    region, a large uniform part, one cell far above the rest): each split
    takes its own scale where the row's sampled one does not bound it, and
    the split sums bring them together exactly.  A value beyond the float
    range takes the split's FP64 form; a NaN reaches every datum."""
    s = small_survey(W.JOINT, seed=311, nx=24, ny=20, nz=10, nmeas=20)
    W.setup_context(ctx, s)
    ctx.build_sensitivity(capi.STORE_F16X2)
    rng = np.random.default_rng(32)
    ng = s.ngrid
    models = np.tile(s.model, (8, 1))
    models[0, :ng // 2] *= 1e-9                       # half the cells near zero
    models[1, :ng] += 1e6                             # a large uniform part
    models[2, 40] = 1e7                               # one outlier cell, not sampled
    models[3, :ng] = rng.normal(size=ng) * np.logspace(-6, 6, ng)
    models[4, :ng] = -models[4, :ng]
    models[5, :ng] = 0.0                              # background only
    models[6, 40] = 1e39                              # beyond the float range: FP64 split
    models[7, 40] = np.nan                            # propagates to every datum
    mis = rng.normal(size=(8, s.stations.shape[0] * 10))
    d = ctx.batched_forward(models)
    g = ctx.batched_lqderivative(models, mis)
    for i in range(7):
        check_groups(s, d[i], oracle_forward(oracle_lib, s, models[i]))
        assert relerr(g[i], oracle_lqderivative(oracle_lib, s, mis[i], models[i])) <= TOL
    assert np.isnan(d[7]).all()


def test_batched_adjoint_long_residual_rows(ctx, oracle_lib):
    """More than 2340 joint stations (16800 stored rows): the residual weights
    take the separate weights launch and the three-pass split of long rows."""
    s = small_survey(W.JOINT, seed=312, nx=9, ny=8, nz=6, nmeas=2400)
    W.setup_context(ctx, s)
    ctx.build_sensitivity(capi.STORE_F16X2)
    rng = np.random.default_rng(33)
    models = s.model[None, :] * (1 + 0.1 * rng.normal(size=(3, s.nparm)))
    mis = rng.normal(size=(3, s.stations.shape[0] * 10))
    g = ctx.batched_lqderivative(models, mis)
    d = ctx.batched_forward(models)
    for i in range(3):
        check_groups(s, d[i], oracle_forward(oracle_lib, s, models[i]))
        assert relerr(g[i], oracle_lqderivative(oracle_lib, s, mis[i], models[i])) <= TOL


def test_stored_is_dropped_on_new_geometry(ctx):
    s = small_survey(W.SCALAR, seed=5)
    W.setup_context(ctx, s)
    ctx.build_sensitivity(capi.STORE_FP32)
    assert ctx.sensitivity_info()["storage"] == capi.STORE_FP32
    ctx.set_stations(s.stations[:, 0] + 1.0, s.stations[:, 1], s.stations[:, 2])
    assert ctx.sensitivity_info()["storage"] == 0
    with pytest.raises(capi.J3GError):
        ctx.batched_forward(s.model[None, :])


def test_config2_fp32_stored_full(ctx):
    """Config 2 at full size (FP32 J, 5 GB): stored forward and adjoint
    against the FP64 matrix-free path."""
    import torch
    s = W.config2()
    W.setup_context(ctx, s)
    n = s.stations.shape[0]
    dm = dev(s.model)
    ref = torch.zeros(n * 9, dtype=torch.float64, device="cuda")
    ctx.forward_device(dm.data_ptr(), ref.data_ptr())
    mis = dev(np.random.default_rng(2).normal(size=n * 9))
    gref = torch.zeros(s.nparm, dtype=torch.float64, device="cuda")
    ctx.lqderivative_device(dm.data_ptr(), mis.data_ptr(), gref.data_ptr())
    ctx.synchronize()
    ctx.build_sensitivity(capi.STORE_FP32)
    d = torch.zeros_like(ref)
    g = torch.zeros_like(gref)
    ctx.stored_forward_device(dm.data_ptr(), d.data_ptr())
    ctx.stored_lqderivative_device(dm.data_ptr(), mis.data_ptr(), g.data_ptr())
    ctx.synchronize()
    assert relerr(d.cpu().numpy(), ref.cpu().numpy()) <= TOL
    assert relerr(g.cpu().numpy(), gref.cpu().numpy()) <= TOL
    ctx.drop_sensitivity()


def test_config4_batched_full(ctx, oracle_lib):
    """Config 4 at full size: 256 models through the tensor-core products;
    four of them checked against the FP64 matrix-free path, one station
    subset against the oracle."""
    import torch
    s = W.config4()
    W.setup_context(ctx, s)
    n = s.stations.shape[0]
    ctx.build_sensitivity(capi.STORE_F16X2)
    models = dev(s.models)
    data = torch.zeros((256, n * 10), dtype=torch.float64, device="cuda")
    ctx.batched_forward_device(256, models.data_ptr(), data.data_ptr())
    rng = np.random.default_rng(4)
    mis_h = rng.normal(size=(256, n * 10)) * np.tile([1e8] + [1e9] * 9, n)
    mis = dev(mis_h)
    grads = torch.zeros_like(models)
    ctx.batched_lqderivative_device(256, models.data_ptr(), mis.data_ptr(), grads.data_ptr())
    ctx.synchronize()
    data_h, grads_h = data.cpu().numpy(), grads.cpu().numpy()
    ctx.drop_sensitivity()
    for i in (0, 77, 255):
        ref = torch.zeros(n * 10, dtype=torch.float64, device="cuda")
        gref = torch.zeros(s.nparm, dtype=torch.float64, device="cuda")
        ctx.forward_device(models[i].data_ptr(), ref.data_ptr())
        ctx.lqderivative_device(models[i].data_ptr(), mis[i].contiguous().data_ptr(),
                                gref.data_ptr())
        ctx.synchronize()
        check_groups(s, data_h[i], ref.cpu().numpy())
        assert relerr(grads_h[i], gref.cpu().numpy()) <= TOL
    sub = s.subset(np.arange(0, n, 128))
    idx = np.arange(0, n, 128)
    dsub = data_h[5].reshape(n, 10)[idx].ravel()
    check_groups(sub, dsub, oracle_forward(oracle_lib, sub, s.models[5]))


def test_config4_all_models_on_station_subset(oracle_lib):
    """Config 4 at full size, every one of the 256 models checked: the
    batched data of 128 stations (every eighth) against the FP64 matrix-free
    forward of those stations, and the batched gradients of misfits that are
    non-zero on those stations only against the FP64 matrix-free gradient of
    the same misfits; g_z, tensor and gradient groups each <= 1e-6."""
    import torch
    s = W.config4()
    n = s.stations.shape[0]
    idx = np.arange(0, n, 8)
    sub = s.subset(idx)
    big, small = capi.Context(0), capi.Context(0)
    try:
        W.setup_context(big, s)
        big.build_sensitivity(capi.STORE_F16X2)
        models = dev(s.models)
        data = torch.zeros((256, n * 10), dtype=torch.float64, device="cuda")
        big.batched_forward_device(256, models.data_ptr(), data.data_ptr())
        rng = np.random.default_rng(41)
        mis_sub = rng.normal(size=(256, idx.size, 10)) * np.array([1e8] + [1e9] * 9)
        mis_h = np.zeros((256, n, 10))
        mis_h[:, idx, :] = mis_sub
        mis = dev(mis_h.reshape(256, n * 10))
        grads = torch.zeros_like(models)
        big.batched_lqderivative_device(256, models.data_ptr(), mis.data_ptr(), grads.data_ptr())
        big.synchronize()
        data_h = data.cpu().numpy().reshape(256, n, 10)[:, idx, :].reshape(256, -1)
        grads_h = grads.cpu().numpy()
        W.setup_context(small, sub)
        ref = torch.zeros(idx.size * 10, dtype=torch.float64, device="cuda")
        gref = torch.zeros(s.nparm, dtype=torch.float64, device="cuda")
        ms = dev(mis_sub.reshape(256, -1))
        worst = [0.0, 0.0, 0.0]
        for i in range(256):
            small.forward_device(models[i].data_ptr(), ref.data_ptr())
            small.lqderivative_device(models[i].data_ptr(), ms[i].data_ptr(), gref.data_ptr())
            small.synchronize()
            r = ref.cpu().numpy().reshape(-1, 10)
            got = data_h[i].reshape(-1, 10)
            e = [relerr(got[:, 0], r[:, 0]), relerr(got[:, 1:], r[:, 1:]),
                 relerr(grads_h[i], gref.cpu().numpy())]
            worst = [max(a, b) for a, b in zip(worst, e)]
        assert max(worst) <= TOL, worst
    finally:
        big.close()
        small.close()


def test_batched_step_captured_in_cuda_graph(ctx, oracle_lib):
    """One batched step (forward, weighted misfit, adjoint) captured in a CUDA
    graph after a warm-up call and replayed on new models written in place:
    the same results as the eager calls, and against the oracle."""
    import torch
    s = small_survey(W.JOINT, seed=270, nx=12, ny=10, nz=7, nmeas=15)
    W.setup_context(ctx, s)
    ctx.build_sensitivity(capi.STORE_F16X2)
    n, nmod = s.stations.shape[0], 300
    rng = np.random.default_rng(9)
    base = s.model[None, :] + 2.0 * rng.normal(size=(nmod, s.nparm))
    obs = dev(oracle_forward(oracle_lib, s))
    w = dev(rng.uniform(0.5, 2.0, n * 10))
    models = dev(base)
    data = torch.zeros((nmod, n * 10), dtype=torch.float64, device="cuda")
    misfit = torch.zeros_like(data)
    grads = torch.zeros_like(models)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)

    def step():
        ctx.batched_forward_device(nmod, models.data_ptr(), data.data_ptr())
        torch.mul(torch.sub(data, obs, out=misfit), w, out=misfit)
        ctx.batched_lqderivative_device(nmod, models.data_ptr(), misfit.data_ptr(),
                                        grads.data_ptr())

    with torch.cuda.stream(stream):
        step()  # warm-up: every buffer of the step is allocated here
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        step()
    new = base * (1 + 0.1 * rng.normal(size=base.shape))
    models.copy_(dev(new))
    graph.replay()
    torch.cuda.synchronize()
    d_graph, g_graph = data.cpu().numpy(), grads.cpu().numpy()
    with torch.cuda.stream(stream):
        step()  # eager, same models
    torch.cuda.synchronize()
    ctx.set_stream(None)
    assert np.array_equal(d_graph, data.cpu().numpy())
    assert np.array_equal(g_graph, grads.cpu().numpy())
    for i in (0, nmod - 1):
        check_groups(s, d_graph[i], oracle_forward(oracle_lib, s, new[i]))
        mis = (d_graph[i] - obs.cpu().numpy()) * w.cpu().numpy()
        assert relerr(g_graph[i], oracle_lqderivative(oracle_lib, s, mis, new[i])) <= TOL


def test_autotuned_products(ctx, oracle_lib):
    """Autotuned tensor-core plans: results within the mixed tolerance, the
    plan keeps at most 128 k-blocks per split, and the cached plan is reused
    (same plan, bit-identical results on the second call)."""
    s = small_survey(W.JOINT, seed=280, nx=16, ny=14, nz=10, nmeas=40)
    W.setup_context(ctx, s)
    ctx.build_sensitivity(capi.STORE_F16X2)
    ctx.set_autotune(True)
    try:
        rng = np.random.default_rng(28)
        models = s.model[None, :] + 2.0 * rng.normal(size=(300, s.nparm))
        mis = rng.normal(size=(300, s.stations.shape[0] * 10))
        d1 = ctx.batched_forward(models)
        g1 = ctx.batched_lqderivative(models, mis)
        plans = [ctx.gemm_plan(0), ctx.gemm_plan(1)]
        d2 = ctx.batched_forward(models)
        g2 = ctx.batched_lqderivative(models, mis)
        assert [ctx.gemm_plan(0), ctx.gemm_plan(1)] == plans
        assert np.array_equal(d1, d2) and np.array_equal(g1, g2)
    finally:
        ctx.set_autotune(False)
    info = ctx.sensitivity_info()
    kb_fwd = -(-info["cols"] // 64)            # k-blocks of the forward (cells)
    kb_adj = -(-info["rows"] // 64)            # k-blocks of the adjoint (rows)
    for p, kb in zip(plans, (kb_fwd, kb_adj)):
        assert p["tile"] in (128, 256) and p["tuned_ms"] > 0
        assert p["nsplit"] >= -(-kb // 128)
    for i in (0, 299):
        check_groups(s, d1[i], oracle_forward(oracle_lib, s, models[i]))
        assert relerr(g1[i], oracle_lqderivative(oracle_lib, s, mis[i], models[i])) <= TOL
