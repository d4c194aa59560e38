"""The failure path of the tensor-core products' bounded waits, without a GPU
fault.

Every mbarrier wait of the tensor-core kernels has a deadline; on expiry the
kernel records an error code, stops issuing, waits (bounded) for the copies
and MMAs it has issued, frees its TMEM and returns, and the host turns the
code into J3G_ERR_CUDA.  j3g_set_test_fault makes the drain warps withhold
their accumulator releases, so the MMA issuer's wait for one runs out (20 ms)
while every wait for a copy or an MMA keeps its full limit.  The reference's
CUDA layer has no such path: it exits the process on any error
(Global/CudaError.h:13-22).

Checked: the error reaches the caller through j3g_synchronize and through a
pipelined call's j3g_batched_wait (also when that call's ring slot was
reused before it was waited for), and the next normal call on the same
context succeeds and matches the oracle (mixed-path tolerance 1e-6).
"""
import numpy as np
import pytest

from helpers import oracle_forward, oracle_lqderivative, relerr, small_survey
from jif3d_gb300 import capi, workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-6
NMOD = 260  # more than 128 models: the CTA-pair kernel


@pytest.fixture
def one_split(ctx):
    """One K split per product, so that every CTA runs more than one k-block
    and its MMA issuer reaches a wait for a released accumulator; the plans
    are unpinned afterwards for the other tests on the shared context."""
    ctx.set_gemm_plan(0, 1, 0)
    ctx.set_gemm_plan(1, 1, 0)
    yield ctx
    ctx.set_test_fault(0)
    ctx.set_gemm_plan(0, 0, 0)
    ctx.set_gemm_plan(1, 0, 0)


def setup(ctx):
    # few rows and cells: every CTA of a launch is resident at once, so a
    # simulated stall costs one 2 s wait
    s = small_survey(W.JOINT, seed=808, nx=12, ny=11, nz=9, nmeas=16)
    W.setup_context(ctx, s)
    ctx.build_sensitivity(capi.STORE_F16X2)
    rng = np.random.default_rng(8)
    models = s.model[None, :] * (1 + 0.1 * rng.normal(size=(NMOD, s.nparm)))
    mis = rng.normal(size=(NMOD, s.stations.shape[0] * s.dpm))
    return s, models, mis


def check_against_oracle(O, s, models, mis, d, g):
    for i in (0, NMOD - 1):
        assert relerr(d[i], oracle_forward(O, s, models[i])) <= TOL
        assert relerr(g[i], oracle_lqderivative(O, s, mis[i], models[i])) <= TOL


def test_stalled_pipeline_reports_and_context_recovers(one_split, oracle_lib):
    import torch
    ctx = one_split
    s, models, mis = setup(ctx)
    n = s.stations.shape[0]
    dm = torch.tensor(models, dtype=torch.float64, device="cuda")
    dd = torch.zeros((NMOD, n * s.dpm), dtype=torch.float64, device="cuda")
    ctx.set_test_fault(1)
    try:
        ctx.batched_forward_device(NMOD, dm.data_ptr(), dd.data_ptr())
        with pytest.raises(capi.J3GError) as e:
            ctx.synchronize()
        assert e.value.code == capi.ERR_CUDA
        assert "wait expired" in str(e.value)
        # the host-buffer call checks the flag itself
        with pytest.raises(capi.J3GError) as e:
            ctx.batched_lqderivative(models, mis)
        assert e.value.code == capi.ERR_CUDA
    finally:
        ctx.set_test_fault(0)
    ctx.synchronize()  # the flag was cleared: nothing left to report
    d = ctx.batched_forward(models)
    g = ctx.batched_lqderivative(models, mis)
    check_against_oracle(oracle_lib, s, models, mis, d, g)


def test_stalled_pipelined_call_reports_at_its_wait(one_split, oracle_lib):
    ctx = one_split
    s, models, mis = setup(ctx)
    n = s.stations.shape[0]
    out = [np.zeros((NMOD, n * s.dpm)) for _ in range(6)]
    # a failing call waited for directly
    ctx.set_test_fault(1)
    try:
        t = ctx.batched_forward_async(models, out[0])
        with pytest.raises(capi.J3GError) as e:
            ctx.batched_wait(t)
        assert e.value.code == capi.ERR_CUDA
        # a failing call whose ring slot is reused before it is waited for
        t0 = ctx.batched_forward_async(models, out[1])
    finally:
        ctx.set_test_fault(0)
    later = [ctx.batched_forward_async(models, out[2 + k]) for k in range(4)]
    with pytest.raises(capi.J3GError) as e:
        ctx.batched_wait(t0)
    assert e.value.code == capi.ERR_CUDA
    for t in later:  # the calls queued behind it may see the same flag
        try:
            ctx.batched_wait(t)
        except capi.J3GError as err:
            assert err.code == capi.ERR_CUDA
    ctx.synchronize()
    d = ctx.batched_forward(models)
    g = ctx.batched_lqderivative(models, mis)
    check_against_oracle(oracle_lib, s, models, mis, d, g)
