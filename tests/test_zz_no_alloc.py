"""The allocation-free forward entry point, j3g_forward_noalloc.

It serves hosts that cannot let this library allocate device memory (an
application that has reserved all device memory for its own pool, or a loop
that must not take the synchronisation cudaMalloc/cudaFree imply); its
scratch is a fixed array inside the library.  Here it is called through the
C ABI with caller-owned device buffers and compared with the allocating
entry point (j3g_forward_device on a context) within the FP64 tolerance of
the parity tests, on two calls in a row so that contents left in the shared
scratch by the first call cannot leak into the second.

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

from helpers import relerr, small_survey
from jif3d_gb300 import capi, workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _noalloc(lib, s, d_nodes, d_st, d_model, d_data, stream=None):
    nx, ny, nz = s.shape
    return lib.j3g_forward_noalloc(
        s.kind, nx, ny, nz, d_nodes[0].data_ptr(), d_nodes[1].data_ptr(), d_nodes[2].data_ptr(),
        s.stations.shape[0], d_st[0].data_ptr(), d_st[1].data_ptr(), d_st[2].data_ptr(),
        s.inc, s.dec, s.fs, d_model.data_ptr(), d_data.data_ptr(), stream)


@pytest.mark.parametrize("kind", [W.SCALAR, W.TENSOR, W.MAGNETIC, W.JOINT])
def test_noalloc_matches_allocating_forward_twice(kind):
    import torch
    lib = capi.load()
    s = small_survey(kind, nx=21, ny=17, nz=9, nmeas=37, seed=500 + kind, bg=False)
    dev = torch.device("cuda", 0)
    f64 = dict(dtype=torch.float64, device=dev)
    d_nodes = [torch.tensor(s.coords(a), **f64) for a in range(3)]
    d_st = [torch.tensor(np.ascontiguousarray(s.stations[:, a]), **f64) for a in range(3)]
    ctx = capi.Context(0)
    W.setup_context(ctx, s)
    rng = np.random.default_rng(kind)
    for call in range(2):
        model = s.model * (1.0 + call) + rng.normal(size=s.model.size)
        d_model = torch.tensor(model, **f64)
        d_ref = torch.zeros(s.stations.shape[0] * s.raw, **f64)
        d_out = torch.full_like(d_ref, float("nan"))
        torch.cuda.synchronize()
        ctx.forward_device(d_model.data_ptr(), d_ref.data_ptr())
        ctx.synchronize()
        rc = _noalloc(lib, s, d_nodes, d_st, d_model, d_out)
        assert rc == capi.OK, lib.j3g_status_string(rc)
        torch.cuda.synchronize()
        ref = d_ref.cpu().numpy()
        out = d_out.cpu().numpy()
        assert np.all(np.isfinite(out))
        assert relerr(out, ref) <= TOL, (call, relerr(out, ref))
    ctx.close()


@pytest.mark.parametrize("kind", [W.SCALAR, W.JOINT])
def test_noalloc_larger_call_then_smaller_call(kind):
    """A large problem fills more of the shared scratch (more node blocks of
    partial sums, component sums at other offsets); the smaller problem after
    it must not read anything the large one left behind."""
    import torch
    lib = capi.load()
    dev = torch.device("cuda", 0)
    f64 = dict(dtype=torch.float64, device=dev)
    for n, (nx, ny, nz, nmeas) in enumerate(((40, 31, 12, 211), (9, 7, 5, 11))):
        s = small_survey(kind, nx=nx, ny=ny, nz=nz, nmeas=nmeas, seed=700 + 10 * kind + n,
                         bg=False)
        d_nodes = [torch.tensor(s.coords(a), **f64) for a in range(3)]
        d_st = [torch.tensor(np.ascontiguousarray(s.stations[:, a]), **f64) for a in range(3)]
        ctx = capi.Context(0)
        W.setup_context(ctx, s)
        d_model = torch.tensor(s.model, **f64)
        d_ref = torch.zeros(nmeas * s.raw, **f64)
        d_out = torch.full_like(d_ref, float("nan"))
        ctx.forward_device(d_model.data_ptr(), d_ref.data_ptr())
        ctx.synchronize()
        rc = _noalloc(lib, s, d_nodes, d_st, d_model, d_out)
        assert rc == capi.OK, lib.j3g_status_string(rc)
        torch.cuda.synchronize()
        out, ref = d_out.cpu().numpy(), d_ref.cpu().numpy()
        assert np.all(np.isfinite(out))
        assert relerr(out, ref) <= TOL, ((nx, ny, nz, nmeas), relerr(out, ref))
        ctx.close()


def test_noalloc_rejects_problems_beyond_its_scratch():
    import torch
    lib = capi.load()
    s = small_survey(W.TENSOR, nx=4, ny=4, nz=4, nmeas=3, seed=1, bg=False)
    f64 = dict(dtype=torch.float64, device=torch.device("cuda", 0))
    # 160 x 160 x 90 cells: 2.37 M nodes, more than the 2 Mi doubles of scratch
    nodes = [torch.arange(161, **f64), torch.arange(161, **f64), torch.arange(91, **f64)]
    st = [torch.zeros(3, **f64) for _ in range(3)]
    model = torch.zeros(160 * 160 * 90, **f64)
    out = torch.full((27,), 7.0, **f64)
    rc = lib.j3g_forward_noalloc(s.kind, 160, 160, 90, nodes[0].data_ptr(), nodes[1].data_ptr(),
                                 nodes[2].data_ptr(), 3, st[0].data_ptr(), st[1].data_ptr(),
                                 st[2].data_ptr(), 0.0, 0.0, 0.0, model.data_ptr(),
                                 out.data_ptr(), None)
    assert rc == capi.ERR_SCRATCH_LIMIT
    torch.cuda.synchronize()
    assert torch.all(out == 7.0)
