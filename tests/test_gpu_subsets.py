"""Batches of station subsets of uneven size (j3g_subsets_*): one node-term
launch per direction for all subsets, one gradient per subset.  Checked
against the oracle on each subset as a survey of its own (FP64 tolerance,
relative norm error <= 1e-10), and on the config-5 mesh against the ordinary
entry points called subset by subset."""
import numpy as np
import pytest

from helpers import (oracle_forward, oracle_forward_lqderivative, oracle_lqderivative, relerr,
                     small_survey)
from jif3d_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-10


def dev(a):
    import torch
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def run_subsets(ctx, s, subsets, misfits):
    import torch
    W.setup_context(ctx, s)
    total = sum(len(x) for x in subsets)
    d = torch.zeros(max(total * s.dpm, 1), dtype=torch.float64, device="cuda")
    m = dev(s.model)
    ctx.subsets_forward_device(subsets, m.data_ptr(), d.data_ptr())
    g = torch.zeros((len(subsets), s.nparm), dtype=torch.float64, device="cuda")
    r = dev(np.concatenate(misfits) if total else np.zeros(1))
    ctx.subsets_lqderivative_device(subsets, m.data_ptr(), r.data_ptr(), g.data_ptr())
    ctx.synchronize()
    return d.cpu().numpy()[:total * s.dpm], g.cpu().numpy()


@pytest.mark.parametrize("kind,transform,bg", [(W.MAGNETIC, W.T_TFA, True),
                                               (W.JOINT, W.T_NONE, True),
                                               (W.TENSOR, W.T_FTG_INVARIANT, False)])
def test_subsets_against_oracle(ctx, oracle_lib, kind, transform, bg):
    s = small_survey(kind, seed=600 + kind, nx=9, ny=8, nz=6, nmeas=40, bg=bg,
                     transform=transform)
    rng = np.random.default_rng(kind)
    sizes = [7, 1, 0, 23, 40, 12]  # uneven, one empty, one with every station
    subsets = [np.sort(rng.choice(40, n, replace=False)) for n in sizes]
    subsets[1] = np.array([subsets[3][0]])  # a station shared by two subsets
    misfits = [rng.normal(size=len(x) * s.dpm) for x in subsets]
    d, g = run_subsets(ctx, s, subsets, misfits)
    o = 0
    for k, (sub, mis) in enumerate(zip(subsets, misfits)):
        ss = s.subset(sub)
        if len(sub):
            ref = oracle_forward(oracle_lib, ss)
            assert relerr(d[o:o + ref.size], ref) <= TOL, (k, relerr(d[o:o + ref.size], ref))
            o += ref.size
            gref = oracle_lqderivative(oracle_lib, ss, mis)
            assert relerr(g[k], gref) <= TOL, (k, relerr(g[k], gref))
        else:
            assert np.all(g[k] == 0.0)


def test_subsets_corner_path(ctx, oracle_lib):
    """Corner coordinates that are not running sums (eight-corner path)."""
    s = small_survey(W.SCALAR, seed=620, nmeas=20, origin=(0.1, 0.2, 0.0))
    s.xsize = s.xsize + 0.1 / 3.0
    xc = s.coords(0)
    xc[1:-1] += np.array([1e-9, -2e-9, 3e-9, 0.0, 1e-9, 0.0])[: xc.size - 2]
    subsets = [np.arange(0, 20, 3), np.arange(5, 17)]
    rng = np.random.default_rng(3)
    misfits = [rng.normal(size=len(x)) for x in subsets]
    import torch
    W.setup_context(ctx, s)
    ctx.set_mesh(xc, s.coords(1), s.coords(2), s.xsize, s.ysize, s.zsize)
    m = dev(s.model)
    d = torch.zeros(sum(len(x) for x in subsets), dtype=torch.float64, device="cuda")
    g = torch.zeros((2, s.nparm), dtype=torch.float64, device="cuda")
    ctx.subsets_forward_device(subsets, m.data_ptr(), d.data_ptr())
    ctx.subsets_lqderivative_device(subsets, m.data_ptr(), dev(np.concatenate(misfits)).data_ptr(),
                                    g.data_ptr())
    ctx.synchronize()
    O = oracle_lib
    o = 0
    for k, sub in enumerate(subsets):
        p = O.Problem(xc, s.coords(1), s.coords(2), s.xsize, s.ysize, s.zsize, s.stations[sub],
                      kind=W.SCALAR, bg_thick=s.bg_thick)
        assert relerr(d.cpu().numpy()[o:o + len(sub)], p.forward(s.model)) <= TOL
        o += len(sub)
        assert relerr(g[k].cpu().numpy(), p.lqderivative(s.model, misfits[k])) <= TOL


def test_config5_uneven_subsets(ctx, oracle_lib):
    """Config 5 (TFA magnetics, 128 x 128 x 64 cells) with four uneven
    subsets of its seeded batch: the batched subset calls against the
    ordinary calls made subset by subset, and two stations against the oracle."""
    import torch
    s = W.config5()
    subsets = [x[:n] for x, n in zip(s.subsets[:4], (256, 40, 160, 96))]
    rng = np.random.default_rng(5)
    misfits = [rng.normal(size=len(x)) for x in subsets]
    d, g = run_subsets(ctx, s, subsets, misfits)
    m = dev(s.model)
    o = 0
    for k, sub in enumerate(subsets):
        ss = s.subset(sub)
        W.setup_context(ctx, ss)
        dk = torch.zeros(len(sub), dtype=torch.float64, device="cuda")
        gk = torch.zeros(s.nparm, dtype=torch.float64, device="cuda")
        ctx.forward_device(m.data_ptr(), dk.data_ptr())
        ctx.lqderivative_device(m.data_ptr(), dev(misfits[k]).data_ptr(), gk.data_ptr())
        ctx.synchronize()
        assert relerr(d[o:o + len(sub)], dk.cpu().numpy()) <= 1e-12
        assert relerr(g[k], gk.cpu().numpy()) <= 1e-12
        o += len(sub)
    few = s.subset(subsets[1][:2])
    assert relerr(d[256:258], oracle_forward(oracle_lib, few)) <= TOL


def test_config5_full_batch_all_subsets(ctx, oracle_lib):
    """Config 5 as specified: all 32 seeded uneven subsets (282 to 3967
    stations, 74,753 in all) of total-field-anomaly magnetics on 128 x 128 x 64
    cells, through one subsets forward and one subsets adjoint call, as the
    reference runs one calculator per subset.  For every subset:
    * 16 seeded stations against the oracle: their data, and the subset's
      gradient of a misfit that is non-zero on those stations only (a second
      adjoint call over the whole batch);
    * over all of the subset's stations, the adjoint identity
      <d_k, r_k> = <m, g_k> / 2 of the first call pair (the TFA is linear in
      the field and config 5 has no background, so d_k = J_k m)."""
    import torch
    s = W.config5()
    subsets = s.subsets
    assert len(subsets) == 32
    rng = np.random.default_rng(55)
    misfits = [rng.normal(size=len(x)) for x in subsets]
    d, g = run_subsets(ctx, s, subsets, misfits)
    offsets = np.concatenate([[0], np.cumsum([len(x) for x in subsets])])
    for k in range(32):
        dk = d[offsets[k]:offsets[k + 1]]
        lhs = float(np.dot(dk, misfits[k]))
        rhs = 0.5 * float(np.dot(s.model, g[k]))
        assert abs(lhs - rhs) <= 1e-10 * np.linalg.norm(dk) * np.linalg.norm(misfits[k]), k
    del g
    pick = [np.sort(rng.choice(len(x), 16, replace=False)) for x in subsets]
    masked = []
    for k, x in enumerate(subsets):
        mk = np.zeros(len(x))
        mk[pick[k]] = misfits[k][pick[k]]
        masked.append(mk)
    gm = torch.zeros((32, s.nparm), dtype=torch.float64, device="cuda")
    ctx.subsets_lqderivative_device(subsets, dev(s.model).data_ptr(),
                                    dev(np.concatenate(masked)).data_ptr(), gm.data_ptr())
    ctx.synchronize()
    for k, x in enumerate(subsets):
        ss = s.subset(x[pick[k]])
        dref, gref = oracle_forward_lqderivative(oracle_lib, ss, misfits[k][pick[k]])
        got = d[offsets[k] + pick[k]]
        assert relerr(got, dref) <= TOL, (k, relerr(got, dref))
        gk = gm[k].cpu().numpy()
        assert relerr(gk, gref) <= TOL, (k, relerr(gk, gref))


def test_uneven_subsets_captured_in_cuda_graph(ctx, oracle_lib):
    """The uneven-subset forward and adjoint (one launch per direction for
    all subsets) captured in one CUDA graph after a warm-up call and replayed
    on a new model written in place: bit for bit the eager calls, and the
    oracle on each subset."""
    import torch
    s = small_survey(W.MAGNETIC, seed=640, nx=10, ny=9, nz=6, nmeas=60, transform=W.T_TFA)
    rng = np.random.default_rng(41)
    subsets = [np.sort(rng.choice(60, k, replace=False)) for k in (7, 31, 1, 18, 60)]
    W.setup_context(ctx, s)
    total = sum(len(x) for x in subsets)
    m = dev(s.model)
    d = torch.zeros(total * s.dpm, dtype=torch.float64, device="cuda")
    r = dev(rng.normal(size=total * s.dpm))
    g = torch.zeros((len(subsets), s.nparm), dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)

    def step():
        ctx.subsets_forward_device(subsets, m.data_ptr(), d.data_ptr())
        ctx.subsets_lqderivative_device(subsets, m.data_ptr(), r.data_ptr(), g.data_ptr())

    try:
        with torch.cuda.stream(stream):
            step()  # warm-up: buffers, background and the chunk table
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream):
            step()
        new = s.model * rng.uniform(0.5, 1.5, s.model.size)
        m.copy_(dev(new))
        graph.replay()
        torch.cuda.synchronize()
        d_graph, g_graph = d.cpu().numpy(), g.cpu().numpy()
        with torch.cuda.stream(stream):
            step()
        torch.cuda.synchronize()
    finally:
        ctx.set_stream(None)
    assert np.array_equal(d_graph, d.cpu().numpy())
    assert np.array_equal(g_graph, g.cpu().numpy())
    rr = r.cpu().numpy()
    o = 0
    for k, sub in enumerate(subsets):
        sk = s.subset(sub)
        n = len(sub)
        assert relerr(d_graph[o:o + n], oracle_forward(oracle_lib, sk, new)) <= TOL
        assert relerr(g_graph[k], oracle_lqderivative(oracle_lib, sk, rr[o:o + n], new)) <= TOL
        o += n
