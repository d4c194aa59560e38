"""GPU parity of the FP64 matrix-free path against the oracle.

Tolerance (FP64 path): relative norm error <= 1e-10 per output group, the
bound stated for the FP64 prism path.  The GPU evaluates the same corner
terms with CUDA's libm (log / atan2 may differ from glibc's in the last
bit); far-field prism terms cancel by up to ~(r/h)^3, so elementwise
relative differences of far cells are larger, but the norm-wise error of
data, sensitivity rows and gradients stays at the 1e-11 level.
"""
import math

import numpy as np
import pytest

from helpers import (maxrel, oracle_forward, oracle_forward_lqderivative, oracle_lqderivative,
                     oracle_problem, relerr, small_survey)
from jif3d_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-10


def gpu(ctx, s):
    W.setup_context(ctx, s)
    return ctx


KINDS = [W.SCALAR, W.TENSOR, W.MAGNETIC, W.JOINT]


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("bg", [False, True])
def test_forward_small(ctx, oracle_lib, kind, bg):
    s = small_survey(kind, seed=kind * 10 + bg, bg=bg)
    d = gpu(ctx, s).forward(s.model)
    ref = oracle_forward(oracle_lib, s)
    assert relerr(d, ref) <= TOL, relerr(d, ref)
    assert maxrel(d, ref) <= TOL


@pytest.mark.parametrize("kind", KINDS)
def test_sensitivity_rows(ctx, oracle_lib, kind):
    s = small_survey(kind, seed=40 + kind)
    d, J = gpu(ctx, s).forward_sens(s.model)
    dref, Jref = oracle_forward(oracle_lib, s, want_sens=True)
    assert J.shape == Jref.shape
    for r in range(J.shape[0]):
        assert relerr(J[r], Jref[r]) <= TOL, (r, relerr(J[r], Jref[r]))
    assert relerr(d, dref) <= TOL
    # data formed from the rows agree with the rows applied to the model
    raw = s.raw
    n = s.stations.shape[0]
    if s.transform == W.T_NONE:
        assert relerr(d, J @ s.model) <= 1e-13


@pytest.mark.parametrize("kind", KINDS)
def test_lqderivative(ctx, oracle_lib, kind):
    s = small_survey(kind, seed=60 + kind)
    rng = np.random.default_rng(kind)
    misfit = rng.normal(size=s.stations.shape[0] * s.dpm)
    g = gpu(ctx, s).lqderivative(s.model, misfit)
    ref = oracle_lqderivative(oracle_lib, s, misfit)
    assert relerr(g, ref) <= TOL, relerr(g, ref)


@pytest.mark.parametrize("kind,transform", [(W.TENSOR, W.T_FTG_INVARIANT),
                                            (W.MAGNETIC, W.T_TOTAL_FIELD),
                                            (W.MAGNETIC, W.T_TFA)])
def test_transforms(ctx, oracle_lib, kind, transform):
    s = small_survey(kind, seed=70 + transform, transform=transform)
    c = gpu(ctx, s)
    d = c.forward(s.model)
    ref = oracle_forward(oracle_lib, s)
    assert d.size == s.stations.shape[0]
    assert relerr(d, ref) <= TOL
    misfit = np.random.default_rng(5).normal(size=d.size)
    g = c.lqderivative(s.model, misfit)
    gref = oracle_lqderivative(oracle_lib, s, misfit)
    assert relerr(g, gref) <= TOL, relerr(g, gref)


@pytest.mark.parametrize("kind", [W.SCALAR, W.TENSOR])
def test_non_running_sum_coordinates_use_corner_path(ctx, oracle_lib, kind):
    """Corner coordinates that are not running sums of the sizes: every prism
    corner is evaluated on its own (no node sharing), as the reference does."""
    s = small_survey(kind, seed=80, origin=(0.1, 0.2, 0.0))
    s.xsize = s.xsize + 0.1 / 3.0
    xc = s.coords(0)
    xc[1:-1] += np.array([1e-9, -2e-9, 3e-9, 0.0, 1e-9, 0.0])[: xc.size - 2]
    c = gpu(ctx, s)
    c.set_mesh(xc, s.coords(1), s.coords(2), s.xsize, s.ysize, s.zsize)
    d = c.forward(s.model)
    O = oracle_lib
    p = O.Problem(xc, s.coords(1), s.coords(2), s.xsize, s.ysize, s.zsize, s.stations,
                  kind=kind, bg_thick=s.bg_thick)
    ref = p.forward(s.model)
    assert relerr(d, ref) <= TOL
    misfit = np.random.default_rng(2).normal(size=d.size)
    assert relerr(c.lqderivative(s.model, misfit), p.lqderivative(s.model, misfit)) <= TOL


@pytest.mark.parametrize("kind", KINDS)
def test_many_background_layers(ctx, oracle_lib, kind):
    """Forty background layers (one thread per station and layer), some
    inside the gridded depth, some across its bottom and some below it, with
    80 stations (several thread blocks): data and gradient, background
    columns included, against the oracle."""
    s = small_survey(kind, seed=95 + kind, nmeas=80)
    rng = np.random.default_rng(kind)
    s.bg_thick = rng.uniform(5.0, 60.0, 40)
    s.model = np.concatenate([s.model[:s.ngrid], rng.uniform(1, 5, 40)])
    c = gpu(ctx, s)
    d = c.forward(s.model)
    assert relerr(d, oracle_forward(oracle_lib, s)) <= TOL
    misfit = rng.normal(size=d.size)
    g = c.lqderivative(s.model, misfit)
    gref = oracle_lqderivative(oracle_lib, s, misfit)
    assert relerr(g, gref) <= TOL
    assert relerr(g[s.ngrid:], gref[s.ngrid:]) <= TOL


def test_edge_cases(ctx, oracle_lib):
    O = oracle_lib
    # background only, no grid cells (test_ScalarCalculation.cpp:123-147)
    rng = np.random.default_rng(3)
    st = np.stack([rng.integers(0, 50000, 10) + 2e4, rng.integers(0, 50000, 10) + 2e4,
                   np.zeros(10)], axis=1)
    s = W.Survey("bg", np.zeros(0), np.zeros(0), np.zeros(0), (0.0, 0.0, 0.0), st, W.SCALAR,
                 np.array([1.0, 1.0, 5.0, 5.0]), bg_thick=np.array([200.0, 300.0, 3500.0, 1000.0]))
    d = gpu(ctx, s).forward(s.model)
    analytic = 2 * math.pi * 6.67428e-11 * (500.0 + 5.0 * 4500.0)
    np.testing.assert_allclose(d, analytic, rtol=1e-4)
    assert relerr(d, oracle_problem(O, s).forward(s.model)) <= 1e-14
    g = ctx.lqderivative(s.model, np.ones(10))
    assert g.size == 4 and relerr(g, oracle_problem(O, s).lqderivative(s.model, np.ones(10))) <= 1e-13
    # no stations
    s2 = small_survey(W.TENSOR, nmeas=1, seed=4)
    s2.stations = np.zeros((0, 3))
    c = gpu(ctx, s2)
    assert c.forward(s2.model).size == 0
    assert np.all(c.lqderivative(s2.model, np.zeros(0)) == 0)
    # one cell, stations on a corner, an edge and a face of the prism
    s3 = W.Survey("one", np.array([10.0]), np.array([10.0]), np.array([10.0]), (0.0, 0.0, 0.0),
                  np.array([[0.0, 0.0, 0.0], [5.0, 0.0, 0.0], [5.0, 5.0, 0.0], [0.0, 5.0, -3.0]]),
                  W.SCALAR, np.array([1000.0]))
    for kind in (W.SCALAR, W.TENSOR):
        s3.kind = kind
        d = gpu(ctx, s3).forward(s3.model)
        ref = oracle_problem(O, s3).forward(s3.model)
        assert np.array_equal(np.isnan(d), np.isnan(ref))
        ok = ~np.isnan(ref)
        assert relerr(d[ok], ref[ok]) <= TOL


def test_bad_arguments_raise(ctx):
    from jif3d_gb300 import capi
    s = small_survey(W.SCALAR, seed=1)
    c = gpu(ctx, s)
    with pytest.raises(capi.J3GError):
        c.forward(np.zeros(3))
    with pytest.raises(capi.J3GError):
        c.set_transform(capi.T_FTG_INVARIANT)
    with pytest.raises(capi.J3GError):
        c.set_kind(17)


def test_repeatable_bit_identical(ctx):
    s = small_survey(W.JOINT, seed=90, nx=20, ny=18, nz=9, nmeas=40)
    c = gpu(ctx, s)
    d0 = c.forward(s.model)
    misfit = np.random.default_rng(1).normal(size=d0.size)
    g0 = c.lqderivative(s.model, misfit)
    for _ in range(5):
        assert np.array_equal(c.forward(s.model), d0)
        assert np.array_equal(c.lqderivative(s.model, misfit), g0)


def test_config1_full(ctx, oracle_lib):
    """Config 1 at full size: g_z of 400 stations and the full sensitivity matrix."""
    s = W.config1()
    c = gpu(ctx, s)
    d, J = c.forward_sens(s.model)
    dref, Jref = oracle_forward(oracle_lib, s, want_sens=True)
    assert relerr(d, dref) <= TOL
    assert relerr(J, Jref) <= TOL
    d2 = c.forward(s.model)
    assert relerr(d2, dref) <= TOL
    # the same without the constant background part
    ngrid = s.ngrid
    bgpart = Jref[:, ngrid:] @ s.model[ngrid:]
    assert relerr(d2 - bgpart, dref - bgpart) <= TOL


def test_config2_subset_and_adjoint_identity(ctx, oracle_lib):
    """Config 2 (FTG, 64 x 64 x 32 cells): 134 of its 1600 stations (every
    twelfth) against the oracle, data and gradient; at full size the adjoint
    identity."""
    s = W.config2()
    sub = s.subset(np.arange(0, 1600, 12))
    misfit = np.random.default_rng(21).normal(size=sub.stations.shape[0] * 9)
    c = gpu(ctx, sub)
    d = c.forward(sub.model)
    g = c.lqderivative(sub.model, misfit)
    dref, gref = oracle_forward_lqderivative(oracle_lib, sub, misfit)
    assert relerr(d, dref) <= TOL, relerr(d, dref)
    assert relerr(g, gref) <= TOL, relerr(g, gref)
    # full size: <J m, r> = <m, J^T r> (LQDerivative returns 2 J^T r)
    c = gpu(ctx, s)
    rng = np.random.default_rng(9)
    m2 = rng.normal(size=s.nparm)
    r = rng.normal(size=s.stations.shape[0] * 9)
    d2 = c.forward(m2)
    g2 = c.lqderivative(s.model, r)
    lhs = float(np.dot(d2, r))
    rhs = 0.5 * float(np.dot(m2, g2))
    # random signs: the dot products cancel, so the scale is |J m| |r|
    assert abs(lhs - rhs) <= 1e-10 * np.linalg.norm(d2) * np.linalg.norm(r)


def test_config3_gradient_subset_and_fd(ctx, oracle_lib):
    """Joint g_z + FTG weighted gradient: oracle LQDerivative on a station
    subset, and central differences (relative step 1e-4) on seeded cells."""
    s = W.config3()
    sub = s.subset(np.arange(0, 2500, 19))  # 132 stations
    rng = np.random.default_rng(31)
    n = sub.stations.shape[0]
    sigma = np.tile(np.array([1e-8] + [1e-9] * 9), n)
    r = sigma * rng.normal(size=n * 10)
    misfit = r / sigma ** 2
    c = gpu(ctx, sub)
    d = c.forward(sub.model)
    g = c.lqderivative(sub.model, misfit)
    dref, ref = oracle_forward_lqderivative(oracle_lib, sub, misfit)
    dg, dt = d.reshape(n, 10), dref.reshape(n, 10)
    assert relerr(dg[:, 0], dt[:, 0]) <= TOL and relerr(dg[:, 1:], dt[:, 1:]) <= TOL
    assert relerr(g, ref) <= TOL, relerr(g, ref)
    # central differences of phi(m) = sum (d(m) - d_obs)^2 / sigma^2 around d_obs = d(m0) - r
    d0 = c.forward(sub.model)
    obs = d0 - r
    phi = lambda m: float(np.sum((c.forward(m) - obs) ** 2 / sigma ** 2))
    grad = c.lqderivative(sub.model, (d0 - obs) / sigma ** 2)
    cells = np.random.default_rng(33).choice(sub.ngrid, 64, replace=False)
    for i in cells:
        h = 1e-4 * abs(sub.model[i])
        mp, mm = sub.model.copy(), sub.model.copy()
        mp[i] += h
        mm[i] -= h
        fd = (phi(mp) - phi(mm)) / (2 * h)
        assert abs(fd - grad[i]) <= 1e-4 * abs(grad[i]) + 1e-6 * np.abs(grad).max(), (i, fd, grad[i])


def test_config5_tfa_subset(ctx, oracle_lib):
    s = W.config5()
    sub = s.subset(s.subsets[0][:6])
    c = gpu(ctx, sub)
    d = c.forward(sub.model)
    assert relerr(d, oracle_forward(oracle_lib, sub)) <= TOL
    misfit = np.random.default_rng(4).normal(size=d.size)
    g = c.lqderivative(sub.model, misfit)
    assert relerr(g, oracle_lqderivative(oracle_lib, sub, misfit)) <= TOL
