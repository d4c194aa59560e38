"""CPU tests of the FP64 oracle against the reference's golden values.

These pin the oracle before it is trusted as the checker of the GPU path:
* bit-exact agreement with the reference's own box terms (golden fixture made
  from jif3D Gravity/BasicGravElements.cpp, and live where that build exists);
* the known-answer tests of the reference's test files, with their tolerances.
"""
import json
import math
import os

import numpy as np
import pytest

from helpers import oracle_problem, small_survey
from jif3d_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
G = 6.67428e-11
FLT_EPS = float(np.finfo(np.float32).eps)
DBL_EPS = float(np.finfo(np.float64).eps)


def check_close(a, b, pct):
    """BOOST_CHECK_CLOSE: relative difference to both values within pct percent."""
    d = abs(a - b)
    assert d <= abs(a) * pct / 100 and d <= abs(b) * pct / 100, (a, b, pct)


def test_box_terms_bit_exact_vs_reference_golden(oracle_lib):
    O = oracle_lib
    with open(os.path.join(GOLDEN, "box_terms.json")) as f:
        cases = json.load(f)["cases"]
    assert len(cases) > 300
    for c in cases:
        gz = O.grav_box(*c["args"])
        t = O.tensor_box(*c["args"])
        assert np.array_equal(np.float64(gz), np.float64(c["gz"]), equal_nan=True), c["args"]
        assert np.array_equal(t, np.array(c["tensor"]), equal_nan=True), c["args"]


def test_box_terms_bit_exact_vs_reference_build(oracle_lib):
    O = oracle_lib
    R = O.ref_lib()
    if R is None:
        pytest.skip("reference BasicGravElements.cpp not built on this machine")
    rng = np.random.default_rng(7)
    for _ in range(20000):
        a = list(rng.uniform(-2000, 2000, 6)) + list(rng.uniform(0.5, 300, 3))
        t = np.zeros(9)
        R.ref_tensor_box(*a, t.ctypes.data_as(O._P))
        assert O.grav_box(*a) == R.ref_grav_box(*a)
        assert np.array_equal(O.tensor_box(*a), t)
    for mz in (-5.0, 0.0, 50.0, 150.0, 300.0):
        for top, bot in ((0.0, 100.0), (100.0, 250.0)):
            assert O.lib().orc_inf_sheet(mz, top, bot) == R.ref_inf_sheet(mz, top, bot)
            assert O.lib().orc_uzz_inf_sheet(mz, top, bot) == R.ref_uzz_inf_sheet(mz, top, bot)


def test_box_gravity_calc_kat(oracle_lib):
    """Gravity/test_ScalarCalculation.cpp:32-64."""
    O = oracle_lib
    assert abs(O.grav_box(0, 0, 0, -10, -10, -10, 20, 20, 20)) < DBL_EPS
    top = O.grav_box(0, 0, -10, -10, -10, -10, 20, 20, 20)
    check_close(top, 3.46426e-9, 0.1)
    bottom = O.grav_box(0, 0, 10, -10, -10, -10, 20, 20, 20)
    check_close(top, -bottom, FLT_EPS)
    check_close(top, O.grav_box(10, 10, 0, 0, 0, 0, 20, 20, 20), FLT_EPS)
    assert O.grav_box(1e5, 10, 10, -10, -10, -10, 20, 20, 20) < DBL_EPS
    check_close(O.grav_box(100, 100, 10, -10, -10, -10, 20, 20, 20), -1.873178e-12, 0.1)
    assert abs(O.grav_box(0, 0, 0, -1e6, -1e6, -1e6, 2e6, 2e6, 2e6)) < DBL_EPS


def _cube_survey(kind, ncells=10, cell=2.0, meas=(9.0, 8.0, -0.1)):
    xs = np.full(ncells, cell)
    return W.Survey("cube", xs, xs.copy(), xs.copy(), (0.0, 0.0, 0.0),
                    np.array([meas]), kind, np.ones(ncells ** 3))


def test_model_gravity_boxcomp(oracle_lib):
    """10^3 grid of 2 m cells equals one 20 m prism (test_ScalarCalculation.cpp:67-120)."""
    O = oracle_lib
    box = O.grav_box(9, 8, -0.1, 0, 0, 0, 20, 20, 20)
    tbox = O.tensor_box(9, 8, -0.1, 0, 0, 0, 20, 20, 20)
    s = _cube_survey(W.SCALAR)
    d, J = oracle_problem(O, s).forward(s.model, True)
    check_close(box, d[0], FLT_EPS)
    check_close(d[0], (J @ s.model)[0], FLT_EPS)
    t = oracle_problem(O, _cube_survey(W.TENSOR)).forward(s.model)
    for i in range(9):
        check_close(t[i], tbox[i], FLT_EPS)
    check_close(t[0] + t[4], -t[8], FLT_EPS)


def test_background_only(oracle_lib):
    """No grid cells, 4 layers: 2 pi G sum(rho h) (test_ScalarCalculation.cpp:123-147)."""
    O = oracle_lib
    rng = np.random.default_rng(3)
    st = np.stack([rng.integers(0, 50000, 10) + 2e4, rng.integers(0, 50000, 10) + 2e4,
                   np.zeros(10)], axis=1)
    s = W.Survey("bg", np.zeros(0), np.zeros(0), np.zeros(0), (0.0, 0.0, 0.0), st, W.SCALAR,
                 np.array([1.0, 1.0, 5.0, 5.0]), bg_thick=np.array([200.0, 300.0, 3500.0, 1000.0]))
    d = oracle_problem(O, s).forward(s.model)
    analytic = 2 * math.pi * G * (500.0 + 5.0 * 4500.0)
    for v in d:
        check_close(analytic, v, 0.01)


def layered_survey(kind, seed=5, nmeas=10):
    """Random lateral cells over a 1-D layering plus background
    (test_ScalarCalculation.cpp:150-244)."""
    rng = np.random.default_rng(seed)
    nh, nz = int(rng.integers(10, 25)), 10
    xs = rng.integers(1000, 11000, nh).astype(float)
    ys = rng.integers(1000, 11000, nh).astype(float)
    zs = np.full(nz, 500.0)
    rho = np.full((nh, nh, nz), 5.0)
    rho[:, :, 0] = 1.0
    st = np.stack([rng.integers(0, 50000, nmeas) + 2e4, rng.integers(0, 50000, nmeas) + 2e4,
                   np.full(nmeas, -1.0)], axis=1)
    return W.Survey("layered", xs, ys, zs, (0.0, 0.0, 0.0), st, kind,
                    np.concatenate([rho.ravel(), [1.0, 1.0, 5.0, 5.0]]),
                    bg_thick=np.array([200.0, 300.0, 3500.0, 2000.0]))


def test_model_gravity_1danaly(oracle_lib):
    O = oracle_lib
    analytic = 2 * math.pi * G * (500.0 + 5.0 * 5500.0)
    s = layered_survey(W.SCALAR)
    d, J = oracle_problem(O, s).forward(s.model, True)
    for v, vj in zip(d, J @ s.model):
        check_close(analytic, v, 0.01)
        check_close(analytic, vj, 0.01)
    t = oracle_problem(O, layered_survey(W.TENSOR)).forward(s.model)
    assert np.all(np.abs(t) < DBL_EPS)


def test_tensor_poisson(oracle_lib):
    """Trace jump -4 pi G rho across the surface (test_TensorCalculation.cpp:187-227)."""
    O = oracle_lib
    xs = np.full(10, 10.0)
    dens = 2.1
    s = W.Survey("poisson", xs, xs.copy(), xs.copy(), (0.0, 0.0, 0.0),
                 np.array([[5.0, 5.0, -1.0], [5.0, 5.0, 50.0]]), W.TENSOR,
                 np.concatenate([np.full(1000, dens), [dens]]), bg_thick=np.array([100.0]))
    t = oracle_problem(O, s).forward(s.model)
    tr1, tr2 = t[0] + t[4] + t[8], t[9] + t[13] + t[17]
    check_close(-4 * math.pi * G * dens, tr1 - tr2, FLT_EPS)
    check_close(dens, tr2 / (4 * math.pi * G), FLT_EPS)


def test_random_tensor_properties(oracle_lib):
    """Traceless and symmetric above the surface (test_TensorCalculation.cpp:32-57)."""
    O = oracle_lib
    s = small_survey(W.TENSOR, nmeas=15, seed=11)
    t = oracle_problem(O, s).forward(s.model).reshape(-1, 9)
    for r in t:
        check_close(r[0] + r[4], -r[8], FLT_EPS)
        assert r[1] == r[3] and r[2] == r[6] and r[5] == r[7]


def test_fd_tensor(oracle_lib):
    """Uz* equal central differences of g_z (test_TensorCalculation.cpp:60-106)."""
    O = oracle_lib
    s = small_survey(W.TENSOR, seed=12, bg=False, nx=8, ny=8, nz=6, origin=(0.0, 0.0, 0.0))
    delta, p = 1e-6, 0.05
    x, y, z = 50.0, 70.0, -5.1
    pts = [(x, y, z), (x, y, z - delta), (x, y, z + delta), (x, y - delta, z),
           (x, y + delta, z), (x - delta, y, z), (x + delta, y, z)]
    s.stations = np.array(pts)
    t = oracle_problem(O, s).forward(s.model)
    g = oracle_problem(O, s, W.SCALAR).forward(s.model)
    check_close(t[8], (g[2] - g[1]) / (2 * delta), p)
    check_close(t[7], (g[4] - g[3]) / (2 * delta), p)
    check_close(t[6], (g[6] - g[5]) / (2 * delta), p)


@pytest.mark.parametrize("kind", [W.SCALAR, W.TENSOR, W.MAGNETIC])
def test_lqderivative_equals_2JTr(oracle_lib, kind):
    """LQDerivative = 2 J^T r (test_ScalarCalculation.cpp:289-306, test_TensorCalculation.cpp:285-318)."""
    O = oracle_lib
    s = small_survey(kind, seed=13)
    p = oracle_problem(O, s)
    rng = np.random.default_rng(1)
    r = rng.uniform(0, 1, s.stations.shape[0] * s.raw)
    g = p.lqderivative(s.model, r)
    _, J = p.forward(s.model, True)
    ref = O.sens_rmatvec2(J, r)
    np.testing.assert_allclose(g, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("kind,transform", [(W.SCALAR, W.T_NONE), (W.TENSOR, W.T_FTG_INVARIANT),
                                            (W.MAGNETIC, W.T_TFA), (W.MAGNETIC, W.T_NONE)])
def test_fused_forward_lqderivative_is_both_calls(oracle_lib, kind, transform):
    """The one-pass oracle call gives the forward and the derivative of the
    two separate calls bit for bit."""
    O = oracle_lib
    s = small_survey(kind, seed=17 + kind, transform=transform)
    p = oracle_problem(O, s)
    r = np.random.default_rng(2).normal(size=s.stations.shape[0] * s.dpm)
    d, g = p.forward_lqderivative(s.model, r)
    assert np.array_equal(d, p.forward(s.model))
    assert np.array_equal(g, p.lqderivative(s.model, r))


def test_ftg_invariant_kat():
    """Gravity/test_transforms.cpp:27-56."""
    from jif3d_gb300.gravmag import FTGInvariant
    t = FTGInvariant()
    x = np.array([1, 2, 3, 2, 4, 5, 3, 5, 6], float)
    assert t.Transform(x)[0] == -4.0
    assert list(t.Derivative(x)[0]) == [10, -2, -3, -2, 7, -5, -3, -5, 5]


def _simpeg_survey(kind=W.MAGNETIC, transform=W.T_NONE, yscale=2.0, inc_deg=15.0, dec_deg=10.0):
    n = 10
    xs, ys, zs = np.full(n, 2.0), np.full(n, 2.0 * yscale), np.full(n, 0.5)
    st = np.array([[-20.0 + i / 5.0, 10.0, -1.0] for i in range(200)])
    inc, dec = math.radians(inc_deg), math.radians(dec_deg)
    return W.Survey("simpeg", xs, ys, zs, (-xs.sum() / 2, -ys.sum() / 2, 0.0), st, kind,
                    np.full(n ** 3, 0.2), inc=inc, dec=dec, fs=50000.0, transform=transform,
                    t_inc=inc, t_dec=dec)


def test_magnetics_simpeg_golden(oracle_lib):
    """Bx, By, Bz and TFA vs SimPEG within 0.2 % (test_MagneticCalculation.cpp:110-217)."""
    O = oracle_lib
    with open(os.path.join(GOLDEN, "simpeg_mag.json")) as f:
        sim = json.load(f)
    s = _simpeg_survey()
    b = oracle_problem(O, s).forward(s.model).reshape(-1, 3)
    for i in range(200):
        check_close(b[i, 0], sim["x"][i], 0.2)
        check_close(b[i, 1], sim["y"][i], 0.2)
        check_close(b[i, 2], sim["z"][i], 0.2)
    t = oracle_problem(O, _simpeg_survey(transform=W.T_TFA)).forward(s.model)
    for i in range(200):
        check_close(t[i], sim["t"][i], 0.2)


def mag_block(xpos, width, depth, height, magnetization):
    """2-D analytic block, test_MagneticCalculation.cpp:9-19."""
    m = width / 2.0
    f = magnetization / (2 * math.pi)
    return f * (math.atan2(xpos + m, depth) - math.atan2(xpos - m, depth)
                - math.atan2(xpos + m, depth + height) + math.atan2(xpos - m, depth + height))


def test_magnetics_boxcomp_analytic(oracle_lib):
    """Elongated block at I = 90 deg vs the 2-D solution (test_MagneticCalculation.cpp:28-108)."""
    O = oracle_lib
    s = _simpeg_survey(transform=W.T_TFA, yscale=100.0, inc_deg=90.0, dec_deg=0.0)
    t = oracle_problem(O, s).forward(s.model)
    for i in range(200):
        ref = mag_block(s.stations[i, 0], 20.0, 1.0, 5.0, 50000 * 0.2)
        check_close(t[i], ref, 0.1)


def objective(O, s, model, observed, sigma2):
    d = oracle_problem(O, s).forward(model)
    return float(np.sum((d - observed) ** 2 / sigma2)), d


@pytest.mark.parametrize("kind", [W.SCALAR, W.TENSOR])
def test_objective_fd_gradient(oracle_lib, kind):
    """Objective gradient vs central differences, step 1 % (test_GravityObjective.cpp:31-110)."""
    O = oracle_lib
    s = small_survey(kind, nx=4, ny=3, nz=3, nmeas=3, seed=21, bg=False)
    obs = oracle_problem(O, s).forward(s.model) * 1.1
    sigma2 = np.ones_like(obs)
    _, d = objective(O, s, s.model, obs, sigma2)
    grad = oracle_problem(O, s).lqderivative(s.model, (d - obs) / sigma2)
    for i in range(s.model.size):
        delta = s.model[i] * 0.01
        mp, mm = s.model.copy(), s.model.copy()
        mp[i] += delta
        mm[i] -= delta
        fd = (objective(O, s, mp, obs, sigma2)[0] - objective(O, s, mm, obs, sigma2)[0]) / (2 * delta)
        check_close(fd, grad[i], 0.001)


def test_openmp_thread_count_invariance(oracle_lib):
    O = oracle_lib
    s = small_survey(W.TENSOR, seed=17, nx=12, ny=11, nz=9)
    d1 = oracle_problem(O, s).forward(s.model)
    p = oracle_problem(O, s)
    p.nthreads = 1
    d2 = p.forward(s.model)
    np.testing.assert_allclose(d1, d2, rtol=1e-12, atol=1e-22)


def magnetization_survey(seed, nx=4, ny=3, nz=3, nmeas=3, transform=W.T_NONE):
    """Small magnetisation survey: three cell blocks, no background."""
    s = small_survey(W.MAGNETIZATION, nx=nx, ny=ny, nz=nz, nmeas=nmeas, seed=seed, bg=False,
                     transform=transform)
    rng = np.random.default_rng(seed + 1000)
    s.model = rng.uniform(0.1, 2.0, 3 * s.ngrid)
    return s


@pytest.mark.parametrize("kind", [W.MAG_GRADIENT, W.MAGNETIZATION])
def test_objective_fd_gradient_magnetic_kinds(oracle_lib, kind):
    """Objective gradient vs central differences for the vertical magnetic
    gradient (test_MagneticGradObjective.cpp:72-110) and magnetisation
    (test_MagneticObjective.cpp:176-211), step 1 %, 0.01 %."""
    O = oracle_lib
    s = (magnetization_survey(31) if kind == W.MAGNETIZATION
         else small_survey(kind, nx=4, ny=3, nz=3, nmeas=3, seed=31, bg=False))
    obs = oracle_problem(O, s).forward(s.model) * 1.1
    sigma2 = np.ones_like(obs)
    _, d = objective(O, s, s.model, obs, sigma2)
    grad = oracle_problem(O, s).lqderivative(s.model, (d - obs) / sigma2)
    for i in range(s.model.size):
        delta = s.model[i] * 0.01
        mp, mm = s.model.copy(), s.model.copy()
        mp[i] += delta
        mm[i] -= delta
        fd = (objective(O, s, mp, obs, sigma2)[0] - objective(O, s, mm, obs, sigma2)[0]) / (2 * delta)
        check_close(fd, grad[i], 0.01)


def test_magnetization_equals_induced(oracle_lib):
    """Magnetisation M = chi F b / (1e9 mu0) reproduces the induced field of
    the susceptibility chi (the two implementations share the tensor terms:
    OMPMagnetizationImp.cpp:58-68 vs OMPMagneticSusceptibilityImp.cpp:116-170)."""
    O = oracle_lib
    s = small_survey(W.MAGNETIC, seed=33, bg=False)
    chi = s.model[:s.ngrid]
    b = np.array([math.cos(s.inc) * math.cos(s.dec), math.cos(s.inc) * math.sin(s.dec),
                  math.sin(s.inc)])
    mu0 = 4e-7 * math.pi
    ref = oracle_problem(O, s).forward(chi)
    m = magnetization_survey(33)
    m.xsize, m.ysize, m.zsize, m.stations = s.xsize, s.ysize, s.zsize, s.stations
    m.origin = s.origin
    model = np.concatenate([chi * s.fs * b[j] / (1e9 * mu0) for j in range(3)])
    got = oracle_problem(O, m).forward(model)
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


def test_vertical_gradient_is_field_difference(oracle_lib):
    """Bz(z) - Bz(z + 1 m) of OMPMagneticGradImp equals the difference of the
    magnetic Bz rows at the two heights times mu0 (its factor 1e-7 / G
    against 1 / (4 pi G)); background layers contribute nothing."""
    O = oracle_lib
    s = small_survey(W.MAG_GRADIENT, seed=35, bg=True)
    got = oracle_problem(O, s).forward(s.model)
    m = small_survey(W.MAGNETIC, seed=35, bg=False)
    chi = s.model[:s.ngrid]
    top = m.subset(np.arange(s.stations.shape[0]))
    top.stations = s.stations + np.array([0.0, 0.0, 1.0])
    bz0 = oracle_problem(O, m).forward(chi).reshape(-1, 3)[:, 2]
    bz1 = oracle_problem(O, top).forward(chi).reshape(-1, 3)[:, 2]
    ref = (bz0 - bz1) * 4e-7 * math.pi
    np.testing.assert_allclose(got, ref, rtol=1e-9, atol=1e-9 * np.abs(ref).max())
    # the background columns of the sensitivity are zero
    _, J = oracle_problem(O, s).forward(s.model, True)
    assert J.shape == (s.stations.shape[0], s.nparm)
    assert np.all(J[:, s.ngrid:] == 0.0)


def test_lqderivative_equals_2JTr_magnetic_kinds(oracle_lib):
    O = oracle_lib
    for s in (small_survey(W.MAG_GRADIENT, seed=37), magnetization_survey(37, nx=5, ny=4, nz=3,
                                                                          nmeas=6)):
        p = oracle_problem(O, s)
        r = np.random.default_rng(2).uniform(-1, 1, s.stations.shape[0] * s.raw)
        g = p.lqderivative(s.model, r)
        _, J = p.forward(s.model, True)
        ref = O.sens_rmatvec2(J, r)
        np.testing.assert_allclose(g, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


# -- model refinement (ModelBase/test_ModelRefiner.cpp) -------------------------
def refiner_case():
    """MakeModelandRefinement (test_ModelRefiner.cpp:37-75): a 2 x 3 x 5 coarse
    grid of 50 / 40 / 30 m cells, refinement coordinates 10 i, 20 i, 5 i."""
    cs = [np.full(2, 50.0), np.full(3, 40.0), np.full(5, 30.0)]
    refs = [10.0 * np.arange(20), 20.0 * np.arange(20), 5.0 * np.arange(50)]
    return cs, refs


def test_refiner_basic_axis_refinement(oracle_lib):
    """basic_axis_refinement (test_ModelRefiner.cpp:77-113): the refined
    corners are the union of coarse and refinement coordinates, the domain
    ends where the coarse one ends."""
    O = oracle_lib
    cs, refs = refiner_case()
    for c, r in zip(cs, refs):
        cc = O.corners(0.0, c)
        f = O.refine_axis(cc, c, r)
        fc = O.corners(0.0, f)
        union = np.unique(np.concatenate([r, cc]))
        assert np.array_equal(fc[:-1], union[:f.size])      # CheckAxis :20-35
        assert fc[-1] == cc[-1]                             # :99-110
    # the reference's sizes: 10 x 10 m, 6 x 20 m, 30 x 5 m
    assert [O.refine_axis(O.corners(0.0, c), c, r).size for c, r in zip(cs, refs)] == [10, 6, 30]


def test_refiner_model_projection(oracle_lib):
    """model_projection (test_ModelRefiner.cpp:115-147): a unit fine gradient
    combines to 60 on every coarse cell (5 x 2 x 6 refined cells each), and
    every refined cell takes the value of the coarse cell that contains it."""
    O = oracle_lib
    cs, refs = refiner_case()
    fs = [O.refine_axis(O.corners(0.0, c), c, r) for c, r in zip(cs, refs)]
    nfine = int(np.prod([f.size for f in fs]))
    g = O.refine_combine(cs, fs, np.ones(nfine))
    assert g.size == 30 and np.all(g == 60.0)
    coarse = np.arange(30, dtype=float)                     # std::iota (:128-130)
    fine = O.refine_project(cs, fs, coarse).reshape([f.size for f in fs])
    cen = [O.corners(0.0, f)[:-1] + 0.5 * f for f in fs]
    owner = [np.searchsorted(O.corners(0.0, c), x) - 1 for c, x in zip(cs, cen)]
    expect = coarse.reshape(2, 3, 5)[np.ix_(*owner)]
    assert np.array_equal(fine, expect)


def test_refiner_walk_edge_cases(oracle_lib):
    """Refined cells past every coarse run keep their values; coarse corners
    that repeat refinement coordinates are not doubled; a coarse cell whose
    walk finds no refined cells combines to 0."""
    O = oracle_lib
    cs = [np.array([10.0]), np.array([4.0, 6.0]), np.array([5.0])]
    fs = [np.array([5.0, 5.0, 5.0]), np.array([2.0, 2.0, 6.0]), np.array([5.0])]
    fine0 = np.full(9, -7.0)
    fine = O.refine_project(cs, fs, np.array([1.0, 2.0]), fine0).reshape(3, 3, 1)
    assert np.all(fine[:2, :2] == 1.0) and np.all(fine[:2, 2] == 2.0)
    assert np.all(fine[2] == -7.0)
    assert np.array_equal(O.refine_combine(cs, fs, np.arange(9.0)), [0 + 1 + 3 + 4, 2 + 5])
    # refinement coordinates equal to coarse corners
    f = O.refine_axis([0.0, 10.0, 20.0], [10.0, 10.0], [0.0, 5.0, 10.0, 15.0, 20.0])
    assert np.array_equal(f, [5.0, 5.0, 5.0, 5.0])
    cs2 = [np.array([10.0]), np.array([1.0]), np.array([3.0, 3.0])]
    fs2 = [np.array([10.0]), np.array([1.0]), np.array([3.0, 3.0, 1.0])]
    assert np.array_equal(O.refine_combine(cs2, fs2, np.array([1.0, 2.0, 4.0])), [1.0, 2.0])
    cs3 = [np.array([1.0]), np.array([1.0]), np.array([3.0, 3.0, 2.0])]
    fs3 = [np.array([1.0]), np.array([1.0]), np.array([4.0, 4.0])]
    assert np.array_equal(O.refine_combine(cs3, fs3, np.array([1.0, 2.0])), [1.0, 2.0, 0.0])


def test_capi_refine_axis_matches_oracle(oracle_lib):
    """j3g_refine_axis (host code of the library) against the oracle on
    irregular axes with rounding in the corner sums (bit-exact)."""
    from jif3d_gb300 import capi
    O = oracle_lib
    rng = np.random.default_rng(77)
    for t in range(200):
        n = int(rng.integers(1, 9))
        c = rng.uniform(0.05, 3.0, n).round(int(rng.integers(1, 4)))
        cc = O.corners(round(float(rng.uniform(-5, 5)), 2), c)
        r = np.sort(rng.uniform(cc[0] - 1, cc[-1] + 1, int(rng.integers(1, 30))).round(2))
        if t % 3 == 0:
            r = np.unique(np.concatenate([r, cc[rng.integers(0, n, 2)]]))
        ref = O.refine_axis(cc, c, r)
        if ref is None:
            with pytest.raises(capi.J3GError):
                capi.refine_axis(cc, c, r)
            continue
        got = capi.refine_axis(cc, c, r)
        assert np.array_equal(got, ref), (cc, c, r)
    with pytest.raises(capi.J3GError):
        capi.refine_axis([0.0, 1.0], [1.0], [])
    # a last coarse cell of zero size leaves a last refined cell of zero size:
    # the reference throws (ModelRefiner.cpp:63-71)
    assert O.refine_axis([0.0, 10.0, 10.0], [10.0, 0.0], [0.0, 5.0, 10.0]) is None
    with pytest.raises(capi.J3GError):
        capi.refine_axis([0.0, 10.0, 10.0], [10.0, 0.0], [0.0, 5.0, 10.0])
