"""The jif3D calculator chain over the GB300 implementations (Python mirror of
GravMag/*Calculator.h): MinMem, FullSensitivity (host J filled through
HandleSensitivities), and the device-resident twin; the objective gradient
through a calculator for the magnetic kinds, as the reference's objective
tests do (test_MagneticGradObjective.cpp:72-110, test_MagneticObjective.cpp:176-211).

Tolerances: FP64 paths 1e-10 (relative norm), device-stored products 1e-6.
"""
import numpy as np
import pytest

from helpers import oracle_forward, oracle_lqderivative, relerr, small_survey
from jif3d_gb300 import capi, gravmag as G, workloads as W

pytestmark = pytest.mark.gpu
TOL, TOL_MIXED = 1e-10, 1e-6

IMPS = {W.SCALAR: lambda s: G.ScalarGB300GravityImp(),
        W.TENSOR: lambda s: G.TensorGB300GravityImp(),
        W.MAGNETIC: lambda s: G.GB300MagneticSusceptibilityImp(s.inc, s.dec, s.fs),
        W.MAG_GRADIENT: lambda s: G.GB300MagneticGradImp(s.inc, s.dec, s.fs),
        W.MAGNETIZATION: lambda s: G.GB300MagnetizationImp()}


def model_and_data(s, model=None):
    model = s.model if model is None else model
    nx, ny, nz = s.shape
    if s.kind == W.MAGNETIZATION:
        M = G.ThreeDMagnetizationModel()
        M.SetMeshSize(nx, ny, nz)
        M.SetMagnetization_X()[...] = model[:s.ngrid].reshape(nx, ny, nz)
        M.SetMagnetization_Y()[...] = model[s.ngrid:2 * s.ngrid].reshape(nx, ny, nz)
        M.SetMagnetization_Z()[...] = model[2 * s.ngrid:].reshape(nx, ny, nz)
        D = G.ThreeComponentMagneticData()
    else:
        M = (G.ThreeDGravityModel() if s.kind in (W.SCALAR, W.TENSOR)
             else G.ThreeDSusceptibilityModel())
        M.SetMeshSize(nx, ny, nz)
        M.SetData()[...] = model[:s.ngrid].reshape(nx, ny, nz)
        M.SetBackgroundThicknesses(s.bg_thick)
        M.SetBackgroundValues(model[s.ngrid:])
        D = {W.SCALAR: G.ScalarGravityData, W.TENSOR: G.TensorGravityData}.get(
            s.kind, G.TotalFieldMagneticData)()
    M.SetXCellSizes(s.xsize)
    M.SetYCellSizes(s.ysize)
    M.SetZCellSizes(s.zsize)
    M.SetOrigin(*s.origin)
    for x, y, z in s.stations:
        D.AddMeasurementPoint(x, y, z)
    return M, D


def survey(kind, seed, **kw):
    s = small_survey(kind, seed=seed, bg=kind != W.MAGNETIZATION, **kw)
    if kind == W.MAGNETIZATION:
        s.model = np.random.default_rng(seed).uniform(-2, 2, 3 * s.ngrid)
    return s


@pytest.mark.parametrize("kind", [W.SCALAR, W.TENSOR, W.MAGNETIC])
def test_calculators_agree_with_oracle(oracle_lib, kind):
    s = survey(kind, seed=400 + kind, nx=9, ny=8, nz=6, nmeas=13)
    M, D = model_and_data(s)
    dref, Jref = oracle_forward(oracle_lib, s, want_sens=True)
    misfit = np.random.default_rng(kind).normal(size=dref.size)
    gref = oracle_lqderivative(oracle_lib, s, misfit)

    minmem = G.MinMemGravMagCalculator(IMPS[kind](s))
    assert relerr(minmem.Calculate(M, D), dref) <= TOL
    assert relerr(minmem.LQDerivative(M, D, misfit), gref) <= TOL

    full = G.FullSensitivityGravMagCalculator(IMPS[kind](s))
    d1 = full.Calculate(M, D)  # fills Sensitivities through HandleSensitivities
    assert relerr(d1, dref) <= TOL
    J = full.GetSensitivities()
    assert J.shape == Jref.shape
    # norm-wise per output group (the FP64 bound); single rows with strong
    # cancellation between corner terms amplify libm last-bit differences
    assert relerr(J, Jref) <= TOL
    for r in range(J.shape[0]):
        assert relerr(J[r], Jref[r]) <= 1e-8
    d2 = full.Calculate(M, D)  # cached: J m on the host
    assert relerr(d2, dref) <= TOL
    assert relerr(full.LQDerivative(M, D, misfit), gref) <= TOL

    dev = G.DeviceSensitivityGravMagCalculator(IMPS[kind](s), capi.STORE_FP32)
    assert relerr(dev.Calculate(M, D), dref) <= TOL        # first call: FP64, builds J
    assert relerr(dev.Calculate(M, D), dref) <= TOL_MIXED  # stored product in HBM
    assert relerr(dev.LQDerivative(M, D, misfit), gref) <= TOL_MIXED


def test_device_calculator_f16x2_and_new_model(oracle_lib):
    s = survey(W.TENSOR, seed=410, nx=10, ny=9, nz=7, nmeas=15)
    M, D = model_and_data(s)
    dev = G.DeviceSensitivityGravMagCalculator(G.TensorGB300GravityImp(), capi.STORE_F16X2)
    dev.Calculate(M, D)
    m2 = s.model * np.random.default_rng(1).uniform(0.5, 1.5, s.model.size)
    M2, _ = model_and_data(s, m2)
    assert relerr(dev.Calculate(M2, D), oracle_forward(oracle_lib, s, m2)) <= TOL_MIXED


def test_device_cache_key_includes_stations(oracle_lib):
    """Moving the stations rebuilds the device J.  The reference's
    GridBackgroundModelCache keys only on cell sizes and background
    (ModelBase/GridBackgroundModelCache.h:37-85), so its cached calculators
    keep returning J m of the old stations; the host mirror keeps that
    behaviour."""
    s = survey(W.SCALAR, seed=420, nmeas=10)
    M, D = model_and_data(s)
    dev = G.DeviceSensitivityGravMagCalculator(G.ScalarGB300GravityImp())
    full = G.FullSensitivityGravMagCalculator(G.ScalarGB300GravityImp())
    dev.Calculate(M, D)
    old = full.Calculate(M, D)
    moved = s.subset(np.arange(s.stations.shape[0]))
    moved.stations = s.stations + np.array([3.0, -2.0, -5.0])
    _, D2 = model_and_data(moved)
    ref = oracle_forward(oracle_lib, moved)
    assert relerr(dev.Calculate(M, D2), ref) <= TOL  # recomputed in FP64
    assert relerr(full.Calculate(M, D2), old) <= 1e-12  # the reference's stale cache


@pytest.mark.parametrize("kind", [W.MAG_GRADIENT, W.MAGNETIZATION])
def test_objective_gradient_through_calculator(oracle_lib, kind):
    """Least-squares objective of observed = 1.1 x synthetic data: the
    calculator's LQDerivative against central differences (step 1 %, 0.01 %),
    and against the oracle."""
    s = survey(kind, seed=430 + kind, nx=4, ny=3, nz=3, nmeas=3)
    calc = G.MinMemGravMagCalculator(IMPS[kind](s))
    M, D = model_and_data(s)
    obs = calc.Calculate(M, D) * 1.1

    def phi(model):
        Mi, _ = model_and_data(s, model)
        d = calc.Calculate(Mi, D)
        return float(np.sum((d - obs) ** 2)), d

    _, d0 = phi(s.model)
    grad = calc.LQDerivative(M, D, d0 - obs)
    assert relerr(grad, oracle_lqderivative(oracle_lib, s, d0 - obs)) <= TOL
    for i in range(s.ngrid if kind == W.MAG_GRADIENT else s.model.size):
        delta = abs(s.model[i]) * 0.01
        if delta < 1e-3:  # the reference skips parameters it cannot step (delta > 0)
            continue
        mp, mm = s.model.copy(), s.model.copy()
        mp[i] += delta
        mm[i] -= delta
        fd = (phi(mp)[0] - phi(mm)[0]) / (2 * delta)
        assert abs(fd - grad[i]) <= 1e-4 * max(abs(fd), abs(grad[i])) + 1e-30, (i, fd, grad[i])


def test_ftg_invariant_through_calculators(oracle_lib):
    s = survey(W.TENSOR, seed=440, nx=8, ny=7, nz=5, transform=W.T_FTG_INVARIANT)
    M, D = model_and_data(s)
    dref = oracle_forward(oracle_lib, s)
    misfit = np.random.default_rng(7).normal(size=dref.size)
    gref = oracle_lqderivative(oracle_lib, s, misfit)
    for calc, tol in ((G.FullSensitivityGravMagCalculator(G.TensorGB300GravityImp()), TOL),
                      (G.DeviceSensitivityGravMagCalculator(G.TensorGB300GravityImp()),
                       TOL_MIXED)):
        calc.SetDataTransform(G.FTGInvariant())
        assert relerr(calc.Calculate(M, D), dref) <= TOL
        assert relerr(calc.Calculate(M, D), dref) <= tol      # cached
        assert relerr(calc.LQDerivative(M, D, misfit), gref) <= tol
