"""The data of jif3D's Tutorial 5 through the GPU path: the netCDF-4 gravity
and total-field magnetic files (tests/golden/tutorial5_*.nc) are read with the
library's own reader, a mesh covering the survey area is built, and the
forward responses at the tutorial's 760 gravity and 748 magnetic stations
(inducing field of the tutorial's run: inclination 1.17, declination 0.22,
52671 nT) are compared with the oracle (FP64 path, relative error <= 1e-10);
the synthetic data are written back and read again."""
import os

import numpy as np
import pytest

from helpers import relerr
from jif3d_gb300 import gravmag as G, netcdf as N, workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-10


def survey_mesh(x, y, cls, nz=6, seed=0):
    """A 16 x 14 x nz mesh (integer sizes, so corners are exact sums)
    covering the stations with a 20 km margin."""
    rng = np.random.default_rng(seed)
    x0, y0 = np.floor(x.min()) - 20000.0, np.floor(y.min()) - 20000.0
    wx = np.ceil((x.max() + 20000.0 - x0) / 16)
    wy = np.ceil((y.max() + 20000.0 - y0) / 14)
    M = cls()
    M.SetMeshSize(16, 14, nz)
    M.SetXCellSizes(np.full(16, wx))
    M.SetYCellSizes(np.full(14, wy))
    M.SetZCellSizes(np.array([2000.0 * 1.5 ** k for k in range(nz)]).round())
    M.SetOrigin(x0, y0, 0.0)
    return M, rng


def oracle_problem(M, D, kind, **kw):
    st = np.stack([D.GetMeasPosX(), D.GetMeasPosY(), D.GetMeasPosZ()], axis=1)
    return O.Problem(M.GetXCoordinates(), M.GetYCoordinates(), M.GetZCoordinates(),
                     M.GetXCellSizes(), M.GetYCellSizes(), M.GetZCellSizes(), st, kind=kind,
                     bg_thick=M.GetBackgroundThicknesses(), **kw)


def test_tutorial_gravity_data(tmp_path):
    D = G.ScalarGravityData()
    D.ReadNetCDF(os.path.join(GOLDEN, "tutorial5_gravdata.nc"))
    assert D.GetMeasPosX().size == 760
    M, rng = survey_mesh(D.GetMeasPosX(), D.GetMeasPosY(), G.ThreeDGravityModel)
    M.SetData()[...] = rng.normal(0, 100, M.GetData().shape)  # kg/m3 contrasts
    M.SetBackgroundThicknesses([30000.0])
    M.SetBackgroundValues([300.0])
    calc = G.MinMemGravMagCalculator(G.ScalarGB300GravityImp())
    d = calc.Calculate(M, D)
    ref = oracle_problem(M, D, O.SCALAR).forward(M.GetModelParameters())
    assert relerr(d, ref) <= TOL
    misfit = d - D.GetData()
    g = calc.LQDerivative(M, D, misfit)
    assert relerr(g, oracle_problem(M, D, O.SCALAR).lqderivative(M.GetModelParameters(),
                                                                  misfit)) <= TOL
    out = str(tmp_path / "synthetic_grav.nc")
    N.SaveScalarGravityMeasurements(out, d, D.GetMeasPosX(), D.GetMeasPosY(),
                                    D.GetMeasPosZ(), D.GetErrors())
    assert np.array_equal(N.ReadScalarGravityMeasurements(out)[0], d)
    model_file = str(tmp_path / "start_grav.nc")
    M.WriteNetCDF(model_file)
    M2 = G.ThreeDGravityModel()
    M2.ReadNetCDF(model_file)
    assert np.array_equal(calc.Calculate(M2, D), d)


def test_tutorial_magnetic_data():
    D = G.TotalFieldMagneticData()
    D.ReadNetCDF(os.path.join(GOLDEN, "tutorial5_magdata.nc"))
    assert D.GetMeasPosX().size == 748
    M, rng = survey_mesh(D.GetMeasPosX(), D.GetMeasPosY(), G.ThreeDSusceptibilityModel, seed=1)
    M.SetData()[...] = np.clip(rng.normal(0.01, 0.01, M.GetData().shape), 0, None)
    inc, dec, fs = 1.17, 0.22, 52671.0
    calc = G.MinMemGravMagCalculator(G.GB300MagneticSusceptibilityImp(inc, dec, fs))
    calc.SetDataTransform(G.TotalFieldAnomaly(inc, dec))
    d = calc.Calculate(M, D)
    p = oracle_problem(M, D, O.MAGNETIC, inc=inc, dec=dec, fs=fs, transform=W.T_TFA,
                       t_inc=inc, t_dec=dec)
    assert relerr(d, p.forward(M.GetModelParameters())) <= TOL
    misfit = d - D.GetData()
    assert relerr(calc.LQDerivative(M, D, misfit),
                  p.lqderivative(M.GetModelParameters(), misfit)) <= TOL
