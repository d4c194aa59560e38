"""The objective function over the GPU calculators with a refined forward
grid (Inversion/ThreeDModelObjective.h with ObjectiveFunction.h:160-229),
against the oracle: chi^2 and its gradient with respect to the coarse
parameters (FP64 path: relative error <= 1e-10), central differences of
chi^2, and the refiner mirror (bit-exact).
"""
import numpy as np
import pytest

from helpers import oracle_forward, oracle_lqderivative, relerr, small_survey
from jif3d_gb300 import gravmag as G, inversion as I, workloads as W
import dataclasses

pytestmark = pytest.mark.gpu
TOL = 1e-10


def model_of(s, values=None):
    """The model object of survey s (gravity / susceptibility / magnetisation)."""
    values = s.model if values is None else values
    nx, ny, nz = s.shape
    if s.kind == W.MAGNETIZATION:
        M = G.ThreeDMagnetizationModel()
        M.SetMeshSize(nx, ny, nz)
        M.SetMagnetization_X()[...] = values[:s.ngrid].reshape(nx, ny, nz)
        M.SetMagnetization_Y()[...] = values[s.ngrid:2 * s.ngrid].reshape(nx, ny, nz)
        M.SetMagnetization_Z()[...] = values[2 * s.ngrid:].reshape(nx, ny, nz)
    else:
        M = G.ThreeDGravityModel() if s.kind in (W.SCALAR, W.TENSOR) else \
            G.ThreeDSusceptibilityModel()
        M.SetMeshSize(nx, ny, nz)
        M.SetData()[...] = values[:s.ngrid].reshape(nx, ny, nz)
        M.SetBackgroundThicknesses(s.bg_thick)
        M.SetBackgroundValues(values[s.ngrid:])
    M.SetXCellSizes(s.xsize)
    M.SetYCellSizes(s.ysize)
    M.SetZCellSizes(s.zsize)
    M.SetOrigin(*s.origin)
    return M


IMPS = {W.SCALAR: (G.ScalarGB300GravityImp, G.ScalarGravityData),
        W.TENSOR: (G.TensorGB300GravityImp, G.TensorGravityData),
        W.MAGNETIZATION: (G.GB300MagnetizationImp, G.ThreeComponentMagneticData)}


def halves(s):
    """Fine-model corners that split every coarse cell in two along each axis."""
    out = []
    for a in range(3):
        c = s.coords(a)
        out.append(np.sort(np.concatenate([c, c[:-1] + 0.5 * np.diff(c)])))
    return out


def refined_survey(s, refs):
    from jif3d_gb300 import capi
    fs = [capi.refine_axis(s.coords(a), (s.xsize, s.ysize, s.zsize)[a], refs[a])
          for a in range(3)]
    return dataclasses.replace(s, xsize=fs[0], ysize=fs[1], zsize=fs[2])


def project(O, s, f, values, nblock):
    cg, fg = s.ngrid, f.ngrid
    cs, fs = [s.xsize, s.ysize, s.zsize], [f.xsize, f.ysize, f.zsize]
    blocks = [O.refine_project(cs, fs, values[b * cg:(b + 1) * cg]) for b in range(nblock)]
    return np.concatenate(blocks + [values[nblock * cg:]])


def combine(O, s, f, grad, nblock):
    cg, fg = s.ngrid, f.ngrid
    cs, fs = [s.xsize, s.ysize, s.zsize], [f.xsize, f.ysize, f.zsize]
    blocks = [O.refine_combine(cs, fs, grad[b * fg:(b + 1) * fg]) for b in range(nblock)]
    return np.concatenate(blocks + [grad[nblock * fg:]])


@pytest.mark.parametrize("kind", [W.SCALAR, W.TENSOR, W.MAGNETIZATION])
def test_objective_with_refinement(oracle_lib, kind):
    O = oracle_lib
    s = small_survey(kind, seed=80 + kind, nx=4, ny=3, nz=3, nmeas=6,
                     bg=kind != W.MAGNETIZATION)
    rng = np.random.default_rng(kind)
    if kind == W.MAGNETIZATION:
        s.model = rng.uniform(-2, 2, 3 * s.ngrid)
    nblock = 3 if kind == W.MAGNETIZATION else 1
    f = refined_survey(s, halves(s))
    imp, DataT = IMPS[kind]
    D = DataT()
    for x, y, z in s.stations:
        D.AddMeasurementPoint(x, y, z)
    fine_truth = project(O, s, f, s.model, nblock)
    dtrue = oracle_forward(O, f, fine_truth)
    err = 0.02 * np.abs(dtrue) + 1e-3 * np.abs(dtrue).max()
    D.SetDataAndErrors(dtrue * (1 + 0.05 * rng.normal(size=dtrue.size)), err)

    obj = I.ThreeDModelObjective(G.MinMemGravMagCalculator(imp()))
    obj.SetObservedData(D)
    obj.SetCoarseModelGeometry(model_of(s))
    obj.SetFineModelGeometry(model_of(f, np.zeros(f.nparm)))
    m = s.model * rng.uniform(0.8, 1.2, s.model.size)

    chi = obj.CalcMisfit(m)
    fm = project(O, s, f, m, nblock)
    dsyn = oracle_forward(O, f, fm)
    w = (dsyn - D.GetData()) / err ** 2
    ref_chi = float(np.sum((dsyn - D.GetData()) ** 2 / err ** 2))
    assert abs(chi - ref_chi) <= TOL * ref_chi
    assert relerr(obj.GetSyntheticData(), dsyn) <= TOL
    g = obj.CalcGradient(m)
    gref = combine(O, s, f, oracle_lqderivative(O, f, w, fm), nblock)
    assert g.size == m.size
    assert relerr(g, gref) <= TOL
    # central differences of chi^2 in two coarse cells and one extra parameter
    for i in (0, s.ngrid - 1, m.size - 1):
        h = 1e-4 * max(1.0, abs(m[i]))
        mp, mm = m.copy(), m.copy()
        mp[i] += h
        mm[i] -= h
        fd = (I.ThreeDModelObjective.CalcMisfit(obj, mp) -
              I.ThreeDModelObjective.CalcMisfit(obj, mm)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * max(abs(fd), abs(g[i])) + 1e-12, (i, fd, g[i])


def test_objective_without_refinement_and_errors(oracle_lib):
    s = small_survey(W.SCALAR, seed=90, nx=4, ny=4, nz=3, nmeas=5)
    D = G.ScalarGravityData()
    for x, y, z in s.stations:
        D.AddMeasurementPoint(x, y, z)
    d = oracle_forward(oracle_lib, s)
    D.SetDataAndErrors(d * 1.1, np.full(d.size, 1e-8))
    obj = I.ThreeDModelObjective(G.MinMemGravMagCalculator(G.ScalarGB300GravityImp()))
    obj.SetObservedData(D)
    obj.SetCoarseModelGeometry(model_of(s))
    chi = obj.CalcMisfit(s.model)
    assert abs(chi - float(np.sum((0.1 * d / 1e-8) ** 2))) <= 1e-10 * chi
    g = obj.CalcGradient(s.model)
    assert relerr(g, oracle_lqderivative(oracle_lib, s, -0.1 * d / 1e-16)) <= TOL
    with pytest.raises(G.FatalException):  # the gradient needs the model of the misfit
        obj.CalcGradient(s.model * 1.01)
    with pytest.raises(G.FatalException):
        obj.CalcMisfit(s.model[:5])
    with pytest.raises(G.FatalException):
        I.ThreeDModelObjective(None).SetObservedData(G.ScalarGravityData())


def test_refiner_mirror(oracle_lib):
    """The ModelRefiner mirror on the reference's refiner case: axes, the
    projected iota and the combined unit gradient (60 everywhere)."""
    M = G.ThreeDGravityModel()
    M.SetMeshSize(2, 3, 5)
    M.SetXCellSizes(np.full(2, 50.0))
    M.SetYCellSizes(np.full(3, 40.0))
    M.SetZCellSizes(np.full(5, 30.0))
    M.SetData()[...] = np.arange(30.0).reshape(2, 3, 5)
    F = G.ThreeDGravityModel()
    R = I.ModelRefiner()
    R.SetXCoordinates(10.0 * np.arange(20))
    R.SetYCoordinates(20.0 * np.arange(20))
    R.SetZCoordinates(5.0 * np.arange(50))
    R.RefineModel(M, F)
    assert F.GetData().shape == (10, 6, 30)
    cs = [M.GetXCellSizes(), M.GetYCellSizes(), M.GetZCellSizes()]
    fs = [F.GetXCellSizes(), F.GetYCellSizes(), F.GetZCellSizes()]
    assert np.array_equal(F.GetData().ravel(), oracle_lib.refine_project(cs, fs, np.arange(30.0)))
    assert np.all(R.CombineGradient(np.ones(F.GetData().size), M, F) == 60.0)
