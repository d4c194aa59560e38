"""The GPU implementations inside an L-BFGS inversion loop, unchanged.

jif3D's inversion (Inversion/LimitedMemoryQuasiNewton.cpp:32-117) only calls
the objective's CalcMisfit and CalcGradient (Inversion/ObjectiveFunction.h:
160-229) in a quasi-Newton loop; the implementations sit below the
calculators that ThreeDModelObjective holds.  Here a joint g_z + FTG
objective (one ThreeDModelObjective per data set, summed as jif3D's
JointObjective does with unit weights) over the GPU implementations is
minimised with scipy's L-BFGS-B for ten iterations, and the same loop runs on
an objective of the same formulas over the oracle.  The FP64 matrix-free
calculators must give the oracle's iterates and misfits within 1e-8 relative.
The device-resident calculator (stored FP32 sensitivities, each product
within 1e-6 of FP64) must give the iterates within 1e-5, since the iteration
carries each evaluation's error forward, and the misfits within 1e-3: chi^2
sums squares of the data residuals, which are a few per cent of the data
once the loop has fitted them, so the data's relative error of up to 1e-6 is
amplified about a hundredfold in it.
"""
import numpy as np
import pytest

from helpers import oracle_forward, oracle_lqderivative, small_survey
from jif3d_gb300 import gravmag as G, inversion as I, workloads as W

pytestmark = pytest.mark.gpu
ITERATIONS = 10


def gravity_model(s, values):
    nx, ny, nz = s.shape
    M = G.ThreeDGravityModel()
    M.SetMeshSize(nx, ny, nz)
    M.SetData()[...] = values[:s.ngrid].reshape(nx, ny, nz)
    M.SetBackgroundThicknesses(s.bg_thick)
    M.SetBackgroundValues(values[s.ngrid:])
    M.SetXCellSizes(s.xsize)
    M.SetYCellSizes(s.ysize)
    M.SetZCellSizes(s.zsize)
    M.SetOrigin(*s.origin)
    return M


def survey_and_data(oracle_lib):
    """A small joint survey: its scalar and tensor views, the observed data
    of a true model (oracle) with 2 % noise, and their errors."""
    s = small_survey(W.SCALAR, seed=321, nx=8, ny=7, nz=5, nmeas=14)
    t = small_survey(W.TENSOR, seed=321, nx=8, ny=7, nz=5, nmeas=14)
    rng = np.random.default_rng(5)
    truth = s.model * rng.uniform(0.5, 1.5, s.model.size)
    obs = {}
    for v in (s, t):
        d = oracle_forward(oracle_lib, v, truth)
        err = 0.02 * np.abs(d) + 1e-3 * np.abs(d).max()
        obs[v.kind] = (d + err * rng.normal(size=d.size), err)
    return s, t, obs


class OracleObjective:
    """chi^2 = sum ((d(m) - d_obs) / err)^2 and its gradient
    2 J^T ((d - d_obs) / err^2) from the oracle, the formulas of
    ObjectiveFunction::CalcMisfit / CalcGradient."""

    def __init__(self, O, surveys, obs):
        self.O, self.surveys, self.obs = O, surveys, obs

    def __call__(self, m):
        chi, grad = 0.0, np.zeros(m.size)
        for v in self.surveys:
            d_obs, err = self.obs[v.kind]
            diff = oracle_forward(self.O, v, m) - d_obs
            chi += float(np.sum(diff * diff / err ** 2))
            grad += oracle_lqderivative(self.O, v, diff / err ** 2, m)
        return chi, grad


class GPUObjective:
    """The sum of one ThreeDModelObjective per data set over GPU calculators."""

    def __init__(self, s, t, obs, make_calc):
        self.objs = []
        for v, imp, DataT in ((s, G.ScalarGB300GravityImp, G.ScalarGravityData),
                              (t, G.TensorGB300GravityImp, G.TensorGravityData)):
            D = DataT()
            for x, y, z in v.stations:
                D.AddMeasurementPoint(x, y, z)
            D.SetDataAndErrors(*obs[v.kind])
            obj = I.ThreeDModelObjective(make_calc(imp()))
            obj.SetObservedData(D)
            obj.SetCoarseModelGeometry(gravity_model(v, v.model))
            self.objs.append(obj)

    def __call__(self, m):
        chi = sum(o.CalcMisfit(m) for o in self.objs)
        grad = sum(o.CalcGradient(m) for o in self.objs)
        return chi, np.asarray(grad)


def lbfgs(fun, m0):
    """Ten L-BFGS iterations; the iterates and the misfit at each."""
    from scipy.optimize import minimize
    xs, fs = [], []

    def f(m):
        chi, g = fun(m)
        return chi, g

    def record(xk):
        xs.append(np.array(xk))
        fs.append(fun(xk)[0])

    minimize(f, m0, jac=True, method="L-BFGS-B", callback=record,
             options={"maxiter": ITERATIONS, "maxcor": 5, "ftol": 0.0, "gtol": 0.0})
    return np.array(xs), np.array(fs)


@pytest.mark.parametrize("calc,tol,ftol", [("minmem", 1e-8, 1e-8), ("device", 1e-5, 1e-3)])
def test_lbfgs_iterates_match_oracle(oracle_lib, calc, tol, ftol):
    pytest.importorskip("scipy")
    s, t, obs = survey_and_data(oracle_lib)
    m0 = s.model.copy()
    x_ref, f_ref = lbfgs(OracleObjective(oracle_lib, (s, t), obs), m0)
    make = (G.MinMemGravMagCalculator if calc == "minmem" else
            (lambda imp: G.DeviceSensitivityGravMagCalculator(imp)))
    x_gpu, f_gpu = lbfgs(GPUObjective(s, t, obs, make), m0)
    assert len(x_ref) == ITERATIONS and len(x_gpu) == ITERATIONS
    chi0 = OracleObjective(oracle_lib, (s, t), obs)(m0)[0]
    assert f_ref[-1] < 0.5 * chi0  # the loop makes progress
    for k in range(ITERATIONS):
        ex = np.linalg.norm(x_gpu[k] - x_ref[k]) / np.linalg.norm(x_ref[k])
        ef = abs(f_gpu[k] - f_ref[k]) / f_ref[k]
        assert ex <= tol and ef <= ftol, (k, ex, ef)
