"""GPU parity of the vertical magnetic gradient (OMPMagneticGradImp) and of
remanent magnetisation (OMPMagnetizationImp) against the oracle.

Tolerance (FP64 path): relative norm error <= 1e-10 per output group, as for
the other kinds.  Both kinds run through the node-term kernels (virtual
components: the gradient evaluates every node at the station and 1 m below
it; magnetisation accumulates U_kj against three model blocks) and through
the eight-corner path when the mesh corners are not running sums.  Their
device-resident sensitivity (batched stored products) is checked at the
mixed-path tolerance, 1e-6.
"""
import numpy as np
import pytest

from helpers import oracle_forward, oracle_lqderivative, relerr, small_survey
from jif3d_gb300 import capi, workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-10


def survey(kind, seed, bg=True, transform=W.T_NONE, **kw):
    s = small_survey(kind, seed=seed, bg=bg and kind == W.MAG_GRADIENT, transform=transform,
                     **kw)
    if kind == W.MAGNETIZATION:
        rng = np.random.default_rng(seed + 1000)
        s.model = rng.uniform(-2.0, 2.0, 3 * s.ngrid)
    return s


def setup(ctx, s):
    W.setup_context(ctx, s)
    return ctx


@pytest.mark.parametrize("kind", [W.MAG_GRADIENT, W.MAGNETIZATION])
def test_forward_rows_and_gradient(ctx, oracle_lib, kind):
    s = survey(kind, seed=300 + kind, nx=8, ny=7, nz=6, nmeas=11)
    c = setup(ctx, s)
    assert c.sizes()["nparm"] == s.nparm
    d = c.forward(s.model)
    dref, Jref = oracle_forward(oracle_lib, s, want_sens=True)
    assert relerr(d, dref) <= TOL, relerr(d, dref)
    d2, J = c.forward_sens(s.model)
    assert J.shape == Jref.shape
    for r in range(J.shape[0]):
        assert relerr(J[r], Jref[r]) <= TOL, (r, relerr(J[r], Jref[r]))
    assert relerr(d2, dref) <= TOL
    misfit = np.random.default_rng(kind).normal(size=d.size)
    g = c.lqderivative(s.model, misfit)
    gref = oracle_lqderivative(oracle_lib, s, misfit)
    assert relerr(g, gref) <= TOL, relerr(g, gref)
    if kind == W.MAG_GRADIENT:
        # background parameters: zero sensitivity and zero gradient
        assert np.all(J[:, s.ngrid:] == 0.0) and np.all(g[s.ngrid:] == 0.0)


@pytest.mark.parametrize("transform", [W.T_TOTAL_FIELD, W.T_TFA])
def test_magnetization_transforms(ctx, oracle_lib, transform):
    s = survey(W.MAGNETIZATION, seed=320 + transform, transform=transform, nx=7, ny=6, nz=5)
    c = setup(ctx, s)
    d = c.forward(s.model)
    assert relerr(d, oracle_forward(oracle_lib, s)) <= TOL
    misfit = np.random.default_rng(transform).normal(size=d.size)
    assert relerr(c.lqderivative(s.model, misfit),
                  oracle_lqderivative(oracle_lib, s, misfit)) <= TOL


@pytest.mark.parametrize("kind", [W.MAG_GRADIENT, W.MAGNETIZATION])
def test_corner_path(ctx, oracle_lib, kind):
    """Corner coordinates that are not running sums: eight-corner evaluation."""
    s = survey(kind, seed=340 + kind, origin=(0.1, 0.2, 0.0))
    s.xsize = s.xsize + 0.1 / 3.0
    xc = s.coords(0)
    xc[1:-1] += np.array([1e-9, -2e-9, 3e-9, 0.0, 1e-9, 0.0])[: xc.size - 2]
    c = setup(ctx, s)
    c.set_mesh(xc, s.coords(1), s.coords(2), s.xsize, s.ysize, s.zsize)
    d = c.forward(s.model)
    O = oracle_lib
    p = O.Problem(xc, s.coords(1), s.coords(2), s.xsize, s.ysize, s.zsize, s.stations,
                  kind=kind, bg_thick=s.bg_thick, inc=s.inc, dec=s.dec, fs=s.fs)
    assert relerr(d, p.forward(s.model)) <= TOL
    misfit = np.random.default_rng(3).normal(size=d.size)
    assert relerr(c.lqderivative(s.model, misfit), p.lqderivative(s.model, misfit)) <= TOL


STORED_CASES = [(W.MAG_GRADIENT, W.T_NONE), (W.MAGNETIZATION, W.T_NONE),
                (W.MAGNETIZATION, W.T_TOTAL_FIELD), (W.MAGNETIZATION, W.T_TFA)]


@pytest.mark.parametrize("storage", [capi.STORE_FP32, capi.STORE_F16X2])
@pytest.mark.parametrize("kind,transform", STORED_CASES)
def test_stored_sensitivity(ctx, oracle_lib, kind, transform, storage):
    """Device-resident J of both kinds (raw rows: 1 per station for the
    gradient, 3 over the three magnetisation blocks): batched products
    against the oracle at the mixed-path tolerance, 1e-6."""
    s = survey(kind, seed=380 + 10 * kind + transform, transform=transform, nx=9, ny=8, nz=6,
               nmeas=13)
    c = setup(ctx, s)
    c.build_sensitivity(storage)
    info = c.sensitivity_info()
    assert info["storage"] == storage
    assert info["cols"] == (3 if kind == W.MAGNETIZATION else 1) * s.ngrid
    rng = np.random.default_rng(kind + transform)
    models = s.model[None, :] * (1 + 0.2 * rng.normal(size=(4, s.nparm)))
    d = c.batched_forward(models)
    mis = rng.normal(size=d.shape)
    g = c.batched_lqderivative(models, mis)
    for i in range(models.shape[0]):
        assert relerr(d[i], oracle_forward(oracle_lib, s, models[i])) <= 1e-6
        gref = oracle_lqderivative(oracle_lib, s, mis[i], models[i])
        assert relerr(g[i], gref) <= 1e-6
        if kind == W.MAG_GRADIENT:
            assert np.all(g[i, s.ngrid:] == 0.0)  # background parameters: no response


def test_unsupported_combinations(ctx):
    g = survey(W.MAG_GRADIENT, seed=361)
    c = setup(ctx, g)
    with pytest.raises(capi.J3GError):  # the gradient has no total-field transform
        c.set_transform(W.T_TOTAL_FIELD)
    with pytest.raises(capi.J3GError):
        c.forward(np.zeros(3 * g.ngrid))  # wrong model length


def test_magnetization_larger_mesh_adjoint_identity(ctx):
    """<J m, r> = <m, J^T r> on a larger magnetisation survey (node path)."""
    s = survey(W.MAGNETIZATION, seed=370, nx=24, ny=20, nz=12, nmeas=60)
    c = setup(ctx, s)
    d = c.forward(s.model)
    r = np.random.default_rng(5).normal(size=d.size)
    g = c.lqderivative(s.model, r)  # 2 J^T r (linear, no transform)
    lhs, rhs = float(d @ r), 0.5 * float(s.model @ g)
    assert abs(lhs - rhs) <= 1e-11 * np.linalg.norm(d) * np.linalg.norm(r)
