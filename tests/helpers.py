"""Shared helpers of the parity tests: run a Survey through the oracle and
through the GPU library, and the error measures used in the assertions."""
import numpy as np

from jif3d_gb300 import workloads as W


def oracle_problem(O, s, kind=None, transform=None):
    kind = s.kind if kind is None else kind
    transform = s.transform if transform is None else transform
    return O.Problem(s.coords(0), s.coords(1), s.coords(2), s.xsize, s.ysize, s.zsize,
                     s.stations, kind=kind, bg_thick=s.bg_thick, inc=s.inc, dec=s.dec,
                     fs=s.fs, transform=transform, t_inc=s.t_inc, t_dec=s.t_dec)


def oracle_forward(O, s, model=None, want_sens=False):
    """Oracle forward; the joint kind is the scalar and tensor oracles side by side."""
    model = s.model if model is None else model
    if s.kind != W.JOINT:
        return oracle_problem(O, s).forward(model, want_sens)
    g = oracle_problem(O, s, W.SCALAR, W.T_NONE).forward(model, want_sens)
    t = oracle_problem(O, s, W.TENSOR, W.T_NONE).forward(model, want_sens)
    n = s.stations.shape[0]
    if not want_sens:
        return np.concatenate([g.reshape(n, 1), t.reshape(n, 9)], axis=1).ravel()
    d = np.concatenate([g[0].reshape(n, 1), t[0].reshape(n, 9)], axis=1).ravel()
    J = np.concatenate([g[1].reshape(n, 1, -1), t[1].reshape(n, 9, -1)], axis=1)
    return d, J.reshape(n * 10, -1)


def oracle_lqderivative(O, s, misfit, model=None):
    model = s.model if model is None else model
    if s.kind != W.JOINT:
        return oracle_problem(O, s).lqderivative(model, misfit)
    n = s.stations.shape[0]
    m = np.asarray(misfit).reshape(n, 10)
    g = oracle_problem(O, s, W.SCALAR, W.T_NONE).lqderivative(model, m[:, 0].copy())
    t = oracle_problem(O, s, W.TENSOR, W.T_NONE).lqderivative(model, m[:, 1:].ravel().copy())
    return g + t


def oracle_forward_lqderivative(O, s, misfit, model=None):
    """oracle_forward and oracle_lqderivative from one pass over the box terms."""
    model = s.model if model is None else model
    if s.kind != W.JOINT:
        return oracle_problem(O, s).forward_lqderivative(model, misfit)
    n = s.stations.shape[0]
    m = np.asarray(misfit).reshape(n, 10)
    dg, gg = oracle_problem(O, s, W.SCALAR, W.T_NONE).forward_lqderivative(model,
                                                                          m[:, 0].copy())
    dt, gt = oracle_problem(O, s, W.TENSOR, W.T_NONE).forward_lqderivative(
        model, m[:, 1:].ravel().copy())
    d = np.concatenate([dg.reshape(n, 1), dt.reshape(n, 9)], axis=1).ravel()
    return d, gg + gt


def relerr(x, ref):
    x, ref = np.asarray(x, float), np.asarray(ref, float)
    den = np.linalg.norm(ref)
    return np.linalg.norm(x - ref) / (den if den > 0 else 1.0)


def maxrel(x, ref):
    x, ref = np.asarray(x, float), np.asarray(ref, float)
    den = np.max(np.abs(ref))
    return np.max(np.abs(x - ref)) / (den if den > 0 else 1.0)


def small_survey(kind=W.SCALAR, nx=7, ny=6, nz=5, nmeas=9, seed=0, bg=True, transform=W.T_NONE,
                 inc=0.7, dec=0.3, fs=50000.0, origin=(-10.0, 5.0, 0.0)):
    """A small randomised survey in the spirit of Gravity/test_common.h:MakeRandomModel
    (sizes 10-34 m, values 1-11, stations above the surface), with a fixed seed."""
    rng = np.random.default_rng(seed)
    xs = rng.integers(10, 35, nx).astype(float)
    ys = rng.integers(10, 35, ny).astype(float)
    zs = rng.integers(10, 35, nz).astype(float)
    st = np.stack([origin[0] + rng.uniform(0, xs.sum(), nmeas),
                   origin[1] + rng.uniform(0, ys.sum(), nmeas),
                   -rng.uniform(1, 100, nmeas)], axis=1)
    model = rng.uniform(1, 11, nx * ny * nz)
    bgt = np.array([30.0, 70.0, 200.0]) if bg else np.zeros(0)
    bgv = rng.uniform(1, 5, bgt.size)
    return W.Survey("small", xs, ys, zs, origin, st, kind, np.concatenate([model, bgv]),
                    bg_thick=bgt, inc=inc, dec=dec, fs=fs, transform=transform, t_inc=inc,
                    t_dec=dec)
