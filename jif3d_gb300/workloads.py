"""Seeded synthetic survey configurations (meshes, models, stations).

The five configurations of the prism-path benchmark, built from numpy's
PCG64 generator with fixed seeds so that every machine produces the same
arrays.  Densities are drawn in g/cm^3 and converted to kg/m^3 (x1000), the
unit the reference's SI gravitational constant expects
(Gravity/BasicGravElements.h:22); susceptibilities are SI; angles radians.

Each builder returns a ``Survey``; ``stations`` may be thinned with
``subset`` for CPU-sized checks.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

SEEDS = {1: 101, 2: 102, 3: 103, 4: 104, 5: 105}
SCALAR, TENSOR, MAGNETIC, JOINT, MAG_GRADIENT, MAGNETIZATION = 1, 2, 3, 4, 5, 6
T_NONE, T_FTG_INVARIANT, T_TOTAL_FIELD, T_TFA = 0, 1, 2, 3
# Config 1 and 3 have an infinite bottom background layer; an infinite sheet
# term grows without bound with thickness, so it is replaced by this finite
# thickness (m).
BOTTOM_LAYER_THICKNESS = 10000.0


@dataclasses.dataclass
class Survey:
    name: str
    xsize: np.ndarray
    ysize: np.ndarray
    zsize: np.ndarray
    origin: tuple
    stations: np.ndarray            # (n, 3)
    kind: int
    model: np.ndarray               # ngrid + nbg values
    bg_thick: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))
    inc: float = 0.0
    dec: float = 0.0
    fs: float = 0.0
    transform: int = T_NONE
    t_inc: float = 0.0
    t_dec: float = 0.0
    models: np.ndarray | None = None     # extra models (nmodels, nparm) for batched runs
    subsets: list | None = None          # station index subsets for uneven batches
    misfit_sigma: np.ndarray | None = None

    @property
    def shape(self):
        return (self.xsize.size, self.ysize.size, self.zsize.size)

    @property
    def ngrid(self):
        return int(np.prod(self.shape))

    @property
    def nparm(self):
        if self.kind == MAGNETIZATION:   # three cell blocks, no background parameters
            return 3 * self.ngrid
        return self.ngrid + self.bg_thick.size

    def coords(self, axis):
        sizes = (self.xsize, self.ysize, self.zsize)[axis]
        c = np.empty(sizes.size + 1)
        c[0] = s = float(self.origin[axis])
        for i, v in enumerate(sizes):     # running sum, ThreeDModelBase::CalcCoords
            s = s + v
            c[i + 1] = s
        return c

    @property
    def raw(self):
        return {SCALAR: 1, TENSOR: 9, MAGNETIC: 3, JOINT: 10, MAG_GRADIENT: 1,
                MAGNETIZATION: 3}[self.kind]

    @property
    def dpm(self):
        return self.raw if self.transform == T_NONE else 1

    def subset(self, idx):
        s = dataclasses.replace(self)
        s.stations = self.stations[np.asarray(idx)]
        return s


def _grid_stations(n, spacing, start, z):
    v = start + spacing * np.arange(n)
    X, Y = np.meshgrid(v, v, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), np.full(X.size, float(z))], axis=1)


def _blobs(rng, xs, ys, zs, nblob=8, amp=0.3, smin=100.0, smax=400.0):
    xc = np.cumsum(xs) - xs / 2
    yc = np.cumsum(ys) - ys / 2
    zc = np.cumsum(zs) - zs / 2
    X, Y, Z = np.meshgrid(xc, yc, zc, indexing="ij")
    rho = np.zeros(X.shape)
    for _ in range(nblob):
        c = [rng.uniform(0, xs.sum()), rng.uniform(0, ys.sum()), rng.uniform(0, zs.sum())]
        a = amp * (1 if rng.uniform() < 0.5 else -1)
        s = rng.uniform(smin, smax)
        rho += a * np.exp(-((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) / (2 * s * s))
    return rho


def config1():
    """g_z forward + sensitivities, 30x30x15, 3-layer background, 20x20 stations."""
    rng = np.random.default_rng(SEEDS[1])
    xs = np.full(30, 100.0)
    zs = np.array([50.0 * 1.1 ** k for k in range(15)])
    rho = rng.uniform(-0.5, 0.5, 30 * 30 * 15) * 1000.0
    bg_rho = np.array([2.4, 2.6, 2.8]) * 1000.0
    return Survey("config1_gz_30x30x15", xs, xs.copy(), zs, (0.0, 0.0, 0.0),
                  _grid_stations(20, 150.0, 75.0, -1.0), SCALAR,
                  np.concatenate([rho, bg_rho]),
                  bg_thick=np.array([200.0, 500.0, BOTTOM_LAYER_THICKNESS]))


def config2():
    """FTG forward, 64x64x32 Gaussian blobs, 40x40 stations at z=-50 m."""
    rng = np.random.default_rng(SEEDS[2])
    xs = np.full(64, 50.0)
    zs = np.array([25.0 * 1.05 ** k for k in range(32)])
    rho = (_blobs(rng, xs, xs, zs) + rng.normal(0, 0.02, (64, 64, 32))) * 1000.0
    return Survey("config2_ftg_64x64x32", xs, xs.copy(), zs, (0.0, 0.0, 0.0),
                  _grid_stations(40, 80.0, 40.0, -50.0), TENSOR, rho.ravel())


def config3():
    """Joint g_z + FTG adjoint, 96x96x48 40 m cubes, 50x50 stations."""
    rng = np.random.default_rng(SEEDS[3])
    xs = np.full(96, 40.0)
    rho = rng.uniform(-0.5, 0.5, 96 * 96 * 48) * 1000.0
    bg_rho = np.array([2.4, 2.6, 2.8]) * 1000.0
    st = _grid_stations(50, 76.8, 38.4, -1.0)
    sigma = np.tile(np.array([1e-8] + [1e-9] * 9), st.shape[0])
    return Survey("config3_joint_96x96x48", xs, xs.copy(), np.full(48, 40.0), (0.0, 0.0, 0.0),
                  st, JOINT, np.concatenate([rho, bg_rho]),
                  bg_thick=np.array([200.0, 500.0, BOTTOM_LAYER_THICKNESS]),
                  misfit_sigma=sigma)


def config4(nmodels=256):
    """Batched g_z + FTG, 64x64x32 blobs, nmodels perturbed models, 32x32 stations."""
    rng = np.random.default_rng(SEEDS[4])
    xs = np.full(64, 50.0)
    zs = np.array([25.0 * 1.05 ** k for k in range(32)])
    base = _blobs(rng, xs, xs, zs).ravel()
    models = (base[None, :] + rng.normal(0, 0.05, (nmodels, base.size))) * 1000.0
    return Survey("config4_batched_64x64x32", xs, xs.copy(), zs, (0.0, 0.0, 0.0),
                  _grid_stations(32, 100.0, 50.0, -50.0), JOINT, base * 1000.0,
                  models=models)


def config5():
    """TFA magnetics, 128x128x64 25 m cubes, 64x64 stations, 32 uneven subsets."""
    rng = np.random.default_rng(SEEDS[5])
    xs = np.full(128, 25.0)
    chi = np.clip(np.exp(rng.normal(math.log(0.005), 1.0, 128 * 128 * 64)), 0.0, 0.1)
    st = _grid_stations(64, 50.0, 25.0, -30.0)
    sizes = rng.integers(256, 4097, 32)
    subsets = [np.sort(rng.choice(st.shape[0], int(n), replace=False)) for n in sizes]
    inc, dec = math.radians(60.0), math.radians(10.0)
    return Survey("config5_tfa_128x128x64", xs, xs.copy(), np.full(64, 25.0), (0.0, 0.0, 0.0),
                  st, MAGNETIC, chi, inc=inc, dec=dec, fs=50000.0, transform=T_TFA,
                  t_inc=inc, t_dec=dec, subsets=subsets)


CONFIGS = {1: config1, 2: config2, 3: config3, 4: config4, 5: config5}


def setup_context(ctx, s: Survey):
    """Load a survey's geometry into a capi.Context."""
    ctx.set_mesh(s.coords(0), s.coords(1), s.coords(2), s.xsize, s.ysize, s.zsize)
    ctx.set_background(s.bg_thick)
    ctx.set_stations(s.stations[:, 0], s.stations[:, 1], s.stations[:, 2])
    ctx.set_kind(s.kind, s.inc, s.dec, s.fs)
    ctx.set_transform(s.transform, s.t_inc, s.t_dec)
