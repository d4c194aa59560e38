"""ctypes front end of the FP64 CPU oracle (oracle/prism_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``.  The product library never
imports it.

``liboracle.so`` is the C restatement of the reference's prism arithmetic and
drivers; ``_ref/libjif3d_ref_elements.so`` (optional, built only where the
jif3D sources are present) is the reference's own ``BasicGravElements.cpp``,
used to pin the restatement bit for bit.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libjif3d_ref_elements.so")

SCALAR, TENSOR, MAGNETIC, MAG_GRADIENT, MAGNETIZATION = 1, 2, 3, 5, 6
T_NONE, T_FTG_INVARIANT, T_TOTAL_FIELD, T_TFA = 0, 1, 2, 3
GRAV_CONST = 6.67428e-11

_D = ctypes.c_double
_I = ctypes.c_int
_P = ctypes.POINTER(ctypes.c_double)

_lib = None
_ref = None


def build(force: bool = False, ref_src: str | None = None) -> None:
    """Compile liboracle.so; with `ref_src` (the jif3D source tree, or the
    JIF3D_REF environment variable) also the reference box-term library,
    when that tree exists on this machine."""
    srcs = [os.path.join(HERE, f) for f in ("prism_oracle.c", "refine_oracle.c")]
    stale = not os.path.exists(LIB_PATH) or any(
        os.path.getmtime(f) > os.path.getmtime(LIB_PATH) for f in srcs)
    if force or stale:
        subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    ref_src = ref_src or os.environ.get("JIF3D_REF")
    if ref_src and os.path.isdir(ref_src) and (force or not os.path.exists(REF_PATH)):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_src}"], check=True)


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB_PATH)
        box_args = [_D] * 9
        for name in ("orc_grav_box", "orc_uxx_box", "orc_uxy_box"):
            f = getattr(_lib, name)
            f.argtypes = box_args
            f.restype = _D
        _lib.orc_tensor_box.argtypes = box_args + [_P]
        _lib.orc_tensor_box.restype = None
        for name in ("orc_inf_sheet", "orc_uzz_inf_sheet"):
            f = getattr(_lib, name)
            f.argtypes = [_D, _D, _D]
            f.restype = _D
        common = [_I, _I, _I, _P, _P, _P, _P, _P, _P, _I, _P, _I, _P, _P, _P,
                  _I, _D, _D, _D, _I, _D, _D, _I]
        _lib.orc_forward.argtypes = common + [_P, _P, _P]
        _lib.orc_forward.restype = _I
        _lib.orc_lqderivative.argtypes = common + [_P, _P, _P]
        _lib.orc_lqderivative.restype = _I
        _lib.orc_forward_lqderivative.argtypes = common + [_P, _P, _P, _P]
        _lib.orc_forward_lqderivative.restype = _I
        _lib.orc_sens_matvec.argtypes = [_I, _I, _P, _P, _P]
        _lib.orc_sens_rmatvec2.argtypes = [_I, _I, _P, _P, _P]
        _lib.orc_refine_axis.argtypes = [_I, _P, _P, _I, _P, _P]
        _lib.orc_refine_axis.restype = _I
        walk = [_I, _I, _I, _P, _P, _P, _I, _I, _I, _P, _P, _P, _P, _P]
        _lib.orc_refine_project.argtypes = walk
        _lib.orc_refine_combine.argtypes = walk
    return _lib


def ref_lib():
    """The reference's own box terms, or None where they were not built."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        _ref = ctypes.CDLL(REF_PATH)
        box_args = [_D] * 9
        for name in ("ref_grav_box", "ref_uxx_box", "ref_uxy_box"):
            f = getattr(_ref, name)
            f.argtypes = box_args
            f.restype = _D
        _ref.ref_tensor_box.argtypes = box_args + [_P]
        _ref.ref_tensor_box.restype = None
        for name in ("ref_inf_sheet", "ref_uzz_inf_sheet"):
            f = getattr(_ref, name)
            f.argtypes = [_D, _D, _D]
            f.restype = _D
    return _ref


def _ptr(a):
    return a.ctypes.data_as(_P) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def grav_box(*args) -> float:
    return lib().orc_grav_box(*[float(a) for a in args])


def tensor_box(*args) -> np.ndarray:
    out = np.zeros(9)
    lib().orc_tensor_box(*[float(a) for a in args], _ptr(out))
    return out


def raw_per_meas(kind: int) -> int:
    return {SCALAR: 1, TENSOR: 9, MAGNETIC: 3, MAG_GRADIENT: 1, MAGNETIZATION: 3}[kind]


class Problem:
    """Geometry + stations + physics of one oracle evaluation.

    xcoord/ycoord/zcoord are corner coordinates (n+1 values, as
    ThreeDModelBase::GetXCoordinates), x/y/zsize the n cell sizes.
    """

    def __init__(self, xcoord, ycoord, zcoord, xsize, ysize, zsize, stations,
                 kind=SCALAR, bg_thick=(), inc=0.0, dec=0.0, fs=0.0,
                 transform=T_NONE, t_inc=0.0, t_dec=0.0, nthreads=None):
        self.xc, self.yc, self.zc = _f64(xcoord), _f64(ycoord), _f64(zcoord)
        self.xs, self.ys, self.zs = _f64(xsize), _f64(ysize), _f64(zsize)
        self.nx, self.ny, self.nz = len(self.xs), len(self.ys), len(self.zs)
        st = _f64(stations).reshape(-1, 3)
        self.sx, self.sy, self.sz = (np.ascontiguousarray(st[:, i]) for i in range(3))
        self.nmeas = st.shape[0]
        self.kind = kind
        self.bg = _f64(bg_thick) if len(bg_thick) else np.zeros(0)
        self.inc, self.dec, self.fs = float(inc), float(dec), float(fs)
        self.transform = transform
        self.t_inc, self.t_dec = float(t_inc), float(t_dec)
        self.nthreads = nthreads if nthreads is not None else (os.cpu_count() or 1)

    @property
    def ngrid(self):
        return self.nx * self.ny * self.nz

    @property
    def nparm(self):
        # magnetisation: three cell blocks, no background parameters
        # (Magnetics/ThreeDMagnetizationModel.h:66-69)
        if self.kind == MAGNETIZATION:
            return 3 * self.ngrid
        return self.ngrid + len(self.bg)

    @property
    def raw(self):
        return raw_per_meas(self.kind)

    @property
    def dpm(self):
        return self.raw if self.transform == T_NONE else 1

    def _common(self):
        return [self.nx, self.ny, self.nz, _ptr(self.xc), _ptr(self.yc), _ptr(self.zc),
                _ptr(self.xs), _ptr(self.ys), _ptr(self.zs), len(self.bg),
                _ptr(self.bg) if len(self.bg) else None, self.nmeas, _ptr(self.sx),
                _ptr(self.sy), _ptr(self.sz), self.kind, self.inc, self.dec, self.fs,
                self.transform, self.t_inc, self.t_dec, int(self.nthreads)]

    def forward(self, model, want_sens=False):
        model = _f64(model)
        assert model.size == self.nparm
        data = np.zeros(self.nmeas * self.dpm)
        sens = np.zeros((self.nmeas * self.raw, self.nparm)) if want_sens else None
        rc = lib().orc_forward(*self._common(), _ptr(model), _ptr(data), _ptr(sens))
        assert rc == 0
        return (data, sens) if want_sens else data

    def lqderivative(self, model, misfit):
        model, misfit = _f64(model), _f64(misfit)
        assert misfit.size == self.nmeas * self.dpm
        grad = np.zeros(self.nparm)
        rc = lib().orc_lqderivative(*self._common(), _ptr(model), _ptr(misfit), _ptr(grad))
        assert rc == 0
        return grad

    def forward_lqderivative(self, model, misfit):
        """forward(model) and lqderivative(model, misfit) from one station
        loop (the box terms evaluated once for both)."""
        model, misfit = _f64(model), _f64(misfit)
        assert model.size == self.nparm and misfit.size == self.nmeas * self.dpm
        data = np.zeros(self.nmeas * self.dpm)
        grad = np.zeros(self.nparm)
        rc = lib().orc_forward_lqderivative(*self._common(), _ptr(model), _ptr(misfit),
                                            _ptr(data), _ptr(grad))
        assert rc == 0
        return data, grad


def sens_matvec(J, m):
    J, m = _f64(J), _f64(m)
    d = np.zeros(J.shape[0])
    lib().orc_sens_matvec(J.shape[0], J.shape[1], _ptr(J), _ptr(m), _ptr(d))
    return d


def sens_rmatvec2(J, r):
    J, r = _f64(J), _f64(r)
    g = np.zeros(J.shape[1])
    lib().orc_sens_rmatvec2(J.shape[0], J.shape[1], _ptr(J), _ptr(r), _ptr(g))
    return g


# -- model refinement (ModelBase/ModelRefiner.cpp) ----------------------------
def corners(origin, sizes):
    """ThreeDModelBase::CalcCoords (ModelBase/ThreeDModelBase.cpp:96-113)."""
    c = np.empty(len(sizes) + 1)
    c[0] = s = float(origin)
    for i, v in enumerate(sizes):
        s = s + float(v)
        c[i + 1] = s
    return c


def refine_axis(old_coords, old_sizes, ref_coords):
    """RefineOneAxis: refined sizes, or None where the reference throws."""
    oc, os_, rc = _f64(old_coords), _f64(old_sizes), _f64(ref_coords)
    out = np.zeros(os_.size + rc.size)
    n = lib().orc_refine_axis(os_.size, _ptr(oc), _ptr(os_), rc.size, _ptr(rc), _ptr(out))
    return None if n < 0 else out[:n].copy()


def _walk_args(csizes, fsizes):
    cs = [_f64(v) for v in csizes]
    fs = [_f64(v) for v in fsizes]
    return cs, fs, [c.size for c in cs] + [_ptr(c) for c in cs] + \
        [f.size for f in fs] + [_ptr(f) for f in fs]


def refine_project(csizes, fsizes, coarse, fine=None):
    """ProjectValues of one cell block; ``fine`` (if given) supplies the values
    of refined cells outside every coarse run."""
    cs, fs, args = _walk_args(csizes, fsizes)
    out = np.zeros(int(np.prod([f.size for f in fs]))) if fine is None else _f64(fine).copy()
    c = _f64(coarse)
    lib().orc_refine_project(*args, _ptr(c), _ptr(out))
    return out


def refine_combine(csizes, fsizes, fine):
    """CombineGradient of one cell block."""
    cs, fs, args = _walk_args(csizes, fsizes)
    out = np.zeros(int(np.prod([c.size for c in cs])))
    f = _f64(fine)
    lib().orc_refine_combine(*args, _ptr(f), _ptr(out))
    return out
