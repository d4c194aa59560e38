"""ctypes binding of the C ABI in ``include/jif3d_gb300.h``.

The library must have been built (``python -m jif3d_gb300.build`` or
``__graft_entry__.build()``); there is no CPU fallback, a missing library or a
missing GPU raises :class:`J3GError`.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

OK, ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_STATE, ERR_UNSUPPORTED, ERR_SCRATCH_LIMIT = range(7)
SCALAR, TENSOR, MAGNETIC, JOINT, MAG_GRADIENT, MAGNETIZATION = 1, 2, 3, 4, 5, 6
T_NONE, T_FTG_INVARIANT, T_TOTAL_FIELD, T_TFA = 0, 1, 2, 3
STORE_FP32, STORE_F16X2 = 1, 2
(TIMER_NODE_FORWARD, TIMER_NODE_ADJOINT, TIMER_STREAM_FORWARD, TIMER_STREAM_ADJOINT,
 TIMER_GEMM_FORWARD, TIMER_GEMM_ADJOINT, TIMER_SPLIT, TIMER_REDUCE, TIMER_EPILOGUE) = range(9)

_P = ctypes.POINTER(ctypes.c_double)
_VP = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_LL = ctypes.c_longlong

# name -> (restype, argtypes); every function declared in include/jif3d_gb300.h
SIGNATURES = {
    "j3g_status_string": (ctypes.c_char_p, [_I]),
    "j3g_last_error": (ctypes.c_char_p, [_VP]),
    "j3g_create": (_I, [ctypes.POINTER(_VP), _I]),
    "j3g_destroy": (_I, [_VP]),
    "j3g_set_stream": (_I, [_VP, _VP]),
    "j3g_set_mesh": (_I, [_VP, _I, _I, _I, _P, _P, _P, _P, _P, _P]),
    "j3g_set_background": (_I, [_VP, _I, _P]),
    "j3g_set_stations": (_I, [_VP, _I, _P, _P, _P]),
    "j3g_set_kind": (_I, [_VP, _I, _D, _D, _D]),
    "j3g_set_transform": (_I, [_VP, _I, _D, _D]),
    "j3g_get_sizes": (_I, [_VP, ctypes.POINTER(_LL), ctypes.POINTER(_LL), ctypes.POINTER(_I),
                           ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    "j3g_forward": (_I, [_VP, _P, _P]),
    "j3g_forward_sens": (_I, [_VP, _P, _P, _P]),
    "j3g_lqderivative": (_I, [_VP, _P, _P, _P]),
    "j3g_forward_device": (_I, [_VP, _VP, _VP]),
    "j3g_lqderivative_device": (_I, [_VP, _VP, _VP, _VP]),
    "j3g_synchronize": (_I, [_VP]),
    "j3g_build_sensitivity": (_I, [_VP, _I]),
    "j3g_drop_sensitivity": (_I, [_VP]),
    "j3g_sensitivity_info": (_I, [_VP, ctypes.POINTER(_I), ctypes.POINTER(_LL),
                                  ctypes.POINTER(_LL), ctypes.POINTER(_LL)]),
    "j3g_stored_forward_device": (_I, [_VP, _VP, _VP]),
    "j3g_stored_lqderivative_device": (_I, [_VP, _VP, _VP, _VP]),
    "j3g_batched_forward_device": (_I, [_VP, _I, _VP, _VP]),
    "j3g_batched_lqderivative_device": (_I, [_VP, _I, _VP, _VP, _VP]),
    "j3g_batched_forward": (_I, [_VP, _I, _P, _P]),
    "j3g_batched_lqderivative": (_I, [_VP, _I, _P, _P, _P]),
    "j3g_batched_forward_async": (_I, [_VP, _I, _P, _P, ctypes.POINTER(_LL)]),
    "j3g_batched_lqderivative_async": (_I, [_VP, _I, _P, _P, _P, ctypes.POINTER(_LL)]),
    "j3g_batched_wait": (_I, [_VP, _LL]),
    "j3g_launch_count": (_I, [_VP, ctypes.POINTER(_LL)]),
    "j3g_set_timing": (_I, [_VP, _I]),
    "j3g_get_timing": (_I, [_VP, _I, _P, ctypes.POINTER(_LL)]),
    "j3g_subsets_forward_device": (_I, [_VP, _I, ctypes.POINTER(_I), ctypes.POINTER(_I), _VP,
                                        _VP]),
    "j3g_subsets_lqderivative_device": (_I, [_VP, _I, ctypes.POINTER(_I), ctypes.POINTER(_I),
                                             _VP, _VP, _VP]),
    "j3g_set_autotune": (_I, [_VP, _I]),
    "j3g_set_gemm_plan": (_I, [_VP, _I, _I, _I]),
    "j3g_get_gemm_plan": (_I, [_VP, _I, ctypes.POINTER(_I), ctypes.POINTER(_I), _P]),
    "j3g_refine_axis": (_I, [_I, _P, _P, _I, _P, _I, _P, ctypes.POINTER(_I)]),
    "j3g_set_refinement": (_I, [_VP, _I, _I, _I, _P, _P, _P]),
    "j3g_refinement_info": (_I, [_VP, ctypes.POINTER(_LL), ctypes.POINTER(_LL),
                                 ctypes.POINTER(_I)]),
    "j3g_refine_project_device": (_I, [_VP, _I, _VP, _VP]),
    "j3g_refine_combine_device": (_I, [_VP, _I, _VP, _VP]),
    "j3g_refine_project": (_I, [_VP, _I, _P, _P]),
    "j3g_refine_combine": (_I, [_VP, _I, _P, _P]),
    "j3g_nc_last_error": (ctypes.c_char_p, []),
    "j3g_nc_open": (_I, [ctypes.c_char_p, ctypes.POINTER(_VP)]),
    "j3g_nc_close": (_I, [_VP]),
    "j3g_nc_format": (_I, [_VP, ctypes.POINTER(_I)]),
    "j3g_nc_nvars": (_I, [_VP, ctypes.POINTER(_I)]),
    "j3g_nc_var_name": (_I, [_VP, _I, _I, ctypes.c_char_p]),
    "j3g_nc_var_shape": (_I, [_VP, ctypes.c_char_p, _I, ctypes.POINTER(_I),
                              ctypes.POINTER(_LL)]),
    "j3g_nc_read_var": (_I, [_VP, ctypes.c_char_p, _LL, _P]),
    "j3g_nc_dim_len": (_I, [_VP, ctypes.c_char_p, ctypes.POINTER(_LL)]),
    "j3g_nc_text_att": (_I, [_VP, ctypes.c_char_p, ctypes.c_char_p, _I, ctypes.c_char_p]),
    "j3g_nc_create": (_I, [ctypes.c_char_p, ctypes.POINTER(_VP)]),
    "j3g_nc_def_dim": (_I, [_VP, ctypes.c_char_p, _LL]),
    "j3g_nc_def_var": (_I, [_VP, ctypes.c_char_p, _I, _I, ctypes.POINTER(ctypes.c_char_p)]),
    "j3g_nc_put_text_att": (_I, [_VP, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p]),
    "j3g_nc_put_var": (_I, [_VP, ctypes.c_char_p, _LL, _P]),
    "j3g_nc_close_writer": (_I, [_VP]),
    "j3g_nc_discard_writer": (_I, [_VP]),
    "j3g_probe_fp64": (_I, [_VP, _P]),
    "j3g_set_test_fault": (_I, [_VP, _I]),
    "j3g_forward_noalloc": (_I, [_I, _I, _I, _I, _VP, _VP, _VP, _I, _VP, _VP, _VP, _D, _D, _D,
                                 _VP, _VP, _VP]),
}

_lib = None


class J3GError(RuntimeError):
    def __init__(self, code, msg=""):
        self.code = code
        super().__init__(f"jif3d_gb300 error {code}: {msg}")


def library_path() -> str:
    return _build.LIB


def load():
    """Load libjif3d_gb300.so (raises J3GError if it has not been built)."""
    global _lib
    if _lib is None:
        path = library_path()
        if not os.path.exists(path):
            raise J3GError(ERR_STATE, f"{path} is missing: build it with "
                                      "`python -m jif3d_gb300.build`")
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_P)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def refine_axis(coarse_coords, coarse_sizes, ref_coords):
    """RefineOneAxis (ModelBase/ModelRefiner.cpp:17-72) on the host: the
    refined cell sizes of one axis.  ``coarse_coords`` holds the n + 1 corners,
    ``ref_coords`` the refinement coordinates (the last one is not used).
    Raises J3GError where the reference throws (a non-positive last cell)."""
    cc, cs, rc = _f64(coarse_coords), _f64(coarse_sizes), _f64(ref_coords)
    lib, n = load(), _I()
    out = np.zeros(cs.size + rc.size)
    rc_ = lib.j3g_refine_axis(cs.size, _ptr(cc), _ptr(cs), rc.size, _ptr(rc), out.size,
                              _ptr(out), ctypes.byref(n))
    if rc_ != OK:
        raise J3GError(rc_, "Negative cell size in model refinement" if n.value < 0 else
                       "bad refinement arguments")
    return out[:n.value].copy()


NC_INT, NC_FLOAT, NC_DOUBLE = 4, 5, 6


def _nc_check(rc):
    if rc != OK:
        raise J3GError(rc, (load().j3g_nc_last_error() or b"").decode())


def _b(s):
    return None if s is None else s.encode()


class NcFile:
    """A NetCDF file read whole by the library (classic or netCDF-4); host only."""

    def __init__(self, path):
        self._lib = load()
        h = _VP()
        _nc_check(self._lib.j3g_nc_open(os.fsencode(path), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.j3g_nc_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def format(self):
        f = _I()
        _nc_check(self._lib.j3g_nc_format(self._h, ctypes.byref(f)))
        return f.value

    def variables(self):
        n = _I()
        _nc_check(self._lib.j3g_nc_nvars(self._h, ctypes.byref(n)))
        out = []
        for i in range(n.value):
            buf = ctypes.create_string_buffer(1024)
            _nc_check(self._lib.j3g_nc_var_name(self._h, i, 1024, buf))
            out.append(buf.value.decode())
        return out

    def has_var(self, name):
        nd, shp = _I(), (_LL * 32)()
        return self._lib.j3g_nc_var_shape(self._h, _b(name), 32, ctypes.byref(nd), shp) == OK

    def shape(self, name):
        nd, shp = _I(), (_LL * 32)()
        _nc_check(self._lib.j3g_nc_var_shape(self._h, _b(name), 32, ctypes.byref(nd), shp))
        return tuple(int(x) for x in shp[:nd.value])

    def read(self, name):
        shape = self.shape(name)
        out = np.zeros(int(np.prod(shape)) if shape else 1)
        _nc_check(self._lib.j3g_nc_read_var(self._h, _b(name), out.size, _ptr(out)))
        return out.reshape(shape) if shape else out

    def dim(self, name):
        n = _LL()
        _nc_check(self._lib.j3g_nc_dim_len(self._h, _b(name), ctypes.byref(n)))
        return n.value

    def has_dim(self, name):
        n = _LL()
        return self._lib.j3g_nc_dim_len(self._h, _b(name), ctypes.byref(n)) == OK

    def att(self, var, name):
        """A text attribute of variable ``var`` (None: of the file), or None."""
        buf = ctypes.create_string_buffer(1 << 16)
        rc = self._lib.j3g_nc_text_att(self._h, _b(var), _b(name), 1 << 16, buf)
        return buf.value.decode() if rc == OK else None


class NcWriter:
    """A CDF-2 NetCDF file written by the library when closed; host only."""

    def __init__(self, path):
        self._lib = load()
        h = _VP()
        _nc_check(self._lib.j3g_nc_create(os.fsencode(path), ctypes.byref(h)))
        self._h = h

    def add_dim(self, name, n):
        _nc_check(self._lib.j3g_nc_def_dim(self._h, _b(name), int(n)))

    def add_var(self, name, dims=(), type=NC_DOUBLE, values=None, **atts):
        arr = (ctypes.c_char_p * max(1, len(dims)))(*[_b(d) for d in dims])
        _nc_check(self._lib.j3g_nc_def_var(self._h, _b(name), type, len(dims), arr))
        for k, v in atts.items():
            self.put_att(name, k, v)
        if values is not None:
            self.put(name, values)

    def put_att(self, var, name, value):
        _nc_check(self._lib.j3g_nc_put_text_att(self._h, _b(var), _b(name), _b(str(value))))

    def put(self, name, values):
        v = _f64(values).reshape(-1)
        _nc_check(self._lib.j3g_nc_put_var(self._h, _b(name), v.size, _ptr(v)))

    def close(self):
        if getattr(self, "_h", None):
            h, self._h = self._h, None
            _nc_check(self._lib.j3g_nc_close_writer(h))

    def __enter__(self):
        return self

    def __exit__(self, exc_type, *exc):
        if exc_type is None:
            self.close()
        elif getattr(self, "_h", None):  # drop the half-defined file
            h, self._h = self._h, None
            self._lib.j3g_nc_discard_writer(h)


class Context:
    """One engine context on one device (owns its device buffers)."""

    def __init__(self, device: int = 0):
        self._lib = load()
        h = _VP()
        rc = self._lib.j3g_create(ctypes.byref(h), int(device))
        if rc != OK:
            raise J3GError(rc, "j3g_create failed: " +
                           self._lib.j3g_status_string(rc).decode() +
                           " (a CUDA device is required; there is no CPU fallback)")
        self._h = h
        self._keep = []
        self._inflight = {}

    def close(self):
        if getattr(self, "_h", None):
            self._lib.j3g_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def _check(self, rc):
        if rc != OK:
            msg = self._lib.j3g_last_error(self._h)
            raise J3GError(rc, (msg or b"").decode() or
                           self._lib.j3g_status_string(rc).decode())

    # -- setup ---------------------------------------------------------------
    def set_stream(self, stream_ptr):
        self._check(self._lib.j3g_set_stream(self._h, _VP(stream_ptr) if stream_ptr else None))

    def set_mesh(self, xcoord, ycoord, zcoord, xsize, ysize, zsize):
        xs, ys, zs = _f64(xsize), _f64(ysize), _f64(zsize)
        xc, yc, zc = _f64(xcoord), _f64(ycoord), _f64(zcoord)
        self._check(self._lib.j3g_set_mesh(self._h, xs.size, ys.size, zs.size, _ptr(xc),
                                           _ptr(yc), _ptr(zc), _ptr(xs), _ptr(ys), _ptr(zs)))

    def set_background(self, thick):
        t = _f64(thick)
        self._check(self._lib.j3g_set_background(self._h, t.size, _ptr(t) if t.size else None))

    def set_stations(self, x, y, z):
        x, y, z = _f64(x), _f64(y), _f64(z)
        self._check(self._lib.j3g_set_stations(self._h, x.size, _ptr(x), _ptr(y), _ptr(z)))

    def set_kind(self, kind, inclination=0.0, declination=0.0, field_strength=0.0):
        self._check(self._lib.j3g_set_kind(self._h, kind, inclination, declination,
                                           field_strength))

    def set_transform(self, transform, inclination=0.0, declination=0.0):
        self._check(self._lib.j3g_set_transform(self._h, transform, inclination, declination))

    def sizes(self):
        ng, npar = _LL(), _LL()
        nm, raw, dpm = _I(), _I(), _I()
        self._check(self._lib.j3g_get_sizes(self._h, ctypes.byref(ng), ctypes.byref(npar),
                                            ctypes.byref(nm), ctypes.byref(raw),
                                            ctypes.byref(dpm)))
        return dict(ngrid=ng.value, nparm=npar.value, nmeas=nm.value, raw=raw.value,
                    dpm=dpm.value)

    # -- compute (host buffers) ---------------------------------------------
    def forward(self, model):
        s = self.sizes()
        m = _f64(model)
        if m.size != s["nparm"]:
            raise J3GError(ERR_ARG, f"model has {m.size} values, expected {s['nparm']}")
        d = np.zeros(s["nmeas"] * s["dpm"])
        self._check(self._lib.j3g_forward(self._h, _ptr(m), _ptr(d)))
        return d

    def forward_sens(self, model):
        s = self.sizes()
        m = _f64(model)
        if m.size != s["nparm"]:
            raise J3GError(ERR_ARG, f"model has {m.size} values, expected {s['nparm']}")
        d = np.zeros(s["nmeas"] * s["dpm"])
        J = np.zeros((s["nmeas"] * s["raw"], s["nparm"]))
        self._check(self._lib.j3g_forward_sens(self._h, _ptr(m), _ptr(d), _ptr(J)))
        return d, J

    def lqderivative(self, model, misfit):
        s = self.sizes()
        m, r = _f64(model), _f64(misfit)
        if m.size != s["nparm"] or r.size != s["nmeas"] * s["dpm"]:
            raise J3GError(ERR_ARG, "model or misfit size mismatch")
        g = np.zeros(s["nparm"])
        self._check(self._lib.j3g_lqderivative(self._h, _ptr(m), _ptr(r), _ptr(g)))
        return g

    # -- compute (device pointers, e.g. torch tensors' data_ptr()) -----------
    def forward_device(self, d_model, d_data):
        self._check(self._lib.j3g_forward_device(self._h, _VP(d_model), _VP(d_data)))

    def lqderivative_device(self, d_model, d_misfit, d_grad):
        self._check(self._lib.j3g_lqderivative_device(self._h, _VP(d_model), _VP(d_misfit),
                                                      _VP(d_grad)))

    def synchronize(self):
        self._check(self._lib.j3g_synchronize(self._h))

    # -- device-resident sensitivity ----------------------------------------
    def build_sensitivity(self, storage):
        self._check(self._lib.j3g_build_sensitivity(self._h, int(storage)))

    def drop_sensitivity(self):
        self._check(self._lib.j3g_drop_sensitivity(self._h))

    def sensitivity_info(self):
        st, r, c, b = _I(), _LL(), _LL(), _LL()
        self._check(self._lib.j3g_sensitivity_info(self._h, ctypes.byref(st), ctypes.byref(r),
                                                   ctypes.byref(c), ctypes.byref(b)))
        return dict(storage=st.value, rows=r.value, cols=c.value, bytes=b.value)

    def stored_forward_device(self, d_model, d_data):
        self._check(self._lib.j3g_stored_forward_device(self._h, _VP(d_model), _VP(d_data)))

    def stored_lqderivative_device(self, d_model, d_misfit, d_grad):
        self._check(self._lib.j3g_stored_lqderivative_device(self._h, _VP(d_model),
                                                             _VP(d_misfit), _VP(d_grad)))

    def batched_forward_device(self, nmodels, d_models, d_data):
        self._check(self._lib.j3g_batched_forward_device(self._h, int(nmodels), _VP(d_models),
                                                         _VP(d_data)))

    def batched_lqderivative_device(self, nmodels, d_models, d_misfits, d_grads):
        self._check(self._lib.j3g_batched_lqderivative_device(self._h, int(nmodels),
                                                              _VP(d_models), _VP(d_misfits),
                                                              _VP(d_grads)))

    @staticmethod
    def _out(out, shape):
        """A caller's output array (e.g. a view of pinned host memory), checked."""
        if out is None:
            return np.zeros(shape)
        if (out.dtype != np.float64 or not out.flags.c_contiguous or
                out.size != int(np.prod(shape))):
            raise J3GError(ERR_ARG, "out must be a C-contiguous float64 array of the result size")
        return out

    def batched_forward(self, models, out=None):
        s = self.sizes()
        m = _f64(models).reshape(-1, s["nparm"])
        d = self._out(out, (m.shape[0], s["nmeas"] * s["dpm"]))
        self._check(self._lib.j3g_batched_forward(self._h, m.shape[0], _ptr(m), _ptr(d)))
        return d

    def batched_lqderivative(self, models, misfits, out=None):
        """2 J^T r per model; ``models`` may be None unless the transform is
        the FTG invariant or the total field (only those read the models)."""
        s = self.sizes()
        r = _f64(misfits).reshape(-1, s["nmeas"] * s["dpm"])
        m = None if models is None else _f64(models).reshape(r.shape[0], s["nparm"])
        g = self._out(out, (r.shape[0], s["nparm"]))
        self._check(self._lib.j3g_batched_lqderivative(self._h, r.shape[0], _ptr(m), _ptr(r),
                                                       _ptr(g)))
        return g

    # pipelined host-buffer products: the arrays are held until the wait
    def batched_forward_async(self, models, out):
        s = self.sizes()
        m = _f64(models).reshape(-1, s["nparm"])
        d = self._out(out, (m.shape[0], s["nmeas"] * s["dpm"]))
        t = _LL()
        self._check(self._lib.j3g_batched_forward_async(self._h, m.shape[0], _ptr(m), _ptr(d),
                                                        ctypes.byref(t)))
        self._hold(t.value, (m, d))
        return t.value

    def batched_lqderivative_async(self, models, misfits, out):
        s = self.sizes()
        r = _f64(misfits).reshape(-1, s["nmeas"] * s["dpm"])
        m = None if models is None else _f64(models).reshape(r.shape[0], s["nparm"])
        g = self._out(out, (r.shape[0], s["nparm"]))
        t = _LL()
        self._check(self._lib.j3g_batched_lqderivative_async(self._h, r.shape[0], _ptr(m),
                                                             _ptr(r), _ptr(g), ctypes.byref(t)))
        self._hold(t.value, (m, r, g))
        return t.value

    # calls in flight at once in the library's ring of pipelined calls
    PIPELINE_SLOTS = 4

    def _hold(self, ticket, arrays):
        """Keep a call's arrays alive until it is waited for; a call
        PIPELINE_SLOTS or more tickets older has completed (its ring slot was
        reused by a later call, which waited for it)."""
        self._inflight[ticket] = arrays
        for t in [t for t in self._inflight if t <= ticket - self.PIPELINE_SLOTS]:
            del self._inflight[t]

    def batched_wait(self, ticket):
        try:
            self._check(self._lib.j3g_batched_wait(self._h, int(ticket)))
        finally:
            self._inflight.pop(int(ticket), None)

    @staticmethod
    def _subsets(subsets):
        """Offsets and concatenated indices (int32 host arrays) of station subsets."""
        off = np.zeros(len(subsets) + 1, dtype=np.int32)
        off[1:] = np.cumsum([len(x) for x in subsets])
        idx = (np.concatenate([np.asarray(x, dtype=np.int32) for x in subsets])
               if off[-1] else np.zeros(1, dtype=np.int32))
        return off, np.ascontiguousarray(idx, dtype=np.int32)

    def subsets_forward_device(self, subsets, d_model, d_data):
        off, idx = self._subsets(subsets)
        ip = ctypes.POINTER(_I)
        self._check(self._lib.j3g_subsets_forward_device(
            self._h, len(subsets), off.ctypes.data_as(ip), idx.ctypes.data_as(ip),
            _VP(d_model), _VP(d_data)))

    def subsets_lqderivative_device(self, subsets, d_model, d_misfit, d_grads):
        off, idx = self._subsets(subsets)
        ip = ctypes.POINTER(_I)
        self._check(self._lib.j3g_subsets_lqderivative_device(
            self._h, len(subsets), off.ctypes.data_as(ip), idx.ctypes.data_as(ip),
            _VP(d_model), _VP(d_misfit), _VP(d_grads)))

    # -- model refinement (coarse inversion grid over this context's mesh) --
    def set_refinement(self, xsizes, ysizes, zsizes):
        xs, ys, zs = _f64(xsizes), _f64(ysizes), _f64(zsizes)
        self._check(self._lib.j3g_set_refinement(self._h, xs.size, ys.size, zs.size, _ptr(xs),
                                                 _ptr(ys), _ptr(zs)))

    def refinement_info(self):
        cells, nparm, cov = _LL(), _LL(), _I()
        self._check(self._lib.j3g_refinement_info(self._h, ctypes.byref(cells),
                                                  ctypes.byref(nparm), ctypes.byref(cov)))
        return dict(coarse_cells=cells.value, coarse_nparm=nparm.value,
                    covers_all=bool(cov.value))

    def refine_project_device(self, nmodels, d_coarse, d_fine):
        self._check(self._lib.j3g_refine_project_device(self._h, int(nmodels), _VP(d_coarse),
                                                        _VP(d_fine)))

    def refine_combine_device(self, nmodels, d_fine, d_coarse):
        self._check(self._lib.j3g_refine_combine_device(self._h, int(nmodels), _VP(d_fine),
                                                        _VP(d_coarse)))

    def refine_project(self, coarse, fine=None):
        """ProjectValues of one model [coarse nparm] or of a batch [n, coarse
        nparm]; ``fine`` supplies the values of cells outside every coarse run."""
        info, s = self.refinement_info(), self.sizes()
        c = _f64(coarse)
        n = 1 if c.ndim == 1 else c.shape[0]
        c = c.reshape(n, info["coarse_nparm"])
        f = (np.zeros((n, s["nparm"])) if fine is None
             else np.array(fine, dtype=np.float64).reshape(n, s["nparm"]))
        self._check(self._lib.j3g_refine_project(self._h, n, _ptr(c), _ptr(f)))
        return f[0] if np.ndim(coarse) == 1 else f

    def refine_combine(self, fine):
        """CombineGradient of one gradient [nparm] or of a batch [n, nparm]."""
        info, s = self.refinement_info(), self.sizes()
        f = _f64(fine)
        n = 1 if f.ndim == 1 else f.shape[0]
        f = f.reshape(n, s["nparm"])
        c = np.zeros((n, info["coarse_nparm"]))
        self._check(self._lib.j3g_refine_combine(self._h, n, _ptr(f), _ptr(c)))
        return c[0] if np.ndim(fine) == 1 else c

    def set_autotune(self, enable=True):
        self._check(self._lib.j3g_set_autotune(self._h, 1 if enable else 0))

    def set_gemm_plan(self, direction, nsplit, tile=0):
        """Pin the plan of a direction; nsplit <= 0 unpins it."""
        self._check(self._lib.j3g_set_gemm_plan(self._h, int(direction), int(nsplit), int(tile)))

    def gemm_plan(self, direction):
        ns, tile, ms = _I(), _I(), _D()
        self._check(self._lib.j3g_get_gemm_plan(self._h, int(direction), ctypes.byref(ns),
                                                ctypes.byref(tile), ctypes.byref(ms)))
        return dict(nsplit=ns.value, tile=tile.value, tuned_ms=ms.value)

    def set_timing(self, enable=True):
        self._check(self._lib.j3g_set_timing(self._h, 1 if enable else 0))

    def get_timing(self, category):
        ms, n = _D(), _LL()
        self._check(self._lib.j3g_get_timing(self._h, int(category), ctypes.byref(ms),
                                             ctypes.byref(n)))
        return ms.value, n.value

    def set_test_fault(self, fault):
        """Failure-path test of the tensor-core waits (see j3g_set_test_fault)."""
        self._check(self._lib.j3g_set_test_fault(self._h, int(fault)))

    def launch_count(self):
        v = _LL()
        self._check(self._lib.j3g_launch_count(self._h, ctypes.byref(v)))
        return v.value

    def probe_fp64(self):
        v = _D()
        self._check(self._lib.j3g_probe_fp64(self._h, ctypes.byref(v)))
        return v.value
