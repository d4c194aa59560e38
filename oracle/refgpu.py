"""The reference's own CUDA gravity layer, built and driven unmodified, as the
secondary reference-GPU point of the measurements (baseline and test
infrastructure only; the product library never imports it).

jif3D's GPU path (Gravity/gravcuda.cu:8-197 with gravcuda_kernel.cu,
ftgcuda_kernel.cu, common.cu and Global/CudaError.h) exports four C
functions: PrepareData copies the mesh to the device, SingleScalarMeas /
SingleFTGMeas launch one thread-per-cell kernel per station (one per FTG
component) and copy each sensitivity row back to the host, FreeData releases
the buffers.  Its host imps (ScalarCudaGravityImp.cpp:80-154,
TensorCudaGravityImp.cpp:65-172) then take the inner products with the
densities on the host.  This module:

* ``stage(tree)``: copies those five source files, unmodified, from a jif3D
  source tree into ``baseline/_ref/jif3D`` (git-ignored; it travels with the
  repository copy to a GPU machine, where the jif3D tree is absent);
* ``build()``: compiles the staged ``gravcuda.cu`` for sm_103a into
  ``oracle/_ref/libjif3d_ref_gravcuda.so`` (block size and everything else as
  the reference has them);
* ``run(...)``: the reference's per-station loop over a survey -- kernel(s),
  the blocking copy of the row(s) into page-locked host memory, and the host
  inner products -- timed, returning the data and the rows.

The reference's CUDA_SAFE_CALL exits the process on any CUDA error, so
callers run ``run`` in a child process (``python bench.py --case
reference-gpu``).  The reference GPU path has no adjoint: its
implementations do not override LQDerivative (the base class's gradient
then uses device buffers that Calculate freed), so only the forward and the
sensitivity rows are timed.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
STAGE = os.path.join(ROOT, "baseline", "_ref", "jif3D")
LIB = os.path.join(HERE, "_ref", "libjif3d_ref_gravcuda.so")
FILES = ("Gravity/gravcuda.cu", "Gravity/gravcuda_kernel.cu", "Gravity/ftgcuda_kernel.cu",
         "Gravity/common.cu", "Global/CudaError.h")
BLOCK_SIZE = 128  # ScalarCudaGravityImp / TensorCudaGravityImp's blocksize


def staged() -> bool:
    return all(os.path.exists(os.path.join(STAGE, f)) for f in FILES)


def stage(tree: str) -> bool:
    """Copy the reference's CUDA gravity sources from the jif3D tree `tree`."""
    if not all(os.path.exists(os.path.join(tree, f)) for f in FILES):
        return False
    for f in FILES:
        dst = os.path.join(STAGE, f)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        shutil.copyfile(os.path.join(tree, f), dst)
    return True


def build(force: bool = False) -> str | None:
    """Compile the staged sources; the library path, or None if not staged."""
    if not staged():
        return None
    src = os.path.join(STAGE, "Gravity", "gravcuda.cu")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    from jif3d_gb300 import build as B
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = [B.nvcc(), "-O3", B.ARCH, "-shared", "-Xcompiler", "-fPIC", "-w", src, "-o", LIB]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference gravcuda.cu did not build:\n{r.stderr}")
    return LIB


def _lib():
    lib = ctypes.CDLL(LIB)
    P = ctypes.POINTER(ctypes.c_double)
    PP = ctypes.POINTER(P)
    D, U = ctypes.c_double, ctypes.c_uint
    lib.PrepareData.argtypes = [PP] * 7 + [P] * 6 + [U, U, U]
    lib.PrepareData.restype = None
    lib.FreeData.argtypes = [PP] * 7
    lib.FreeData.restype = None
    meas = [D, D, D] + [P] * 7 + [U, U, U, P, U]
    lib.SingleScalarMeas.argtypes = meas
    lib.SingleScalarMeas.restype = None
    lib.SingleFTGMeas.argtypes = meas
    lib.SingleFTGMeas.restype = None
    return lib


def run(xcorner, ycorner, zcorner, xsize, ysize, zsize, stations, model, tensor):
    """The reference GPU forward of `model` (ngrid cell values, z fastest) at
    `stations` ((n, 3)): per station SingleScalarMeas or SingleFTGMeas into a
    page-locked host row buffer, then the host inner products as the
    reference's CalcGridded does.  xcorner etc. are the cells' lower corner
    coordinates (nx values, GetXCoordinates without the last).  Returns
    (data (n, 1) or (n, 6) in the order Uxx Uxy Uxz Uyy Uyz Uzz, the rows of
    the last station, seconds of the station loop, seconds of PrepareData +
    FreeData)."""
    import torch  # page-locked host memory, as the reference's cudaMallocHost
    lib = _lib()
    P = ctypes.POINTER(ctypes.c_double)
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    xc, yc, zc, xs, ys, zs = (f64(a) for a in (xcorner, ycorner, zcorner, xsize, ysize, zsize))
    nx, ny, nz = xs.size, ys.size, zs.size
    ngrid = nx * ny * nz
    ncomp = 6 if tensor else 1
    rows_t = torch.empty(ncomp * ngrid, dtype=torch.float64, pin_memory=True)
    rows = rows_t.numpy()
    m = f64(model)[:ngrid]
    ptrs = [P() for _ in range(7)]
    t0 = time.perf_counter()
    lib.PrepareData(*[ctypes.byref(p) for p in ptrs],
                    *[a.ctypes.data_as(P) for a in (xc, yc, zc, xs, ys, zs)], nx, ny, nz)
    t_prep = time.perf_counter() - t0
    fn = lib.SingleFTGMeas if tensor else lib.SingleScalarMeas
    st = f64(stations).reshape(-1, 3)
    out = np.zeros((st.shape[0], ncomp))
    rp = rows_t.data_ptr()
    t0 = time.perf_counter()
    for i, (x, y, z) in enumerate(st):
        fn(float(x), float(y), float(z), *ptrs[:7], nx, ny, nz, ctypes.cast(rp, P), BLOCK_SIZE)
        for c in range(ncomp):
            out[i, c] = float(np.dot(rows[c * ngrid:(c + 1) * ngrid], m))
    t_loop = time.perf_counter() - t0
    t0 = time.perf_counter()
    lib.FreeData(*[ctypes.byref(p) for p in ptrs])
    t_prep += time.perf_counter() - t0
    return out, rows.copy(), t_loop, t_prep
