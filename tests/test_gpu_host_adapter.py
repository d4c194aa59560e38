"""The C++ implementation objects (jif3d_gb300/host/GB300GravMagImplementation.h)
driven through jif3D-style calculators by tests/cpp/host_adapter_check.cpp:
MinMem and FullSensitivity calculators, LQDerivative, the base class's
per-station loop over CalcGridded / CalcBackground, data transforms set through
the calculators only (as unchanged jif3D callers set them), and the
FatalException on a bad misfit size -- compared with the oracle at the FP64 tolerance (relative
norm error <= 1e-10) -- and the device-resident calculator
(jif3d_gb300/host/GB300DeviceSensitivityCalculator.h): its FP64 first call,
stored-J calls and batches at the mixed-path tolerance (1e-6), and a moved
station that must not hit the cache."""
import dataclasses
import os
import subprocess

import numpy as np
import pytest

from helpers import oracle_forward, oracle_lqderivative, relerr, small_survey
from jif3d_gb300 import build as B, workloads as W

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
TOL, TOL_MIXED = 1e-10, 1e-6


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    B.build()
    out = str(tmp_path_factory.mktemp("host") / "host_adapter_check")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "jif3d_gb300", "host"),
           os.path.join(HERE, "cpp", "host_adapter_check.cpp"),
           "-L", os.path.dirname(B.LIB), "-ljif3d_gb300",
           "-Wl,-rpath," + os.path.dirname(B.LIB), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def write_problem(path, s, misfit):
    vals = [s.kind, s.inc, s.dec, s.fs, s.transform, s.t_inc, s.t_dec, *s.shape,
            *s.xsize, *s.ysize, *s.zsize, *s.origin, s.bg_thick.size, *s.bg_thick,
            s.stations.shape[0], *s.stations.ravel(), s.model.size, *s.model,
            misfit.size, *misfit]
    with open(path, "w") as f:
        f.write(" ".join(repr(float(v)) if isinstance(v, float) or hasattr(v, "dtype")
                         else str(v) for v in vals))


def read_output(path):
    out = {}
    with open(path) as f:
        for line in f:
            parts = line.split()
            if parts[1:2] == ["ok"]:
                out[parts[0]] = True
                continue
            out[parts[0]] = np.array([float(v) for v in parts[2:]])
            assert out[parts[0]].size == int(parts[1])
    return out


CASES = [(W.SCALAR, W.T_NONE), (W.TENSOR, W.T_NONE), (W.TENSOR, W.T_FTG_INVARIANT),
         (W.MAGNETIC, W.T_TFA), (W.MAG_GRADIENT, W.T_NONE), (W.MAGNETIZATION, W.T_NONE),
         (W.MAGNETIZATION, W.T_TOTAL_FIELD)]


@pytest.mark.parametrize("kind,transform", CASES)
def test_cpp_implementation(oracle_lib, exe, tmp_path, kind, transform):
    s = small_survey(kind, seed=500 + 10 * kind + transform, nx=7, ny=6, nz=5, nmeas=8,
                     bg=kind != W.MAGNETIZATION, transform=transform)
    if kind == W.MAGNETIZATION:
        s.model = np.random.default_rng(kind).uniform(-2, 2, 3 * s.ngrid)
    dref, Jref = oracle_forward(oracle_lib, s, want_sens=True)
    misfit = np.random.default_rng(transform).normal(size=dref.size)
    gref = oracle_lqderivative(oracle_lib, s, misfit)
    write_problem(tmp_path / "p.txt", s, misfit)
    r = subprocess.run([exe, str(tmp_path / "p.txt"), str(tmp_path / "o.txt")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    o = read_output(tmp_path / "o.txt")
    assert relerr(o["minmem"], dref) <= TOL
    assert relerr(o["full"], dref) <= TOL
    assert relerr(o["rows"], Jref.ravel()) <= TOL
    assert relerr(o["grad"], gref) <= TOL
    assert o.get("exception")
    if transform == W.T_NONE:  # the per-station loop (stand-in base class, no transform)
        assert relerr(o["loop"], dref) <= TOL
        assert relerr(o["looprows"], Jref.ravel()) <= TOL
    else:  # the transform set through the calculators only, as unchanged callers do
        assert relerr(o["calcminmem"], dref) <= TOL
        assert relerr(o["calcfull"], dref) <= TOL
        assert relerr(o["calcrows"], Jref.ravel()) <= TOL
        assert relerr(o["calcgrad"], gref) <= TOL
        assert relerr(o["calcfullgrad"], gref) <= TOL
    # the device-resident calculator: FP64 first call, then the stored J
    assert relerr(o["devfirst"], dref) <= TOL
    assert relerr(o["devcached"], dref) <= TOL_MIXED
    assert relerr(o["devgrad"], gref) <= TOL_MIXED
    batch, bgrad = o["devbatch"].reshape(3, -1), o["devbatchgrad"].reshape(3, -1)
    for k in range(3):
        mk = s.model * (1.0 + 0.1 * k)
        assert relerr(batch[k], oracle_forward(oracle_lib, s, mk)) <= TOL_MIXED
        assert relerr(bgrad[k], oracle_lqderivative(oracle_lib, s, misfit * (k + 1.0), mk)) \
            <= TOL_MIXED
    moved = dataclasses.replace(s, stations=s.stations.copy())
    moved.stations[0, 0] += 1.0
    assert relerr(o["devmoved"], oracle_forward(oracle_lib, moved)) <= TOL
    assert o.get("devexception")
    assert relerr(o["dev32cached"], dref) <= TOL_MIXED
    assert relerr(o["dev32grad"], gref) <= TOL_MIXED
