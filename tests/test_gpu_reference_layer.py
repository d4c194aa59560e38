"""The reference's own CUDA gravity layer (jif3D Gravity/gravcuda.cu, staged
unmodified into baseline/_ref and built for sm_103a) against the oracle.

This pins the oracle's box terms against a second build of the reference,
its GPU kernels, on this machine's GPU: data and sensitivity rows of a small
survey with the stations above the mesh (where the CPU code's eps clamps,
which the reference's GPU kernels lack, do not act) agree within the FP64
tolerance.  The reference layer exits the process on a CUDA error, so it runs
in a child process.  Skipped where its sources were not staged.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from helpers import oracle_forward, relerr, small_survey
from jif3d_gb300 import workloads as W

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TOL = 1e-10

CHILD = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
import numpy as np
from oracle import refgpu
refgpu.build()
a = json.loads(sys.stdin.read())
d, rows, _, _ = refgpu.run(*[np.array(a[k]) for k in ("xc", "yc", "zc", "xs", "ys", "zs")],
                           np.array(a["st"]), np.array(a["m"]), a["tensor"])
print(json.dumps({"data": d.tolist(), "rows": rows.tolist()}))
"""


@pytest.mark.parametrize("kind", [W.SCALAR, W.TENSOR])
def test_reference_gpu_layer_matches_oracle(oracle_lib, kind):
    from oracle import refgpu
    if not refgpu.staged():
        pytest.skip("reference CUDA sources not staged in baseline/_ref")
    s = small_survey(kind, seed=900 + kind, nx=9, ny=8, nz=6, nmeas=11, bg=False)
    args = {"xc": s.coords(0)[:-1].tolist(), "yc": s.coords(1)[:-1].tolist(),
            "zc": s.coords(2)[:-1].tolist(), "xs": s.xsize.tolist(), "ys": s.ysize.tolist(),
            "zs": s.zsize.tolist(), "st": s.stations.tolist(), "m": s.model.tolist(),
            "tensor": kind == W.TENSOR}
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT], input=json.dumps(args),
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    data = np.array(out["data"])
    dref, J = oracle_forward(oracle_lib, s, want_sens=True)
    n = s.stations.shape[0]
    if kind == W.SCALAR:
        assert relerr(data.ravel(), dref) <= TOL
        assert relerr(np.array(out["rows"]), J[n - 1]) <= TOL  # the last station's row
    else:
        pick = [0, 1, 2, 4, 5, 8]  # Uxx Uxy Uxz Uyy Uyz Uzz of the 3 x 3 tensor
        assert relerr(data, dref.reshape(n, 9)[:, pick]) <= TOL
        rows = np.array(out["rows"]).reshape(6, -1)
        last = J.reshape(n, 9, -1)[n - 1]
        for c, k in enumerate(pick):
            assert relerr(rows[c], last[k]) <= TOL, c
