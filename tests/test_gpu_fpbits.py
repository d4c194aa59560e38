"""The integer-pipe FP64 <-> FP32 conversions used by the streaming passes of
the stored products (jif3d_gb300/csrc/fpbits.cuh), checked on the device
against CUDA's own conversions: every float for the widening, 2^28 random
doubles (half of them exact rounding ties) for the narrowing, and 2^28 cases
each for the truncation estimate, power-of-two scaling and the FP32
two-sum.  Bit-exact: no mismatch is allowed."""
import os
import subprocess

import pytest

from jif3d_gb300 import build as B

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def test_fpbits_bit_exact(tmp_path):
    exe = str(tmp_path / "fpbits_check")
    cmd = [B.nvcc(), "-O3", "-std=c++17", B.ARCH, "-I", B.CSRC,
           os.path.join(HERE, "fpbits_check.cu"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    rows = [line.split() for line in out.stdout.strip().splitlines()]
    assert [row[0] for row in rows] == ["widen", "narrow", "approx", "scale_pow2", "two_sum"]
    for name, bad, tested in rows:
        assert int(tested) > 1 << 26, (name, tested)
        assert int(bad) == 0, (name, bad, tested)
