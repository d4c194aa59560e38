"""The FP64 logarithm and arctangent of jif3d_gb300/csrc/fp64_math.cuh
(table-driven, few FP64 operations) checked on the device: 2^26 random
arguments each against CUDA's log / atan2, 2^20 against the host C library,
fatan2_pair against two fatan2 calls (bit for bit), and special operands (zeros of both signs, infinities, NaN, subnormals, the
octant boundaries) against CUDA's results."""
import os
import subprocess

import pytest

from jif3d_gb300 import build as B

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def test_fp64_math_accuracy(tmp_path):
    exe = str(tmp_path / "fp64math_check")
    cmd = [B.nvcc(), "-O3", "-std=c++17", B.ARCH, "-I", B.CSRC,
           os.path.join(HERE, "fp64math_check.cu"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    rows = {line.split()[0]: [int(v) for v in line.split()[1:]]
            for line in out.stdout.strip().splitlines()}
    print(out.stdout)
    assert set(rows) == {"log_vs_cuda", "atan2_vs_cuda", "log_vs_host", "atan2_vs_host",
                         "specials", "pair"}
    # within one unit in the last place of the host library (itself within
    # about half an ulp of the exact value), within two of CUDA's
    for name in ("log_vs_host", "atan2_vs_host"):
        assert rows[name][0] <= 1, (name, rows[name])
    for name in ("log_vs_cuda", "atan2_vs_cuda"):
        assert rows[name][0] <= 2, (name, rows[name])
    assert rows["specials"][0] == 0, out.stderr
    assert rows["pair"][0] == 0  # fatan2_pair: bit for bit the two separate calls


def test_fp64_weight_probe_runs(tmp_path):
    """The microkernels that the FP64 flop weights are counted on build and
    run (the counting itself is a profiler capture of this executable)."""
    exe = str(tmp_path / "fp64_weights_probe")
    cmd = [B.nvcc(), "-O3", "-std=c++17", B.ARCH, "-I", B.CSRC,
           os.path.join(HERE, "fp64_weights_probe.cu"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert out.stdout.startswith("calls per kernel")
