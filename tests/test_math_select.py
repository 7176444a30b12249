"""The kernels' branch-free exp2 / log2 / sin / cos and the unorm divisions
(vlt_math.cuh) against the oracle's piecewise restatement and the IEEE quotient, bit
for bit, on the host: every 61st binary32 bit pattern (70 million values) here;
`VLT_MATH_STRIDE=1` runs all 2^32 (a few minutes). The GPU side of the same
functions is compared with the oracle on dense sweeps in test_gpu_math.py."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_branch_free_math_matches_piecewise(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    exe = str(tmp_path / "math_select_check")
    src = os.path.join(HERE, "native", "math_select_check.cpp")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe, src], check=True)
    stride = os.environ.get("VLT_MATH_STRIDE", "61")
    r = subprocess.run([exe, stride], capture_output=True, text=True, timeout=1800)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
