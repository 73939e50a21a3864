"""The mixed form's integer-pipe double<->float conversions (hx_device.cuh) equal the
hardware conversions bit for bit (2^26 random inputs each way, with ties, zeros,
subnormal-range exponents, overflow, infinities and NaN); the Newton-Raphson reciprocal
rcp_newton and the corrected quotient div_newton stay within one ulp of IEEE division."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def test_conversions_match_hardware(tmp_path):
    from hommexx_gb300 import build as B
    exe = str(tmp_path / "convert_check")
    subprocess.run([B.nvcc(), *B.flags(), "-o", exe, os.path.join(HERE, "cuda", "convert_check.cu")],
                   check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
