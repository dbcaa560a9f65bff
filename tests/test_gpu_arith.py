"""FastOps, the branch-free correctly rounded division and square root the constraint projections use
(joltphysics_gb300/csrc/kernels/common.cuh), against CUDA's IEEE routines, on the GPU: every divisor
significand of every binade in range (both signs) with four numerators each, and every square-root
argument in range (tests/arith_check.cu). Bar: no difference in any bit."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_fast_division_and_sqrt_equal_ieee(tmp_path):
    from joltphysics_gb300 import build

    exe = str(tmp_path / "arith_check")
    subprocess.run([build.NVCC] + build.ARCH + ["-O3", "--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-std=c++17",
                                               os.path.join(HERE, "arith_check.cu"), "-o", exe], check=True)
    res = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(res.stdout)
    assert res.returncode == 0, res.stdout + res.stderr
