"""The correctly rounded FP64 division and square root of
huji-rich_gb300/csrc/rg_div.cuh, device build, against the device's IEEE
division (a / b) and sqrt, bit for bit, on the operand families of
tests/div_cases.h; the FP32 reciprocal and reciprocal square root
approximations they start from are checked on every float in [1, 2) and
[1, 4) (tests/div_check_gpu.cu, built here with nvcc)."""
import json
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_division_and_square_root_on_the_device_bitwise_equal_to_ieee(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    assert os.path.exists(nvcc), "nvcc is needed to build the division check"
    exe = str(tmp_path / "div_check_gpu")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "-I" + os.path.join(ROOT, "huji-rich_gb300", "csrc"), "-I" + os.path.join(ROOT, "tests"),
                    os.path.join(ROOT, "tests", "div_check_gpu.cu"), "-o", exe], check=True)
    r = subprocess.run([exe, "1000000", "7"], capture_output=True, text=True, timeout=900)
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["mismatches"] == 0, res
    assert r.returncode == 0
    assert res["cases"] > 10_000_000
    # the seed is within 2^-23 of 1/f on [1, 2), so in-range pairs stay on the fast path
    assert res["rcp_max_rel_error"] <= 2.0 ** -23, res
    assert res["fast"] > 0.9 * res["cases"], res
    assert res["sqrt_mismatches"] == 0, res
    assert res["sqrt_cases"] > 10_000_000
    # |1 - f y^2| <= 2^-21 on [1, 4): the square root's fast path always applies
    assert res["rsqrt_max_rel_error"] <= 2.0 ** -21, res
    assert res["sqrt_fast"] > 0.9 * res["sqrt_cases"], res
