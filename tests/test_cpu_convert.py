"""The integer-pipe float <-> double conversions of the FP32-mixed kernels,
the integer-pipe double comparisons and selections of the FP64 kernels
(huji-rich_gb300/csrc/rg_convert.cuh) agree bit for bit with the C casts and
operators.  The header is host-compilable: the same source is built with
g++ here."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(not shutil.which("g++"), reason="needs g++")
def test_conversions_and_comparisons_match_the_casts_and_operators(tmp_path):
    exe = str(tmp_path / "convert_check")
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I" + os.path.join(ROOT, "huji-rich_gb300", "csrc"),
           os.path.join(ROOT, "tests", "convert_check.cpp"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:]
