"""The correctly rounded FP64 division of huji-rich_gb300/csrc/rg_div.cuh
(integer and FP32 pipes only on its fast path), host build, against the
host's IEEE division, bit for bit (tests/div_check.cpp, operand families in
tests/div_cases.h).

The fast path starts from an FP32 reciprocal approximation; the host build
takes it from a stand-in whose error is set per run: the correctly rounded
1/f, one and two ulps off, a crude estimate (every division falls back), and
errors spread over the whole band the fast path accepts (|1 - f*r| up to
2^-22)."""
import json
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def div_check(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("div") / "div_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I" + os.path.join(ROOT, "huji-rich_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "div_check.cpp"), "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("seed_kind", [0, 1, 2, 3, 4, 5, 6])
def test_division_bitwise_equal_to_ieee(div_check, seed_kind):
    r = subprocess.run([div_check, str(seed_kind), "300000", str(11 + seed_kind)],
                       capture_output=True, text=True, timeout=600)
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["mismatches"] == 0, res
    assert r.returncode == 0
    assert res["cases"] > 3_000_000
    if seed_kind in (0, 1, 2):
        # a seed within one ulp never leaves the fast path for an in-range pair
        assert res["fast"] > 0.9 * res["cases"], res
    if seed_kind == 5:
        # only the zero numerators are taken without the seed
        assert res["fast"] < 0.02 * res["cases"], res
