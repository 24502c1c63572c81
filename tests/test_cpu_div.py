"""The correctly rounded FP64 division and square root of
huji-rich_gb300/csrc/rg_div.cuh (integer and FP32 pipes only on their fast
paths), host build, against the host's IEEE division and sqrt, bit for bit
(tests/div_check.cpp and tests/sqrt_check.cpp, operand families in
tests/div_cases.h).

The fast paths start from an FP32 reciprocal (square root) approximation;
the host build takes it from a stand-in whose error is set per run: the
correctly rounded value, one and two ulps off, a crude estimate (everything
falls back), and errors spread over the whole band the fast path accepts."""
import json
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build(tmp_path_factory, name):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp(name) / name)
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I" + os.path.join(ROOT, "huji-rich_gb300", "csrc"),
                    os.path.join(ROOT, "tests", name + ".cpp"), "-o", exe], check=True)
    return exe


@pytest.fixture(scope="module")
def div_check(tmp_path_factory):
    return build(tmp_path_factory, "div_check")


@pytest.fixture(scope="module")
def sqrt_check(tmp_path_factory):
    return build(tmp_path_factory, "sqrt_check")


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


@pytest.mark.parametrize("seed_kind", [0, 1, 2, 3, 4, 5, 6])
def test_square_root_bitwise_equal_to_ieee(sqrt_check, seed_kind):
    r = subprocess.run([sqrt_check, str(seed_kind), "300000", str(31 + seed_kind)],
                       capture_output=True, text=True, timeout=600)
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["mismatches"] == 0, res
    assert r.returncode == 0
    assert res["cases"] > 3_000_000
    if seed_kind in (0, 1, 2):
        assert res["fast"] > 0.9 * res["cases"], res
    if seed_kind == 5:
        # only the zeros are taken without the seed
        assert res["fast"] < 0.05 * res["cases"], res
