"""The RICH-side adapters (huji-rich_gb300/host/rich_gpu_adapters.hpp) compile
against the reference's own plugin interfaces.  Needs the reference's sources
as oracle/ref/Makefile stages them (oracle/_ref/src, made by build() where the
reference tree is present); skipped elsewhere.  The GPU tests
(tests/test_gpu_hdsim.py) link and run the same adapters inside hdsim."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "oracle", "_ref", "src")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "source")) or not shutil.which("g++"),
                    reason="staged reference sources not present")
def test_adapters_compile_against_reference_headers():
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-w", "-include", "cassert", "-include", "cmath",
           "-I" + os.path.join(ROOT, "oracle", "ref", "shim"), "-I" + REF, "-I" + os.path.join(REF, "source"),
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "huji-rich_gb300", "host"),
           os.path.join(ROOT, "tests", "adapter_compile_check.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
