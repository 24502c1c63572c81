"""The RICH-side adapters (huji-rich_gb300/host/rich_gpu_adapters.hpp) compile
against the reference's own plugin interfaces.  Needs the reference source
tree (only where the fixtures are generated); skipped elsewhere."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("RICH_SOURCE_TREE", "/root/reference")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "source")) or not shutil.which("g++"),
                    reason="reference source tree not present")
def test_adapters_compile_against_reference_headers():
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-w", "-include", "cassert", "-include", "cmath",
           "-I" + os.path.join(ROOT, "oracle", "ref", "shim"), "-I" + REF, "-I" + os.path.join(REF, "source"),
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "huji-rich_gb300", "host"),
           os.path.join(ROOT, "tests", "adapter_compile_check.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
