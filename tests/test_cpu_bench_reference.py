"""bench.py's reference arm (`--impl reference`) runs on the host cores
alone and prints the contract line: the reference's own hot path
(oracle/ref/ref_bench.cpp, built from the staged reference sources by
build()), one simulation per core, with the reference's `impl`, its
cpu_baseline and an e2e block with no host-device bytes.  Skipped where
the reference build is absent."""
import json
import os
import platform
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_BENCH = os.path.join(ROOT, "oracle", "_ref", platform.machine(), "ref_bench")


@pytest.mark.skipif(not os.path.exists(REF_BENCH), reason="ref_bench not built here")
def test_reference_arm_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    d = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "cell-updates/s"
    assert d["warmup"] >= 3 and d["steps"] == 1 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "reference" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["workload"] == "sedov2d_512x512_lgi_hllc"
