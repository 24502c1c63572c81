"""The stock side of the hdsim drop-in driver (tests/hdsim_dropin.cpp) on the
CPU: every case builds a complete reference simulation (the reference's own
classes and plugins) and advances it; with a zero perturbation the
sensitivity mode's two runs are identical (the reference build is
deterministic, which the accuracy records rely on), and a perturbation
moves them apart.  Needs the driver that build() makes from the staged
reference sources; skipped where those are absent."""
import json
import os
import platform
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "oracle", "_ref", platform.machine(), "hdsim_dropin")

pytestmark = pytest.mark.skipif(not os.path.exists(DRIVER), reason="hdsim_dropin not built here")


def sensitivity(case, n, steps, delta, every):
    r = subprocess.run([DRIVER, "sensitivity", case, str(n), str(steps), repr(delta), str(every)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])


@pytest.mark.parametrize("case,n", [("sod", 12), ("sedov", 24), ("periodic", 24), ("tracers", 24), ("cas", 24)])
def test_stock_runs_are_deterministic(case, n):
    res = sensitivity(case, n, 6, 0.0, 3)
    assert [s for s, _, _ in res["l1"]] == [3, 6]
    assert all(l1 == 0.0 and dt == 0.0 for _, l1, dt in res["l1"]), res


def test_a_perturbation_is_seen():
    res = sensitivity("cas", 24, 6, 1e-6, 6)
    assert res["l1"][-1][1] > 0.0, res
