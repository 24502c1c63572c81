"""hdsim driven through the GPU plugins, against hdsim driven through the
reference's own plugins.

tests/hdsim_dropin.cpp builds two complete RICH simulations of a case from
the reference's own classes (VoronoiMesh, the outer boundary, point motion,
edge velocities, hdsim) that differ only in their plugin set: SimpleCFL,
SimpleFluxCalculator or ModularFluxCalculator(LinearGaussImproved, Hllc),
SimpleExtensiveUpdater and SimpleCellUpdater, or GpuCFL, GpuFluxCalculator,
GpuExtensiveUpdater and GpuCellUpdater (huji-rich_gb300/host/
rich_gpu_adapters.hpp over librich_gb300.so).  It advances both with
hdsim::TimeAdvance (or TimeAdvance2Heun) and compares, after every step,
every cell, extensive, tracer, mesh point and the time with ==.  The host
rebuilds each simulation's Voronoi mesh every step where the points move.

The driver is built by build() (oracle/ref/Makefile, target dropin); a
missing driver is a failure, not a skip.
"""
import json
import os
import platform
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "oracle", "_ref", platform.machine(), "hdsim_dropin")
DRIVER3D = os.path.join(ROOT, "oracle", "_ref", platform.machine(), "hdsim3d_dropin")


def run_driver(*args, timeout=900, exe=DRIVER):
    assert os.path.exists(exe), (
        f"{exe} is missing: build() builds it (make -C oracle/ref dropin) from the staged reference sources")
    r = subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, timeout=timeout)
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert lines, f"driver printed no result (rc {r.returncode}):\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}"
    return r.returncode, json.loads(lines[-1]), r.stderr


@pytest.mark.parametrize("case,n,steps,geometry", [
    # Sod 200 x 40, Eulerian, first order, 200 steps
    ("sod", 40, 200, "device"),
    # Sedov 128^2, RoundCells(Lagrangian): the mesh moves and is rebuilt on
    # the host every step (and Hilbert-reordered every 25 steps)
    ("sedov", 128, 200, "device"),
    # the same with the host tessellation's own volumes and CMs uploaded
    ("sedov", 96, 100, "hostgeom"),
    # periodic 64^2, Eulerian, TimeAdvance2Heun
    ("periodic", 64, 60, "device"),
    # Sedov 64^2 with RoundCells, three tracers and two stickers (the
    # "Entropy" tracer, p * pow(d, -gamma), within 1e-15 relative: libm's pow
    # against the device's)
    ("tracers", 64, 60, "device"),
    # Sedov 64^2 with RoundCells and ConditionActionSequence2 (rigid-wall and
    # regular face-value fluxes; the GPU set: the same rule table) carrying
    # tracers {"A", "Z"}
    ("cas", 64, 60, "device"),
])
def test_hdsim_with_gpu_plugins_equals_hdsim_with_reference_plugins(case, n, steps, geometry):
    extra = ["hostgeom"] if geometry == "hostgeom" else []
    rc, res, err = run_driver("compare", case, n, steps, *extra)
    assert res["device_geometry"] == (geometry == "device")
    assert res["equal"], (f"{case}: first differing step {res['first_differing_step']}, "
                          f"{res['differing_values']} values differ\n{err[-2000:]}")
    assert rc == 0
    assert res["cycle"] == steps and res["time"] > 0


def test_hdsim_with_gpu_plugins_fp32_mixed_accuracy_on_moving_mesh():
    """FP32-mixed plugins against FP64 plugins on Sedov 128^2 with RoundCells
    (host Voronoi rebuild every step), 200 steps; the stock plugins run too
    and the FP64 plugins must equal them."""
    rc, res, err = run_driver("accuracy", "sedov", 128, 200, "stock")
    assert rc == 0, err[-2000:]
    assert res["fp64_equal_to_stock"], res
    assert res["unmatched"] == 0
    # density L1 of the FP32-mixed path against FP64, relative
    assert res["l1_density_fp32mixed_vs_fp64"] <= 1e-5, res


def test_hdsim_with_gpu_plugins_fp32_mixed_tracers():
    """The FP32-mixed plugins with tracers and stickers (the tracers case:
    Sedov 64^2 with RoundCells, {"A", "Entropy", "Z"}, frozen and
    limiter-skipped cells) against the FP64 plugins through hdsim, 60
    steps: density and every tracer within 1e-5 relative L1."""
    rc, res, err = run_driver("accuracy", "tracers", 64, 60)
    assert rc == 0, err[-2000:]
    assert res["unmatched"] == 0
    assert res["l1_density_fp32mixed_vs_fp64"] <= 1e-5, res
    assert res["l1_tracers_fp32mixed_vs_fp64"] <= 1e-5, res


@pytest.mark.parametrize("case,n,steps", [
    # Sedov-Taylor on a 24^3 CubeGrid (the 3D configuration's problem, smaller)
    ("sedov", 24, 30),
    # seeded states in every cell: every Hllc branch, tangential flow
    ("random", 10, 12),
    # a Sod tube along x
    ("sod", 16, 30),
])
def test_hdsim3d_with_gpu_plugins_equals_hdsim3d_with_reference_plugins(case, n, steps):
    """HDSim3D::timeAdvance with GpuTimeStep3D and GpuFluxCalculator3D
    (rich_gpu_adapters3d.hpp) against CourantFriedrichsLewy and
    FirstOrderHydroFlux(Hllc): cells and each step's dt equal after every
    step (tests/hdsim3d_dropin.cpp)."""
    rc, res, err = run_driver("compare", case, n, steps, exe=DRIVER3D)
    assert res["equal"], (f"{case}: first differing step {res['first_differing_step']}, "
                          f"{res['differing_values']} values differ\n{err[-2000:]}")
    assert rc == 0
