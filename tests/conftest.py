"""Shared pytest setup: the `gpu` marker, import paths and fixture loaders."""
import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "huji-rich_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


GOLDEN_CASES = sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, "*.npz")))
# cases that also hold an N-step hdsim run on a mesh hdsim rebuilt unchanged
RUN_CASES = [c for c in GOLDEN_CASES
             if "run_mesh_unchanged" in np.load(os.path.join(GOLDEN, c + ".npz")).files]


def load_golden(name):
    """Fixture dict (arrays) + packed mesh for one golden case."""
    from meshview import PackedMesh
    z = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    z["mesh"] = PackedMesh.from_npz(z)
    z["gamma"] = float(z["gamma"][0])
    z["order"] = int(z["order"][0])
    z["ghost_kind"] = int(z["ghost_kind"][0])
    z["dt"] = float(z["dt"][0])
    z["heun"] = bool(int(z["time_integrator"])) if "time_integrator" in z else False
    return z


def set_geometry(h, g):
    """The fixture's PhysicalGeometry on a handle (before its upload)."""
    if "geometry" in g and int(g["geometry"][0]) == 1:
        h.set_physical_geometry(1, tuple(g["geometry"][1:3]), tuple(g["geometry"][3:5]))


def upload_golden(h, g, flags=0):
    """Upload the fixture's mesh with its PhysicalGeometry and, for the
    condition/action cases, its flux rules, obstacle stickers (frozen by
    HasSticker + SkipUpdate) and LagrangianExtensiveUpdater."""
    set_geometry(h, g)
    rules = g.get("flux_rules")
    stickers = g.get("tr_stickers") if rules is not None else None
    if stickers is not None:
        h.set_tracer_config(0, n_stickers=1, frozen_sticker=0)
    h.upload_mesh(g["mesh"], flags=flags)
    if stickers is not None:
        h.set_stickers(stickers.astype(np.uint32))
    if rules is not None:
        h.set_flux_rules(rules)
    if "lagrangian_updater" in g:
        h.set_lagrangian_updater(True)


@pytest.fixture(params=GOLDEN_CASES)
def golden(request):
    return load_golden(request.param)
