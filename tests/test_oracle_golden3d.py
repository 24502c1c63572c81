"""The 3D first-order oracle (oracle/rich_oracle.c, ro3_*) and the CubeGrid
packer (synthetic.cube_grid) against fixtures written by the reference's own
HDSim3D (CubeGrid, FirstOrderHydroFlux(Hllc), DefaultCellUpdater,
CourantFriedrichsLewy; oracle/ref/ref_dump3d.cpp), bit for bit."""
import glob
import os

import numpy as np
import pytest

import oracle
import synthetic
from conftest import GOLDEN
from meshview import MESH3_FIELDS, PackedMesh3D
from test_oracle_golden import exact

CASES3 = sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, "3d", "*.npz")))


def load3(name):
    z = dict(np.load(os.path.join(GOLDEN, "3d", name + ".npz")))
    z["mesh"] = PackedMesh3D.from_npz(z)
    z["gamma"] = float(z["gamma"][0])
    return z


@pytest.mark.parametrize("name", CASES3)
def test_packer_reproduces_the_reference_mesh(name):
    g = load3(name)
    nx, ny, nz = (int(v) for v in g["case_params"][:3])
    m = synthetic.cube_grid(nx, ny, nz)
    for k in MESH3_FIELDS:
        exact(getattr(m, k), getattr(g["mesh"], k))


@pytest.mark.parametrize("name", CASES3)
def test_oracle_components(name):
    g = load3(name)
    m, gam = g["mesh"], g["gamma"]
    exact(oracle.init_extensives3(m, g["cells0"], gam), g["ext0"])             # ExtensiveGenerator
    assert oracle.cfl3(m, g["cells0"], gam) == g["dt"][0]                     # CourantFriedrichsLewy
    exact(oracle.flux3(m, g["cells0"], gam), g["fluxes"])                     # FirstOrderHydroFlux
    ext1 = oracle.extensive_update3(m, g["fluxes"], g["dt"][0], g["ext0"])    # update_extensive
    exact(oracle.cell_update3(m, ext1, gam), g["cells1"])                     # DefaultCellUpdater


@pytest.mark.parametrize("name", CASES3)
def test_oracle_hdsim3d_run(name):
    g = load3(name)
    steps = int(g["case_params"][3])
    cells, ext, dts = oracle.run3(g["mesh"], g["cells0"], g["ext0"], g["gamma"], steps)
    exact(dts, g["run_dts"])
    exact(cells, g["run_cells"])


def test_oracle_conserves_in_a_closed_box():
    m = synthetic.cube_grid(10, 9, 8)
    cells = synthetic.cube_blast_cells(10, 9, 8)
    ext0 = oracle.init_extensives3(m, cells, 5 / 3)
    _, ext, _ = oracle.run3(m, cells, ext0, 5 / 3, 20)
    t0, t1 = ext0.sum(0), ext.sum(0)
    assert abs(t1[0] - t0[0]) <= 1e-12 * t0[0]
    assert abs(t1[4] - t0[4]) <= 1e-12 * t0[4]
