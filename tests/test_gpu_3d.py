"""3D first-order path on the GPU (rg3_* C ABI) against the reference's own
HDSim3D fixtures (tests/golden/3d/) and the oracle, bit for bit."""
import numpy as np
import pytest

import oracle
import richgpu
import synthetic
from test_oracle_golden import exact
from test_oracle_golden3d import CASES3, load3

pytestmark = pytest.mark.gpu


def handle3(gamma):
    return richgpu.Handle3(gamma=gamma, device=0)


@pytest.mark.parametrize("name", CASES3)
def test_golden_components(name):
    g = load3(name)
    with handle3(g["gamma"]) as h:
        h.upload_mesh(g["mesh"])
        h.set_cells(g["cells0"])
        h.init_extensives()
        exact(h.get_extensives(), g["ext0"])          # ExtensiveGenerator
        assert h.cfl_dt() == g["dt"][0]               # CourantFriedrichsLewy
        exact(h.flux(), g["fluxes"])                  # FirstOrderHydroFlux
        h.extensive_update(g["dt"][0])                # update_extensive
        h.cell_update()                               # DefaultCellUpdater
        exact(h.get_cells(), g["cells1"])


@pytest.mark.parametrize("name", CASES3)
def test_golden_hdsim3d_run(name):
    g = load3(name)
    steps = int(g["case_params"][3])
    with handle3(g["gamma"]) as h:
        h.upload_mesh(g["mesh"])
        h.set_cells(g["cells0"])
        h.set_extensives(g["ext0"])
        dts = h.run(steps)
        exact(dts, g["run_dts"])
        exact(h.get_cells(), g["run_cells"])


def test_blast_vs_oracle_and_conservation():
    nx, ny, nz = 24, 20, 16
    m = synthetic.cube_grid(nx, ny, nz)
    cells = synthetic.cube_blast_cells(nx, ny, nz)
    ext = oracle.init_extensives3(m, cells, 5 / 3)
    with handle3(5 / 3) as h:
        h.upload_mesh(m)
        h.set_cells(cells)
        h.set_extensives(ext)
        dts = h.run(25)
        gc, ge = h.get_cells(), h.get_extensives()
    oc, oe, odts = oracle.run3(m, cells, ext, 5 / 3, 25)
    exact(dts, odts)
    exact(ge, oe)
    exact(gc, oc)
    # the rigid walls' mass and energy fluxes are round-off (about 1e-16 per face)
    # in the reference too
    t0, t1 = ext.sum(0), ge.sum(0)
    assert abs(t1[0] - t0[0]) <= 1e-12 * t0[0]
    assert abs(t1[4] - t0[4]) <= 1e-12 * t0[4]


def test_full_size_96_cube_one_step_vs_oracle():
    """The 3D configuration's size: a 96^3 CubeGrid (884,736 cells), one
    step bit for bit."""
    n = 96
    m = synthetic.cube_grid(n, n, n, hi=(1.0, 1.0, 1.0))
    cells = synthetic.cube_blast_cells(n, n, n, hi=(1.0, 1.0, 1.0))
    ext = oracle.init_extensives3(m, cells, 5 / 3)
    with handle3(5 / 3) as h:
        h.upload_mesh(m)
        h.set_cells(cells)
        h.set_extensives(ext)
        dt = h.step()
        gc, ge = h.get_cells(), h.get_extensives()
    oc, oe, odts = oracle.run3(m, cells, ext, 5 / 3, 1)
    assert dt == odts[0]
    exact(ge, oe)
    exact(gc, oc)


def test_moving_faces_flux_vs_oracle():
    """Face velocities (Tessellation3D::CalcFaceVelocity inputs) enter the
    bulk faces' Hllc as v.n; rigid walls stay at rest."""
    m = synthetic.cube_grid(10, 8, 6)
    rng = np.random.default_rng(4)
    cells = synthetic.cube_blast_cells(10, 8, 6)
    cells[:, 2:] = rng.uniform(-0.4, 0.4, (m.n_cells, 3))
    fv = rng.normal(0, 0.3, (m.n_faces, 3))
    with handle3(5 / 3) as h:
        h.upload_mesh(m)
        h.set_cells(cells)
        h.set_face_velocities(fv)
        exact(h.flux(), oracle.flux3(m, cells, 5 / 3, fv))
        h.set_face_velocities(None)
        exact(h.flux(), oracle.flux3(m, cells, 5 / 3))


def test_negative_thermal_energy_is_reported():
    m = synthetic.cube_grid(6, 6, 6)
    cells = synthetic.cube_blast_cells(6, 6, 6)
    ext = oracle.init_extensives3(m, cells, 5 / 3)
    ext[17, 4] = 0.0  # energy below the kinetic energy
    with handle3(5 / 3) as h:
        h.upload_mesh(m)
        h.set_cells(cells)
        h.set_extensives(ext)
        with pytest.raises(richgpu.RichError) as ei:
            h.cell_update()
        assert ei.value.status == 11 and ei.value.index == 17


def test_invalid_mesh_is_rejected():
    m = synthetic.cube_grid(4, 4, 4)
    m.face_cells[5, 1] = m.n_cells + 3
    with handle3(5 / 3) as h:
        with pytest.raises(richgpu.RichError) as ei:
            h.upload_mesh(m)
        assert ei.value.status == 1


# ---------------------------------------------------------------- FP32-mixed

def run3(mesh, cells, precision, steps, gamma=5 / 3):
    with richgpu.Handle3(gamma=gamma, device=0, precision=precision) as h:
        h.upload_mesh(mesh)
        h.set_cells(cells)
        h.init_extensives()
        e0 = h.get_extensives()
        dts = h.run(steps)
        return h.get_cells(), h.get_extensives(), e0, dts


@pytest.mark.parametrize("case", ["blast32", "sedov48"])
def test_mixed_density_l1_vs_fp64_and_conservation(case):
    if case == "blast32":
        mesh, cells, steps = synthetic.cube_grid(32, 32, 32), synthetic.cube_blast_cells(32, 32, 32), 60
    else:
        box = dict(lo=(-0.5, -0.5, -0.5), hi=(0.5, 0.5, 0.5))
        mesh, cells, steps = synthetic.cube_grid(48, 48, 48, **box), synthetic.cube_sedov_cells(48), 60
    c64, _, _, _ = run3(mesh, cells, 0, steps)
    c32, e32, e0, _ = run3(mesh, cells, 1, steps)
    l1 = np.abs(c32[:, 0] - c64[:, 0]).sum() / np.abs(c64[:, 0]).sum()
    assert l1 <= 1e-5, l1
    assert np.all(np.isfinite(c32))
    # the FP32 flux of a face enters its two cells with opposite signs; walls carry no mass or energy
    assert abs(e32[:, 0].sum() - e0[:, 0].sum()) <= 1e-13 * e0[:, 0].sum()
    assert abs(e32[:, 4].sum() - e0[:, 4].sum()) <= 1e-12 * e0[:, 4].sum()


def test_mixed_split_operations_equal_the_fused_step():
    mesh = synthetic.cube_grid(20, 16, 12)
    cells = synthetic.cube_blast_cells(20, 16, 12)
    with richgpu.Handle3(gamma=5 / 3, device=0, precision=1) as h:
        h.upload_mesh(mesh)
        h.set_cells(cells)
        h.init_extensives()
        e0 = h.get_extensives()
        dt = h.step()
        fc, fe = h.get_cells(), h.get_extensives()
        h.set_cells(cells)
        h.set_extensives(e0)
        assert h.cfl_dt() == dt
        h.flux(download=False)
        h.extensive_update(dt)
        h.cell_update()
        exact(h.get_extensives(), fe)
        exact(h.get_cells(), fc)


def test_mixed_full_size_sedov_96():
    box = dict(lo=(-0.5, -0.5, -0.5), hi=(0.5, 0.5, 0.5))
    mesh, cells = synthetic.cube_grid(96, 96, 96, **box), synthetic.cube_sedov_cells(96)
    c64, _, _, _ = run3(mesh, cells, 0, 20)
    c32, _, _, _ = run3(mesh, cells, 1, 20)
    l1 = np.abs(c32[:, 0] - c64[:, 0]).sum() / np.abs(c64[:, 0]).sum()
    assert l1 <= 1e-5, l1
