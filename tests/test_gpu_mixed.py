"""FP32-mixed form: reconstruction, HLLC and CFL in FP32 (on FP32 geometry
formed from FP64 coordinate differences); volumes, centroids, the point
motion, extensive accumulation and the internal-energy conversion in FP64.

Accuracy is stated against the FP64 path, which the other GPU tests pin
bit-for-bit to the oracle and the reference fixtures: the relative density
L1 error after N steps must stay under the tolerance written per case.
Conservation must hold to FP64 round-off (each face's flux is widened to
FP64 once and added to one cell exactly as it is taken from the other).
"""
import numpy as np
import pytest

import oracle
import richgpu
import synthetic
from test_oracle_golden import exact

pytestmark = pytest.mark.gpu

# name: (mesh args, gamma, order, ghost kind, state, steps, density L1 tolerance)
CASES = {
    "sedov_512_o2": ((512, 512, (-1.0, 1.0, -1.0, 1.0), "rigid", 2), 5 / 3, 2, 0, "sedov", 100, 1e-5),
    "sedov_128_o2": ((128, 128, (-1.0, 1.0, -1.0, 1.0), "rigid", 2), 5 / 3, 2, 0, "sedov", 200, 1e-5),
    "periodic_128_o2": ((128, 128, (0.0, 1.0, 0.0, 1.0), "periodic", 3), 5 / 3, 2, 1, "bumps", 100, 1e-5),
    "sod_200x40_o1": ((200, 40, (0.0, 1.0, 0.0, 0.2), "rigid", 1), 1.4, 1, 0, "sod", 200, 1e-5),
}


def initial(mesh, kind, gamma):
    return {"sod": synthetic.sod_cells, "sedov": lambda m: synthetic.sedov_cells(m, gamma),
            "bumps": synthetic.bumps_cells}[kind](mesh)


def run(mesh, cells, ext, gamma, order, gk, precision, steps, heun=0):
    with richgpu.Handle(gamma=gamma, order=order, ghost_kind=gk, precision=precision, device=0,
                        time_integrator=heun) as h:
        h.upload_mesh(mesh)
        h.set_cells(cells)
        h.set_extensives(ext)
        h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
        dts = h.run(steps)
        return h.get_cells(), h.get_extensives(), dts


@pytest.mark.parametrize("case", sorted(CASES))
def test_mixed_density_l1_vs_fp64(case):
    (nx, ny, box, bnd, seed), gamma, order, gk, kind, steps, tol = CASES[case]
    mesh = synthetic.lattice_mesh(nx, ny, box, bnd, seed=seed)
    cells = initial(mesh, kind, gamma)
    ext = oracle.init_extensives(mesh, cells, gamma)
    c64, e64, d64 = run(mesh, cells, ext, gamma, order, gk, 0, steps)
    c32, e32, d32 = run(mesh, cells, ext, gamma, order, gk, 1, steps)
    l1 = np.abs(c32[:, 0] - c64[:, 0]).sum() / np.abs(c64[:, 0]).sum()
    assert l1 <= tol, f"density L1 {l1:.3e} > {tol:.0e}"
    assert np.all(np.isfinite(c32))
    # conservation to FP64 round-off
    t0, t1 = ext.sum(0), e32.sum(0)
    assert abs(t1[0] - t0[0]) <= 1e-13 * abs(t0[0])
    assert abs(t1[1] - t0[1]) <= 1e-12 * abs(t0[1])


def test_mixed_heun_density_l1_vs_fp64():
    mesh = synthetic.lattice_mesh(256, 256, (-1.0, 1.0, -1.0, 1.0), "rigid", seed=2)
    gamma = 5 / 3
    cells = synthetic.sedov_cells(mesh, gamma)
    ext = oracle.init_extensives(mesh, cells, gamma)
    c64, _, _ = run(mesh, cells, ext, gamma, 2, 0, 0, 100, heun=1)
    c32, e32, _ = run(mesh, cells, ext, gamma, 2, 0, 1, 100, heun=1)
    l1 = np.abs(c32[:, 0] - c64[:, 0]).sum() / np.abs(c64[:, 0]).sum()
    assert l1 <= 1e-5, l1
    assert abs(e32[:, 0].sum() - ext[:, 0].sum()) <= 1e-13 * ext[:, 0].sum()


def test_mixed_fused_step_equals_split_plugins():
    """rg_step and the plugin sequence rg_cfl_dt / rg_flux / rg_extensive_update
    / rg_cell_update give identical results in the mixed path too."""
    mesh = synthetic.lattice_mesh(96, 96, (-1.0, 1.0, -1.0, 1.0), "rigid", seed=4)
    gamma = 5 / 3
    cells = synthetic.sedov_cells(mesh, gamma)
    ext = oracle.init_extensives(mesh, cells, gamma)
    rng = np.random.default_rng(3)
    ev = synthetic.face_velocities(mesh, rng.normal(0, 0.01, (mesh.n_cells, 2)))
    with richgpu.Handle(gamma=gamma, order=2, ghost_kind=0, precision=1, device=0) as h:
        h.upload_mesh(mesh)
        h.set_cells(cells)
        h.set_extensives(ext)
        h.set_edge_velocities(ev)
        dt = h.step()
        fused_c, fused_e = h.get_cells(), h.get_extensives()
        h.set_cells(cells)
        h.set_extensives(ext)
        assert h.cfl_dt() == dt
        h.flux(dt)
        h.extensive_update(dt)
        h.cell_update()
        assert np.array_equal(h.get_extensives(), fused_e)
        assert np.array_equal(h.get_cells(), fused_c)


def test_mixed_reports_negative_density():
    mesh = synthetic.lattice_mesh(32, 32, (0.0, 1.0, 0.0, 1.0), "periodic", seed=7)
    cells = synthetic.bumps_cells(mesh)
    ext = oracle.init_extensives(mesh, cells, 5 / 3)
    ext[12, 0] = -ext[12, 0]
    with richgpu.Handle(gamma=5 / 3, order=2, ghost_kind=1, precision=1, device=0) as h:
        h.upload_mesh(mesh)
        h.set_cells(cells)
        h.set_extensives(ext)
        h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
        with pytest.raises(richgpu.RichError) as ei:
            h.step()
        assert ei.value.status == 10 and ei.value.index == 12


def test_direct_fp32_geometry_against_rounded_fp64_geometry():
    """Without tracers an FP32-mixed upload forms the FP32 geometry straight
    from the FP64 inputs; asking for the FP64 face areas (rg_get_geometry)
    forms the FP64 geometry and rounds the FP32 copies from it.  The FP64
    motion reads the same FP64 widths and |x1 - x0| either way (point and face
    velocities bit-equal on the same state), and the states after a few
    RoundCells steps agree to FP32 round-off."""
    mesh = synthetic.lattice_mesh(128, 128, (-1.0, 1.0, -1.0, 1.0), "rigid", seed=2)
    cells = synthetic.sedov_cells(mesh, 5 / 3)
    ext = oracle.init_extensives(mesh, cells, 5 / 3)
    out = []
    for rounded in (False, True):
        with richgpu.Handle(gamma=5 / 3, order=2, ghost_kind=0, precision=1, device=0) as h:
            h.set_outer_box(-1.0, 1.0, -1.0, 1.0)
            h.upload_mesh(mesh, flags=richgpu.MESH_DEVICE_GEOMETRY)
            h.set_point_motion(kind=2, edges=0, chi=0.15, eta=0.02)
            if rounded:
                h.geometry(areas=True)
            h.set_cells(cells)
            h.set_extensives(ext)
            steps = []
            for _ in range(4):
                dt, pv = h.advance_begin()
                steps.append((dt, pv, h.edge_velocities()))
                h.cell_update()
            out.append((steps, h.get_cells(), h.get_extensives()))
    (s0, c0, e0), (s1, c1, e1) = out
    exact(s0[0][1], s1[0][1])
    exact(s0[0][2], s1[0][2])
    # the first dt reads the FP32 face velocities (formed from FP64
    # coordinate differences) and FP32 cells: an FP64 handle's dt to FP32
    # rounding
    with richgpu.Handle(gamma=5 / 3, order=2, ghost_kind=0, device=0) as h:
        h.set_outer_box(-1.0, 1.0, -1.0, 1.0)
        h.upload_mesh(mesh, flags=richgpu.MESH_DEVICE_GEOMETRY)
        h.set_point_motion(kind=2, edges=0, chi=0.15, eta=0.02)
        h.set_cells(cells)
        h.set_extensives(ext)
        dt64, _ = h.advance_begin()
    assert abs(s0[0][0] - dt64) <= 1e-6 * dt64
    for k in range(4):
        assert abs(s0[k][0] - s1[k][0]) <= 1e-6 * s1[k][0]
    l1 = np.abs(c0[:, 0] - c1[:, 0]).sum() / np.abs(c1[:, 0]).sum()
    assert l1 <= 1e-7, l1
    assert np.all(np.isfinite(c0))
    # conservation holds on either geometry
    t0 = ext.sum(0)
    assert abs(e0.sum(0)[0] - t0[0]) <= 1e-13 * abs(t0[0])
