"""Device-side geometry and point motion (RG_MESH_DEVICE_GEOMETRY,
rg_set_point_motion, rg_advance_begin) against the reference's fixtures and
the oracle, bit for bit.

Each fixture records the point velocities hdsim::TimeAdvance computed before
and after PointMotion::ApplyFix (pv_cfl, pv_flux), the face velocities of
both (ev_cfl, ev_flux), the reference's volumes and CMs (mesh_*), the
OuterBoundary's box and the case's motion (Eulerian, Lagrangian,
RoundCells hot, or RoundCells cold with CorrectPointsOverShoot).
"""
import numpy as np
import pytest

import oracle
import richgpu
import synthetic
from conftest import GOLDEN_CASES, load_golden, upload_golden
from test_oracle_golden import exact

pytestmark = pytest.mark.gpu

DG = richgpu.MESH_DEVICE_GEOMETRY


def motion_kw(g):
    k, edges, chi, eta, cold, fix = g["motion"]
    return dict(kind=int(k), edges=int(edges), chi=float(chi), eta=float(eta), cold=bool(cold),
                correct_overshoot=bool(fix))


def device_handle(g, **kw):
    h = richgpu.Handle(gamma=g["gamma"], order=g["order"], ghost_kind=g["ghost_kind"], device=0, **kw)
    h.set_outer_box(*g["outer_box"])
    upload_golden(h, g, flags=DG)
    return h


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_device_geometry(name):
    """Volumes, CMs (real and ghost) and the PhysicalGeometry's CacheData
    volumes and face areas (SlabSymmetry, CylindricalSymmetry)."""
    g = load_golden(name)
    m = g["mesh"]
    with device_handle(g) as h:
        vol, cm, cdv, areas = h.geometry(areas=True)
    exact(vol, m.volume)
    exact(cm, m.cm_xy)
    exact(cdv, m.cd_volume)
    exact(areas, g["mesh_cd_area"])


def test_cylindrical_areas_with_uploaded_geometry():
    """CylindricalSymmetry with the caller's CacheData volumes uploaded: the
    device still forms the face areas, and a pass matches the reference."""
    g = load_golden("cyl_blast_o2")
    with richgpu.Handle(gamma=g["gamma"], order=2, ghost_kind=0, device=0) as h:
        upload_golden(h, g)
        exact(h.geometry(areas=True)[3], g["mesh_cd_area"])
        h.set_cells(g["cells0"])
        h.set_extensives(g["ext0"])
        h.set_edge_velocities(g["ev_flux"])
        exact(h.flux(g["dt"]), g["fluxes"])
        h.extensive_update(g["dt"])
        exact(h.get_extensives(), g["ext1"])
        h.set_physical_geometry(0)
        h.upload_mesh(g["mesh"])                 # back to SlabSymmetry: edge lengths
        d = g["mesh"].face_vertices[:, 0:2] - g["mesh"].face_vertices[:, 2:4]
        exact(h.geometry(areas=True)[3], np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]))


def test_cylindrical_mixed_precision_run():
    """The FP32-mixed path scales its fluxes by the cylindrical areas too:
    10 steps stay close to the FP64 path's."""
    g = load_golden("cyl_blast_o2")
    out = []
    for precision in (0, 1):
        with richgpu.Handle(gamma=g["gamma"], order=2, ghost_kind=0, device=0, precision=precision) as h:
            h.set_outer_box(*g["outer_box"])
            upload_golden(h, g, flags=DG)
            h.set_cells(g["cells0"])
            h.set_extensives(g["ext0"])
            h.set_edge_velocities(np.zeros((g["mesh"].n_faces, 2)))
            h.run(10)
            out.append(h.get_cells())
    exact(out[0], g["run_cells"])
    l1 = np.abs(out[1][:, 0] - out[0][:, 0]).sum() / np.abs(out[0][:, 0]).sum()
    assert l1 < 1e-5, l1


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_point_motion_and_edge_velocities(name):
    g = load_golden(name)
    with device_handle(g) as h:
        h.set_point_motion(**motion_kw(g))
        h.set_cells(g["cells0"])
        exact(h.point_velocities(), g["pv_cfl"])
        exact(h.edge_velocities(), g["ev_cfl"])
        assert h.cfl_dt() == g["dt"]
        exact(h.apply_fix(g["dt"]), g["pv_flux"])
        exact(h.edge_velocities(), g["ev_flux"])


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_advance_begin_and_cell_update(name):
    """rg_advance_begin (motion, dt, ApplyFix, fluxes, extensive update in one
    enqueue) then rg_cell_update on the same mesh: the reference's pass."""
    g = load_golden(name)
    with device_handle(g) as h:
        h.set_point_motion(**motion_kw(g))
        h.set_cells(g["cells0"])
        h.set_extensives(g["ext0"])
        dt, pv = h.advance_begin()
        assert dt == g["dt"]
        exact(pv, g["pv_flux"])
        exact(h.get_extensives(), g["ext1"])
        h.cell_update()
        exact(h.get_cells(), g["cells1"])


def test_large_round_cells_vs_oracle():
    """A 256^2 rigid box, RoundCells cold with the overshoot correction on a
    flow into the walls: device geometry and one advance against the oracle."""
    box = (0.0, 1.0, 0.0, 1.0)
    mesh = synthetic.lattice_mesh(256, 256, box, boundary="rigid", seed=12, jitter=0.05)
    cells = synthetic.bumps_cells(mesh, seed=3, amp=0.5)
    cells[:, 1] = 0.02
    cells[:, 2] += 0.8
    gamma = 5 / 3
    vol, cm, cdv = oracle.cell_geometry(mesh, 0, box)
    exact(vol, mesh.volume)        # the packer's geometry is the oracle's
    mo = oracle.motion(2, 0, 0.15, 0.02, 1, 1, box)
    pv = oracle.point_velocities(mesh, cells, gamma, mo)
    ev = oracle.edge_velocities(mesh, mo, pv)
    dt = oracle.cfl(mesh, cells, ev, gamma, 0.3)
    pv0 = pv
    pv = oracle.apply_fix(mesh, cells, gamma, mo, dt, pv)
    assert (pv != pv0).any(axis=1).sum() > 1000     # the cold correction acts
    ev = oracle.edge_velocities(mesh, mo, pv)
    ext = oracle.init_extensives(mesh, cells, gamma)
    fl = oracle.modular_flux(mesh, cells, ev, gamma, oracle.lgi_params(ghost_kind=0))
    ext1 = oracle.extensive_update(mesh, fl, dt, ext)
    with richgpu.Handle(gamma=gamma, order=2, ghost_kind=0, device=0) as h:
        h.set_outer_box(*box)
        h.upload_mesh(mesh, flags=DG)
        gv, gcm, gcd = h.geometry()
        exact(gv, vol)
        exact(gcm, cm)
        exact(gcd, cdv)
        h.set_point_motion(kind=2, edges=0, cold=True, correct_overshoot=True)
        h.set_cells(cells)
        h.set_extensives(ext)
        gdt, gpv = h.advance_begin()
        assert gdt == dt
        exact(gpv, pv)
        exact(h.edge_velocities(), ev)
        exact(h.get_extensives(), ext1)


def test_mixed_precision_advance():
    """The FP32-mixed path with device geometry and motion: runs, and its dt
    and extensives stay close to the FP64 path's."""
    g = load_golden("sedov_o2")
    out = []
    for precision in (0, 1):
        with device_handle(g, precision=precision) as h:
            h.set_point_motion(**motion_kw(g))
            h.set_cells(g["cells0"])
            h.set_extensives(g["ext0"])
            dt, pv = h.advance_begin()
            out.append((dt, pv, h.get_extensives()))
    (d64, p64, e64), (d32, p32, e32) = out
    assert abs(d32 - d64) <= 1e-6 * d64
    assert np.allclose(p32, p64, rtol=1e-5, atol=1e-9)
    assert np.allclose(e32, e64, rtol=1e-5, atol=1e-12)


def test_motion_argument_checks():
    g = load_golden("sedov_o2")
    with richgpu.Handle(gamma=g["gamma"], order=2, ghost_kind=0, device=0) as h:
        with pytest.raises(richgpu.RichError):
            h.upload_mesh(g["mesh"], flags=DG)       # rigid ghosts need the box
        with pytest.raises(richgpu.RichError):
            h.set_point_motion(kind=2, correct_overshoot=True)
        with pytest.raises(richgpu.RichError):
            h.set_outer_box(1.0, -1.0, -1.0, 1.0)
        with pytest.raises(richgpu.RichError):
            h.set_point_motion(kind=7)
