"""GPU parity: the CUDA path through the C ABI against the reference fixtures
and the oracle, bit-for-bit (IEEE ==, FP64 plain path).

Golden cases come from the reference itself (tests/golden/); larger meshes
come from synthetic.lattice_mesh and are checked against the oracle
(oracle/rich_oracle.c), which is pinned to the reference by
test_oracle_golden.py.
"""
import ctypes

import numpy as np
import pytest

import oracle
import richgpu
import synthetic
from conftest import GOLDEN_CASES, RUN_CASES, load_golden, upload_golden
from test_oracle_golden import accumulate, areas_of, exact, oracle_pass

pytestmark = pytest.mark.gpu


def handle_for(gamma, order, ghost_kind, **kw):
    return richgpu.Handle(gamma=gamma, order=order, ghost_kind=ghost_kind, device=0, **kw)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_golden_components(name):
    """Each plugin operation on the reference's inputs gives the reference's outputs."""
    g = load_golden(name)
    with handle_for(g["gamma"], g["order"], g["ghost_kind"]) as h:
        upload_golden(h, g)
        h.set_cells(g["cells0"])
        h.set_edge_velocities(g["ev_cfl"])
        assert h.cfl_dt() == g["dt"]                                  # SimpleCFL
        h.set_edge_velocities(g["ev_flux"])
        exact(h.flux(g["dt"]), g["fluxes"])                            # FluxCalculator
        h.set_extensives(g["ext0"])
        h.extensive_update(g["dt"])                                    # SimpleExtensiveUpdater
        exact(h.get_extensives(), g["ext1"])
        h.cell_update()                                                # SimpleCellUpdater
        exact(h.get_cells(), g["cells1"])


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_golden_extensive_update_from_host_fluxes(name):
    """The extensive updater also accepts fluxes computed elsewhere (rg_set_fluxes)."""
    g = load_golden(name)
    with handle_for(g["gamma"], g["order"], g["ghost_kind"]) as h:
        upload_golden(h, g)
        h.set_extensives(g["ext0"])
        h.set_fluxes(g["fluxes"])
        if "lag_ws" in g:
            # LagrangianExtensiveUpdater reads its LagrangianFlux's face data
            h.set_lagrangian_faces(g["lag_ws"], g["lag_ev"])
        h.extensive_update(g["dt"])
        exact(h.get_extensives(), g["ext1"])


@pytest.mark.parametrize("name", RUN_CASES)
def test_golden_hdsim_run(name):
    """rg_run reproduces N hdsim::TimeAdvance (or TimeAdvance2Heun) steps on a
    fixed mesh exactly."""
    g = load_golden(name)
    steps = int(g["case_params"][3])
    with handle_for(g["gamma"], g["order"], g["ghost_kind"], time_integrator=int(g["heun"])) as h:
        upload_golden(h, g)
        h.set_cells(g["cells0"])
        h.set_extensives(g["ext0"])
        h.set_edge_velocities(np.zeros((g["mesh"].n_faces, 2)))
        dts = h.run(steps)
        exact(accumulate(float(g["time0"][0]), dts), g["run_times"])
        exact(h.get_extensives(), g["run_ext"])
        exact(h.get_cells(), g["run_cells"])


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_golden_fused_step(name):
    """rg_step (dt on the device) equals the split plugin sequence."""
    g = load_golden(name)
    with handle_for(g["gamma"], g["order"], g["ghost_kind"]) as h:
        upload_golden(h, g)
        h.set_cells(g["cells0"])
        h.set_extensives(g["ext0"])
        h.set_edge_velocities(g["ev_cfl"])
        dt = h.step()
        cells, ext = h.get_cells(), h.get_extensives()
    oc, oe, odts = oracle_pass(g, g["cells0"], g["ext0"], g["ev_cfl"], heun=False)
    assert dt == odts[0]
    exact(ext, oe)
    exact(cells, oc)


def moving_faces(mesh, seed, scale):
    rng = np.random.default_rng(seed)
    pv = rng.normal(0, scale, (mesh.n_cells, 2))
    return synthetic.face_velocities(mesh, pv)


CASES = {
    # name: (mesh args, gamma, order, ghost kind, state)
    "sod_200x40_o1": ((200, 40, (0.0, 1.0, 0.0, 0.2), "rigid", 1), 1.4, 1, 0, "sod"),
    "sedov_128_o2": ((128, 128, (-1.0, 1.0, -1.0, 1.0), "rigid", 2), 5 / 3, 2, 0, "sedov"),
    "periodic_128_o2": ((128, 128, (0.0, 1.0, 0.0, 1.0), "periodic", 3), 5 / 3, 2, 1, "bumps"),
    "periodic_96x64_o1": ((96, 64, (0.0, 1.0, 0.0, 1.0), "periodic", 4), 5 / 3, 1, 1, "bumps"),
}


def initial(mesh, kind, gamma):
    return {"sod": synthetic.sod_cells, "sedov": lambda m: synthetic.sedov_cells(m, gamma),
            "bumps": synthetic.bumps_cells}[kind](mesh)


@pytest.mark.parametrize("case", sorted(CASES))
def test_synthetic_multistep_vs_oracle(case):
    """20 fused steps on a larger seeded mesh equal 20 oracle steps."""
    (nx, ny, box, bnd, seed), gamma, order, gk, kind = CASES[case]
    mesh = synthetic.lattice_mesh(nx, ny, box, bnd, seed=seed)
    cells = initial(mesh, kind, gamma)
    ext = oracle.init_extensives(mesh, cells, gamma)
    ev = np.zeros((mesh.n_faces, 2))
    with handle_for(gamma, order, gk) as h:
        h.upload_mesh(mesh)
        h.set_cells(cells)
        h.init_extensives()
        exact(h.get_extensives(), ext)                                 # hdsim init_extensives
        h.set_edge_velocities(ev)
        dts = h.run(20)
        gc, ge = h.get_cells(), h.get_extensives()
    oc, oe, odts = oracle.run(mesh, cells, ext, ev, gamma, 20, 0.3, order, oracle.lgi_params(gk))
    exact(dts, odts)
    exact(ge, oe)
    exact(gc, oc)


@pytest.mark.parametrize("case", sorted(CASES))
def test_synthetic_heun_vs_oracle(case):
    """10 fused TimeAdvance2Heun steps equal 10 oracle Heun steps."""
    (nx, ny, box, bnd, seed), gamma, order, gk, kind = CASES[case]
    mesh = synthetic.lattice_mesh(nx, ny, box, bnd, seed=seed)
    cells = initial(mesh, kind, gamma)
    ext = oracle.init_extensives(mesh, cells, gamma)
    ev = np.zeros((mesh.n_faces, 2))
    with handle_for(gamma, order, gk, time_integrator=1) as h:
        h.upload_mesh(mesh)
        h.set_cells(cells)
        h.set_extensives(ext)
        h.set_edge_velocities(ev)
        dts = h.run(10)
        gc, ge = h.get_cells(), h.get_extensives()
    oc, oe, odts = oracle.run(mesh, cells, ext, ev, gamma, 10, 0.3, order, oracle.lgi_params(gk), heun=True)
    exact(dts, odts)
    exact(ge, oe)
    exact(gc, oc)


@pytest.mark.parametrize("case", sorted(CASES))
def test_synthetic_moving_faces_vs_oracle(case):
    """Non-zero face velocities (moving-mesh boost) on every plugin operation."""
    (nx, ny, box, bnd, seed), gamma, order, gk, kind = CASES[case]
    mesh = synthetic.lattice_mesh(nx, ny, box, bnd, seed=seed)
    cells = initial(mesh, kind, gamma)
    ext = oracle.init_extensives(mesh, cells, gamma)
    ev = moving_faces(mesh, seed, 0.05)
    with handle_for(gamma, order, gk) as h:
        h.upload_mesh(mesh)
        h.set_cells(cells)
        h.set_extensives(ext)
        h.set_edge_velocities(ev)
        dt = h.cfl_dt()
        assert dt == oracle.cfl(mesh, cells, ev, gamma)
        fl = h.flux(dt)
        ofl = (oracle.simple_flux(mesh, cells, ev, gamma) if order == 1
               else oracle.modular_flux(mesh, cells, ev, gamma, oracle.lgi_params(gk)))
        exact(fl, ofl)
        h.extensive_update(dt)
        oe = oracle.extensive_update(mesh, ofl, dt, ext)
        exact(h.get_extensives(), oe)
        h.cell_update()
        exact(h.get_cells(), oracle.cell_update(mesh, oe, gamma))


def test_full_size_sedov_512_one_step_vs_oracle():
    """The headline 512x512 Sedov configuration: one fused step, bit-exact."""
    mesh = synthetic.lattice_mesh(512, 512, (-1.0, 1.0, -1.0, 1.0), "rigid", seed=2)
    gamma = 5 / 3
    cells = synthetic.sedov_cells(mesh, gamma)
    ext = oracle.init_extensives(mesh, cells, gamma)
    ev = moving_faces(mesh, 9, 1e-3)
    with handle_for(gamma, 2, 0) as h:
        h.upload_mesh(mesh)
        h.set_cells(cells)
        h.set_extensives(ext)
        h.set_edge_velocities(ev)
        dt = h.step()
        gc, ge = h.get_cells(), h.get_extensives()
    oc, oe, odt = oracle.step(mesh, cells, ext, ev, gamma, 0.3, 2, oracle.lgi_params(0))
    assert dt == odt
    exact(ge, oe)
    exact(gc, oc)


def test_full_size_sedov_512_100_steps_vs_oracle():
    """The headline 512x512 Sedov configuration over 100 fused steps with
    moving faces: cells, extensives and every dt equal the oracle's (density
    L1 exactly 0)."""
    mesh = synthetic.lattice_mesh(512, 512, (-1.0, 1.0, -1.0, 1.0), "rigid", seed=2)
    gamma = 5 / 3
    cells = synthetic.sedov_cells(mesh, gamma)
    ext = oracle.init_extensives(mesh, cells, gamma)
    ev = moving_faces(mesh, 9, 1e-3)
    with handle_for(gamma, 2, 0) as h:
        h.upload_mesh(mesh)
        h.set_cells(cells)
        h.set_extensives(ext)
        h.set_edge_velocities(ev)
        dts = h.run(100)
        gc, ge = h.get_cells(), h.get_extensives()
    oc, oe, odts = oracle.run(mesh, cells, ext, ev, gamma, 100, 0.3, 2, oracle.lgi_params(0))
    exact(dts, odts)
    exact(ge, oe)
    exact(gc, oc)


def test_full_size_conservation_and_determinism():
    """512x512 Sedov, 100 fused steps: mass, momentum and energy conserved to
    round-off; a second run is bitwise identical (no atomics on the data path)."""
    mesh = synthetic.lattice_mesh(512, 512, (-1.0, 1.0, -1.0, 1.0), "rigid", seed=2)
    gamma = 5 / 3
    cells = synthetic.sedov_cells(mesh, gamma)
    ext0 = oracle.init_extensives(mesh, cells, gamma)
    outs = []
    for _ in range(2):
        with handle_for(gamma, 2, 0) as h:
            h.upload_mesh(mesh)
            h.set_cells(cells)
            h.set_extensives(ext0)
            h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
            dts = h.run(100)
            outs.append((h.get_cells(), h.get_extensives(), dts))
    c1, e1, d1 = outs[0]
    c2, e2, d2 = outs[1]
    assert np.array_equal(c1, c2) and np.array_equal(e1, e2) and np.array_equal(d1, d2)
    tot0, tot1 = ext0.sum(0), e1.sum(0)
    assert abs(tot1[0] - tot0[0]) <= 1e-13 * abs(tot0[0])                # mass
    assert abs(tot1[1] - tot0[1]) <= 1e-12 * abs(tot0[1])                # energy
    assert abs(tot1[2]) <= 1e-12 and abs(tot1[3]) <= 1e-12               # momentum (starts at 0)
    assert np.all(np.isfinite(c1))


def test_condition_action_large_vs_oracle():
    """ConditionActionSequence2 on a 192^2 rigid box: rigid walls, an obstacle
    of sticker cells (frozen), outflow ratchets are exercised on a second
    case; 12 fused steps against the oracle."""
    mesh = synthetic.lattice_mesh(192, 192, (0.0, 1.0, 0.0, 1.0), "rigid", seed=21)
    cells = synthetic.bumps_cells(mesh, seed=21)
    n = mesh.n_cells
    xy = mesh.point_xy[:n]
    st = (np.hypot(xy[:, 0] - 0.4, xy[:, 1] - 0.55) < 0.12).astype(np.uint32)
    cells[st == 1, 2:] = 0.0
    ext = oracle.init_extensives(mesh, cells, 5 / 3)
    ev = np.zeros((mesh.n_faces, 2))
    lp = oracle.lgi_params(ghost_kind=0)
    for rules in ([[1, 0, -1, 4, 0], [1, 2, 0, 4, 0], [1, 1, -1, 3, 0]],
                  [[0, 2, 0, 1, 0], [1, 0, -1, 5, 0], [1, 1, -1, 3, 0]]):
        oc, oe, odts = oracle.run_cas(mesh, cells, ext, ev, 5 / 3, 12, 2, lp, rules, st, 1)
        with richgpu.Handle(gamma=5 / 3, order=2, ghost_kind=0, device=0) as h:
            h.set_tracer_config(0, n_stickers=1, frozen_sticker=0)
            h.upload_mesh(mesh)
            h.set_stickers(st)
            h.set_flux_rules(rules)
            h.set_cells(cells)
            h.set_extensives(ext)
            h.set_edge_velocities(ev)
            exact(h.run(12), odts)
            exact(h.get_cells(), oc)
            exact(h.get_extensives(), oe)


@pytest.mark.parametrize("massflux", [1, 2, 3])
def test_lagrangian_flux_large_vs_oracle(massflux):
    """LagrangianFlux on every face (bulk faces take rs, the wall faces rs2
    by WallsMassFlux) with LagrangianExtensiveUpdater on a 160^2 rigid box,
    for each LagrangianHLLC massflux pairing, 10 fused steps against the
    oracle; then one pass on moving faces with the per-face ws and speeds."""
    mesh = synthetic.lattice_mesh(160, 160, (0.0, 1.0, 0.0, 1.0), "rigid", seed=23)
    cells = synthetic.bumps_cells(mesh, seed=23)
    ext = oracle.init_extensives(mesh, cells, 5 / 3)
    ev = np.zeros((mesh.n_faces, 2))
    lp = oracle.lgi_params(ghost_kind=0)
    rules = [[1, 1, -1, 6, 0, massflux], [1, 0, -1, 6, 0, massflux]]
    oc, oe, odts = oracle.run_cas(mesh, cells, ext, ev, 5 / 3, 10, 2, lp, rules, lagrangian_update=True)
    pv = cells[:, 2:4].copy()
    mev = synthetic.face_velocities(mesh, pv)
    of, ows, oev = oracle.cas_flux(mesh, cells, mev, 5 / 3, 2, lp, rules, lagrangian=True)
    with richgpu.Handle(gamma=5 / 3, order=2, ghost_kind=0, device=0) as h:
        h.upload_mesh(mesh)
        h.set_flux_rules(rules)
        h.set_lagrangian_updater(True)
        h.set_cells(cells)
        h.set_extensives(ext)
        h.set_edge_velocities(ev)
        exact(h.run(10), odts)
        exact(h.get_cells(), oc)
        exact(h.get_extensives(), oe)
        h.set_cells(cells)
        h.set_edge_velocities(mev)
        exact(h.flux(odts[0]), of)
        ws, lev = h.lagrangian_faces()
    exact(ws, ows)
    exact(lev, oev)
    assert np.count_nonzero(ows) > 0 and np.count_nonzero(oev) > 0


@pytest.mark.parametrize("name", ["cas2_lag_o2", "cas2_lag_move_o2"])
def test_lagrangian_faces_vs_reference(name):
    """LagrangianFlux's per-face ws_ and edge_vel_ after a flux pass, against
    the reference's own (the fluxes, extensives and cells of these cases are
    in the golden-case tests above)."""
    g = load_golden(name)
    with handle_for(g["gamma"], g["order"], g["ghost_kind"]) as h:
        upload_golden(h, g)
        h.set_cells(g["cells0"])
        h.set_extensives(g["ext0"])
        h.set_edge_velocities(g["ev_flux"])
        exact(h.flux(g["dt"]), g["fluxes"])
        ws, lev = h.lagrangian_faces()
        exact(ws, g["lag_ws"])
        exact(lev, g["lag_ev"])
        h.extensive_update(g["dt"])
        exact(h.get_extensives(), g["ext1"])


def test_condition_action_rules_checked():
    mesh = synthetic.lattice_mesh(16, 16, (0.0, 1.0, 0.0, 1.0), "rigid", seed=3)
    with richgpu.Handle(gamma=5 / 3, order=1, ghost_kind=0, device=0) as h:
        h.upload_mesh(mesh)
        with pytest.raises(richgpu.RichError):
            h.set_flux_rules([[1, 1, -1, 3, 0]])           # ConditionActionSequence2 needs order 2
        with pytest.raises(richgpu.RichError):
            h.set_flux_rules([[0, 2, 0, 1, 0]])            # RegularSpecialEdge without stickers kept
        with pytest.raises(richgpu.RichError):
            h.set_flux_rules([[0, 1, -1, 6, 0, 1]])        # LagrangianFlux is a ConditionActionSequence2 action
        h.set_flux_rules([[0, 1, -1, 0, 0]])               # bulk edges only: boundary faces match nothing
        h.set_cells(synthetic.sod_cells(mesh))
        h.init_extensives()
        h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
        with pytest.raises(richgpu.RichError) as ei:
            h.step()
        assert ei.value.status == 1 and ei.value.phase == 3
        h.set_flux_rules([])
        h.step()


@pytest.mark.parametrize("precision", [0, 1])
def test_upload_overlapped_with_running_steps(precision):
    """hdsim's loop on an Eulerian mesh rebuilds the same tessellation every
    step: rg_step_async enqueues a step on one mesh slot and rg_upload_mesh
    fills the other slot (side stream) while that step runs.  The cells and
    extensives equal a run without the interleaved uploads, bit for bit, and
    every upload sees the step before it finished."""
    mesh = synthetic.lattice_mesh(192, 192, (-1.0, 1.0, -1.0, 1.0), "rigid", seed=4)
    gamma = 5 / 3
    cells = synthetic.sedov_cells(mesh, gamma)
    ext0 = oracle.init_extensives(mesh, cells, gamma)
    outs = []
    for interleave in (False, True):
        with handle_for(gamma, 2, 0, precision=precision) as h:
            h.upload_mesh(mesh)
            h.set_cells(cells)
            h.set_extensives(ext0)
            h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
            dts = []
            for _ in range(8):
                if interleave:
                    h.step_async()
                    h.upload_mesh(mesh)
                    dts.append(h.synchronize())
                else:
                    dts.append(h.step())
            outs.append((h.get_cells(), h.get_extensives(), np.array(dts)))
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("precision", [0, 1])
def test_state_download_overlapped_with_next_upload(precision):
    """A moving-mesh caller's loop: upload the tessellation (device
    geometry), hdsim::TimeAdvance's first half (rg_advance_begin: RoundCells
    motion, dt, fluxes, extensive update), the cell update, then the cells
    and extensives back to the host.  With rg_get_state_async the download
    of step k runs while the mesh of step k+1 is uploaded; every step's
    cells, extensives and dt equal the synchronous loop's bit for bit."""
    torch = pytest.importorskip("torch")
    mesh = synthetic.lattice_mesh(160, 160, (-1.0, 1.0, -1.0, 1.0), "rigid", seed=4)
    gamma = 5 / 3
    cells = synthetic.sedov_cells(mesh, gamma)
    ext0 = oracle.init_extensives(mesh, cells, gamma)

    def pinned(shape):
        return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()

    runs = []
    for overlap in (False, True):
        with handle_for(gamma, 2, 0, precision=precision) as h:
            h.set_outer_box(-1.0, 1.0, -1.0, 1.0)
            h.upload_mesh(mesh, flags=richgpu.MESH_DEVICE_GEOMETRY)
            h.set_point_motion(kind=2, edges=0, chi=0.15, eta=0.02)
            h.set_cells(cells)
            h.set_extensives(ext0)
            bufs = [(pinned((mesh.n_cells, 4)), pinned((mesh.n_cells, 4))) for _ in range(2)]
            out = []
            pending = None
            for k in range(6):
                h.upload_mesh(mesh, flags=richgpu.MESH_DEVICE_GEOMETRY)
                if pending is not None:
                    h.wait_state()
                    out.append(tuple(a.copy() for a in pending))
                dt, _ = h.advance_begin()
                h.cell_update()
                c_out, e_out = bufs[k % 2]
                if overlap:
                    h.get_state_async(c_out, e_out)
                    pending = (c_out, e_out, np.array([dt]))
                else:
                    out.append((h.get_cells(), h.get_extensives(), np.array([dt])))
            if pending is not None:
                h.wait_state()
                out.append(tuple(a.copy() for a in pending))
        runs.append(out)
    assert len(runs[0]) == len(runs[1]) == 6
    for a, b in zip(*runs):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


TINY = [(1, "rigid"), (2, "rigid"), (3, "rigid"), (2, "periodic"), (3, "periodic"), (5, "periodic")]


@pytest.mark.parametrize("nx,boundary", TINY)
@pytest.mark.parametrize("order", [1, 2])
def test_tiny_meshes_vs_oracle(nx, boundary, order):
    """The smallest tessellations: one cell walled in by four ghosts, 2x2
    and 3x3 lattices whose periodic images make a cell its own neighbour's
    neighbour several times over.  Five steps, bit for bit; the FP32-mixed
    path runs them too."""
    mesh = synthetic.lattice_mesh(nx, nx, (0.0, 1.0, 0.0, 1.0), boundary, seed=3)
    cells = synthetic.bumps_cells(mesh) if boundary == "periodic" else synthetic.sod_cells(mesh)
    gamma, ghost_kind = 1.4, 1 if boundary == "periodic" else 0
    ext = oracle.init_extensives(mesh, cells, gamma)
    ev = np.zeros((mesh.n_faces, 2))
    c_ref, e_ref, dt_ref = oracle.run(mesh, cells, ext, ev, gamma, 5, order=order,
                                      lp=oracle.lgi_params(ghost_kind=ghost_kind))
    for precision in (0, 1):
        with handle_for(gamma, order, ghost_kind, precision=precision) as h:
            h.upload_mesh(mesh)
            h.set_cells(cells)
            h.set_extensives(ext)
            h.set_edge_velocities(ev)
            dts = h.run(5)
            c, e = h.get_cells(), h.get_extensives()
        if precision == 0:
            exact(c, c_ref)
            exact(e, e_ref)
            assert np.array_equal(dts, dt_ref)
        else:
            assert np.all(np.isfinite(c))
            assert np.allclose(c[:, 0], c_ref[:, 0], rtol=1e-4)


def test_empty_mesh_rejected():
    """A view with no cells is refused on the host, before any device work."""
    mesh = synthetic.lattice_mesh(4, 4, (0.0, 1.0, 0.0, 1.0), "periodic", seed=1)
    with handle_for(1.4, 2, 1) as h:
        v = mesh.view()
        n0 = v.n_cells
        v.n_cells = 0
        try:
            with pytest.raises(richgpu.RichError) as ei:
                h._check(h.lib.rg_upload_mesh(h.h, ctypes.byref(v), 0))
        finally:
            v.n_cells = n0
        assert ei.value.status == 1
