"""Tracers under a condition/action rule table (ConditionActionSequence,
ConditionActionSequence2 and LagrangianFlux with LagrangianExtensiveUpdater)
on the GPU against the reference's own fixtures (tests/golden/cas_tracers/,
oracle/ref/ref_dump.cpp's cas*_tracers forms): tracers {"A", "Z"} with "A" in
LinearGaussImproved's calc_tracers, and the case's own "obstacle" sticker
(HasSticker + SkipUpdate).  Every comparison is bit for bit.

The tracer flux of a face is Mass times the tracers of the side its action
picked: the upwind cell (RegularFlux, condition_action_sequence.cpp:111-114),
the aux-side cell of a boundary face (RigidWallFlux, FreeFlowFlux), the
interpolated face value for the ConditionActionSequence2 forms
(condition_action_sequence_2.cpp:29-40), and none for faces no action writes.
"""
import glob
import os

import numpy as np
import pytest

import oracle
import richgpu
import synthetic
from conftest import GOLDEN, load_golden, set_geometry
from test_oracle_golden import accumulate, exact

pytestmark = pytest.mark.gpu

CAS_TRACER_CASES = sorted(os.path.basename(f)[:-4]
                          for f in glob.glob(os.path.join(GOLDEN, "cas_tracers", "*.npz")))


def load_cas_tracers(name):
    return load_golden(os.path.join("cas_tracers", name))


def cas_tracer_handle(g):
    h = richgpu.Handle(gamma=g["gamma"], order=g["order"], ghost_kind=g["ghost_kind"], device=0,
                       time_integrator=1 if g["heun"] else 0)
    set_geometry(h, g)
    h.upload_mesh(g["mesh"])
    obstacle = bool(np.any(g["tr_stickers"] & 1))
    h.set_tracer_config(2, limited=[0], n_stickers=1, frozen_sticker=0 if obstacle else -1)
    h.set_stickers(g["tr_stickers"])
    h.set_flux_rules(g["flux_rules"])
    if "lagrangian_updater" in g:
        h.set_lagrangian_updater(True)
    return h


def test_fixtures_present():
    assert len(CAS_TRACER_CASES) == 4
    for name in CAS_TRACER_CASES:
        g = load_cas_tracers(name)
        # every case moves tracer mass across its faces
        assert np.count_nonzero(g["tr_fluxes"]) > g["mesh"].n_faces // 4


@pytest.mark.parametrize("name", CAS_TRACER_CASES)
def test_golden_components(name):
    g = load_cas_tracers(name)
    with cas_tracer_handle(g) as h:
        h.set_cells(g["cells0"])
        h.set_tracers(g["tr_cells0"])
        h.set_edge_velocities(g["ev_flux"])
        exact(h.flux(g["dt"]), g["fluxes"])
        exact(h.tracer_fluxes(), g["tr_fluxes"])
        if g["order"] == 2:
            exact(h.tracer_slopes(), g["tr_slopes"])
        if "lag_ws" in g:
            ws, lev = h.lagrangian_faces()
            exact(ws, g["lag_ws"])
            exact(lev, g["lag_ev"])
        h.set_extensives(g["ext0"])
        h.set_extensive_tracers(g["tr_ext0"])
        h.extensive_update(g["dt"])
        exact(h.get_extensives(), g["ext1"])
        exact(h.get_extensive_tracers(), g["tr_ext1"])
        h.cell_update()
        exact(h.get_cells(), g["cells1"])
        exact(h.get_tracers(), g["tr_cells1"])
        exact(h.get_extensive_tracers(), g["tr_ext1b"])


@pytest.mark.parametrize("name", CAS_TRACER_CASES)
def test_golden_hdsim_run(name):
    g = load_cas_tracers(name)
    steps = int(g["case_params"][3])
    with cas_tracer_handle(g) as h:
        h.set_cells(g["cells0"])
        h.set_tracers(g["tr_cells0"])
        h.set_extensives(g["ext0"])
        h.set_extensive_tracers(g["tr_ext0"])
        h.set_edge_velocities(np.zeros((g["mesh"].n_faces, 2)))
        dts = h.run(steps)
        exact(accumulate(float(g["time0"][0]), dts), g["run_times"])
        exact(h.get_extensives(), g["run_ext"])
        exact(h.get_cells(), g["run_cells"])
        exact(h.get_extensive_tracers(), g["tr_run_ext"])
        exact(h.get_tracers(), g["tr_run_cells"])


@pytest.mark.parametrize("name", CAS_TRACER_CASES)
def test_graph_steps_equal_plain_steps(name):
    """The captured step (rg_run_graph) and single rg_step calls give the
    same tracers."""
    g = load_cas_tracers(name)
    out = []
    for graph in (True, False):
        with cas_tracer_handle(g) as h:
            h.set_cells(g["cells0"])
            h.set_tracers(g["tr_cells0"])
            h.set_extensives(g["ext0"])
            h.set_extensive_tracers(g["tr_ext0"])
            h.set_edge_velocities(np.zeros((g["mesh"].n_faces, 2)))
            if graph:
                h.run_graph(4)
            else:
                for _ in range(4):
                    h.step()
            out.append((h.get_extensive_tracers(), h.get_tracers()))
    exact(out[0][0], out[1][0])
    exact(out[0][1], out[1][1])


def tracer_field(mesh, seed):
    rng = np.random.default_rng(seed)
    xy = mesh.point_xy[:mesh.n_cells]
    a = xy[:, 0] + (xy[:, 1] > 0.45) * 0.5
    z = (np.hypot(xy[:, 0] - 0.3, xy[:, 1] - 0.3) < 0.2).astype(float) + 0.01 * rng.random(mesh.n_cells)
    return np.stack([a, z], axis=1)


# rule tables: CAS2 rigid walls + obstacle faces (RigidWallFlux2) + bulk
# RegularFlux2; an outflow Ratchet with a CAS first-order wall list; and
# LagrangianFlux on every face with LagrangianExtensiveUpdater
LARGE_RULES = {
    "walls_obstacle": ([[1, 0, -1, 4, 0], [1, 2, 0, 4, 0], [1, 1, -1, 3, 0]], True, False),
    "ratchet": ([[0, 2, 0, 1, 0], [1, 0, -1, 5, 0], [1, 1, -1, 3, 0]], True, False),
    "lagrangian": ([[1, 1, -1, 6, 0, 1], [1, 0, -1, 6, 0, 2]], False, True),
}


@pytest.mark.parametrize("case", sorted(LARGE_RULES))
def test_large_runs_vs_oracle(case):
    """A 160^2 rigid box with tracers {"A" in calc_tracers, "Z"} under each
    rule table: 10 fused steps equal the oracle's (ro_step_cas_tr, pinned to
    the reference's fixtures) bit for bit, tracers included."""
    rules, obstacle, lag = LARGE_RULES[case]
    mesh = synthetic.lattice_mesh(160, 160, (0.0, 1.0, 0.0, 1.0), "rigid", seed=27)
    cells = synthetic.bumps_cells(mesh, seed=27)
    n = mesh.n_cells
    xy = mesh.point_xy[:n]
    st = ((np.hypot(xy[:, 0] - 0.4, xy[:, 1] - 0.55) < 0.12) if obstacle else np.zeros(n, bool)).astype(np.uint32)
    cells[st == 1, 2:] = 0.0
    tr = tracer_field(mesh, 27)
    ext = oracle.init_extensives(mesh, cells, 5 / 3)
    tr_ext = oracle.init_extensives_tr(mesh, cells, tr)
    ev = np.zeros((mesh.n_faces, 2))
    lp = oracle.lgi_params(ghost_kind=0)
    ts = oracle.TracerSetup(2, limited=0b01, frozen_sticker=0 if obstacle else -1, stickers=st)
    oc, oe, otr, otr_ext, odts = oracle.run_cas_tr(mesh, cells, ext, tr, tr_ext, ev, 5 / 3, 10, 2, lp, rules, ts,
                                                   lagrangian_update=lag)
    with richgpu.Handle(gamma=5 / 3, order=2, ghost_kind=0, device=0) as h:
        h.upload_mesh(mesh)
        h.set_tracer_config(2, limited=[0], n_stickers=1, frozen_sticker=0 if obstacle else -1)
        h.set_stickers(st)
        h.set_flux_rules(rules)
        if lag:
            h.set_lagrangian_updater(True)
        h.set_cells(cells)
        h.set_tracers(tr)
        h.set_extensives(ext)
        h.set_extensive_tracers(tr_ext)
        h.set_edge_velocities(ev)
        exact(h.run(10), odts)
        exact(h.get_cells(), oc)
        exact(h.get_extensives(), oe)
        exact(h.get_tracers(), otr)
        exact(h.get_extensive_tracers(), otr_ext)
    assert np.count_nonzero(otr_ext - tr_ext) > n // 10
