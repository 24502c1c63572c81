"""Tracers and stickers on the GPU (rg_set_tracer_config and friends) against
the reference's own tracer fixtures (tests/golden/tracers/) and the oracle.

Everything is compared bit for bit except the "Entropy" tracer, which the
reference computes with the host libm's pow() (IdealGas::dp2s) and the
library with the device pow(): that column is held to ENTROPY_RTOL of each
value plus ENTROPY_RTOL of the column's largest magnitude (a frozen cell's
extensive entropy is a running sum of fluxes of its neighbours' entropies,
where cancellation can leave a small value with the neighbours' absolute
error).  No other value depends on it (tracers do not feed back into the
hydro, and the entropy tracer is not in calc_tracers).
"""
import numpy as np
import pytest

import oracle
import richgpu
import synthetic
from test_oracle_golden import accumulate, exact
from test_oracle_golden_tracers import TRACER_CASES, load_tracers

pytestmark = pytest.mark.gpu

ENTROPY = 1                 # index of "Entropy" among the sorted names {"A", "Entropy", "Z"}
ENTROPY_RTOL = 1e-15        # a few ulp: device pow() against glibc pow()


def tracers_match(got, want):
    got, want = np.asarray(got), np.asarray(want)
    assert got.shape == want.shape
    cols = [j for j in range(got.shape[1]) if j != ENTROPY]
    exact(got[:, cols], want[:, cols])
    w = want[:, ENTROPY]
    np.testing.assert_allclose(got[:, ENTROPY], w, rtol=ENTROPY_RTOL, atol=ENTROPY_RTOL * np.abs(w).max())


def tracer_handle(g, **kw):
    kw.setdefault("time_integrator", 1 if g["heun"] else 0)
    h = richgpu.Handle(gamma=g["gamma"], order=g["order"], ghost_kind=g["ghost_kind"], device=0, **kw)
    h.upload_mesh(g["mesh"])
    h.set_tracer_config(3, limited=[0], entropy=ENTROPY, skip_sticker=1, frozen_sticker=0)
    h.set_stickers(g["tr_stickers"])
    return h


@pytest.mark.parametrize("name", TRACER_CASES)
def test_golden_components(name):
    g = load_tracers(name)
    with tracer_handle(g) as h:
        h.set_cells(g["cells0"])
        h.set_tracers(g["tr_cells0"])
        h.set_edge_velocities(g["ev_flux"])
        exact(h.flux(g["dt"]), g["fluxes"])
        exact(h.tracer_fluxes(), g["tr_fluxes"])
        if g["order"] == 2:
            exact(h.tracer_slopes(), g["tr_slopes"])
        h.set_extensives(g["ext0"])
        h.set_extensive_tracers(g["tr_ext0"])
        h.extensive_update(g["dt"])
        exact(h.get_extensives(), g["ext1"])
        exact(h.get_extensive_tracers(), g["tr_ext1"])
        h.cell_update()
        exact(h.get_cells(), g["cells1"])
        tracers_match(h.get_tracers(), g["tr_cells1"])
        tracers_match(h.get_extensive_tracers(), g["tr_ext1b"])


@pytest.mark.parametrize("name", [c for c in TRACER_CASES if c != "sedov_tracers_o2"])
def test_golden_hdsim_run(name):
    g = load_tracers(name)
    steps = int(g["case_params"][3])
    with tracer_handle(g) as h:
        h.set_cells(g["cells0"])
        h.set_tracers(g["tr_cells0"])
        h.set_extensives(g["ext0"])
        h.set_extensive_tracers(g["tr_ext0"])
        h.set_edge_velocities(np.zeros((g["mesh"].n_faces, 2)))
        dts = h.run(steps)
        exact(accumulate(float(g["time0"][0]), dts), g["run_times"])
        exact(h.get_extensives(), g["run_ext"])
        exact(h.get_cells(), g["run_cells"])
        tracers_match(h.get_extensive_tracers(), g["tr_run_ext"])
        tracers_match(h.get_tracers(), g["tr_run_cells"])


def test_init_extensives():
    g = load_tracers("sod_tracers_o1")
    with tracer_handle(g) as h:
        h.set_cells(g["cells0"])
        h.set_tracers(g["tr_cells0"])
        h.init_extensives()
        exact(h.get_extensives(), g["ext0"])
        exact(h.get_extensive_tracers(), g["tr_ext0"])


def big_case(n, boundary, seed=9):
    box = (0.0, 1.0, 0.0, 1.0)
    mesh = synthetic.lattice_mesh(n, n, box, boundary=boundary, seed=seed)
    cells = synthetic.bumps_cells(mesh, seed=seed)
    rng = np.random.default_rng(seed)
    nt = 5
    tr = rng.uniform(-1, 1, (mesh.n_cells, nt))
    tr[:, 3] = np.where(rng.random(mesh.n_cells) < 0.5, 0.0, 1.0)  # a step tracer
    stickers = (rng.random(mesh.n_cells) < 0.05).astype(np.uint32) | \
        ((rng.random(mesh.n_cells) < 0.08).astype(np.uint32) << 3)
    return mesh, cells, tr, stickers


@pytest.mark.parametrize("boundary,order,heun", [("periodic", 2, False), ("rigid", 2, False), ("rigid", 1, False),
                                               ("rigid", 2, True), ("periodic", 2, True)])
def test_large_run_vs_oracle(boundary, order, heun):
    """A 160^2 lattice, five tracers (three limited), the entropy tracer,
    5% frozen cells and 8% limiter-skipped cells: 12 fused steps (hdsim's
    TimeAdvance or TimeAdvance2Heun) against the oracle."""
    mesh, cells, tr, stickers = big_case(160, boundary)
    gamma, steps = 5 / 3, 12
    ghost = 1 if boundary == "periodic" else 0
    ts = oracle.TracerSetup(5, limited=0b10101, entropy=1, skip_sticker=3, frozen_sticker=0, stickers=stickers)
    ext = oracle.init_extensives(mesh, cells, gamma)
    tr_ext = oracle.init_extensives_tr(mesh, cells, tr)
    ev = np.zeros((mesh.n_faces, 2))
    lp = oracle.lgi_params(ghost_kind=ghost)
    oc, oe, otr, ote, odts = oracle.run_tr(mesh, cells, ext, tr, tr_ext, ev, gamma, steps, ts, 0.3, order, lp,
                                           heun=heun)
    with richgpu.Handle(gamma=gamma, order=order, ghost_kind=ghost, device=0, time_integrator=1 if heun else 0) as h:
        h.upload_mesh(mesh)
        h.set_tracer_config(5, limited=[0, 2, 4], entropy=1, skip_sticker=3, frozen_sticker=0)
        h.set_stickers(stickers)
        h.set_cells(cells)
        h.set_tracers(tr)
        h.init_extensives()
        h.set_edge_velocities(ev)
        dts = h.run(steps)
        exact(dts, odts)
        exact(h.get_cells(), oc)
        exact(h.get_extensives(), oe)
        tracers_match(h.get_tracers(), otr)
        tracers_match(h.get_extensive_tracers(), ote)


def test_graph_steps_equal_plain_steps():
    mesh, cells, tr, stickers = big_case(64, "periodic", seed=4)
    outs = []
    for graph in (False, True):
        with richgpu.Handle(gamma=5 / 3, order=2, ghost_kind=1, device=0) as h:
            h.upload_mesh(mesh)
            h.set_tracer_config(5, limited=[0, 1], entropy=2, skip_sticker=3, frozen_sticker=0)
            h.set_stickers(stickers)
            h.set_cells(cells)
            h.set_tracers(tr)
            h.init_extensives()
            h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
            if graph:
                h.run_graph(9)
            else:
                h.run(9)
            outs.append((h.get_cells(), h.get_tracers(), h.get_extensive_tracers()))
    for a, b in zip(*outs):
        exact(a, b)


def test_stickers_only_without_tracers():
    """Stickers alone (no tracers): frozen cells keep their cells, the skip
    sticker changes the hydro slopes exactly as the oracle."""
    mesh, cells, _, stickers = big_case(48, "rigid", seed=2)
    ts = oracle.TracerSetup(0, skip_sticker=3, frozen_sticker=0, stickers=stickers)
    ext = oracle.init_extensives(mesh, cells, 5 / 3)
    ev = np.zeros((mesh.n_faces, 2))
    oc, oe, _, _, odts = oracle.run_tr(mesh, cells, ext, np.zeros((mesh.n_cells, 0)), np.zeros((mesh.n_cells, 0)),
                                       ev, 5 / 3, 6, ts, 0.3, 2, oracle.lgi_params(ghost_kind=0))
    with richgpu.Handle(gamma=5 / 3, order=2, ghost_kind=0, device=0) as h:
        h.upload_mesh(mesh)
        h.set_tracer_config(0, skip_sticker=3, frozen_sticker=0)
        h.set_stickers(stickers)
        h.set_cells(cells)
        h.set_extensives(ext)
        h.set_edge_velocities(ev)
        exact(h.run(6), odts)
        exact(h.get_cells(), oc)
        exact(h.get_extensives(), oe)
        frozen = (stickers & 1) == 1
        exact(h.get_cells()[frozen], cells[frozen])


MIXED_L1 = 1e-5  # relative L1 of the FP32-mixed path against FP64, per column


def rel_l1(a, b):
    return float(np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-300))


@pytest.mark.parametrize("boundary,order,problems", [("rigid", 2, 1), ("periodic", 2, 1), ("rigid", 1, 1),
                                                    ("rigid", 2, 2)])
def test_fp32_mixed_tracers_against_fp64(boundary, order, problems):
    """Tracers and stickers on the FP32-mixed path: its FP32 hydro passes
    keep each cell's shock decision and each face's mass flux, honour the
    skip_key and SkipUpdate stickers, and the FP64 tracer passes run on
    them.  12 fused steps of the 160^2 case (five tracers, the entropy
    tracer, 5% frozen and 8% limiter-skipped cells) against the FP64 path:
    density and every tracer column within 1e-5 relative L1, the frozen
    cells' states unchanged, the dt sequence within FP32 rounding.  With
    two problems the mesh is split in a batch (per-problem dt)."""
    mesh, cells, tr, stickers = big_case(160, boundary)
    gamma, steps = 5 / 3, 12
    ghost = 1 if boundary == "periodic" else 0
    offsets = None
    if problems > 1:
        # two independent copies of the case (the second seeded differently)
        m2, c2, t2, s2 = big_case(96, boundary, seed=5)
        mesh, offsets = synthetic.concat_meshes([mesh, m2])
        cells, tr, stickers = np.vstack([cells, c2]), np.vstack([tr, t2]), np.concatenate([stickers, s2])
    outs = []
    for precision in (0, 1):
        with richgpu.Handle(gamma=gamma, order=order, ghost_kind=ghost, device=0, precision=precision) as h:
            h.upload_mesh(mesh)
            if problems > 1:
                h.set_problems(offsets, [gamma, 1.4])
            h.set_tracer_config(5, limited=[0, 2, 4], entropy=1, skip_sticker=3, frozen_sticker=0)
            h.set_stickers(stickers)
            h.set_cells(cells)
            h.set_tracers(tr)
            h.init_extensives()
            h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
            dts = h.run(steps)
            outs.append((dts, h.get_cells(), h.get_tracers(), h.get_extensive_tracers()))
    (d64, c64, t64, e64), (d32, c32, t32, e32) = outs
    if problems == 1:
        np.testing.assert_allclose(d32, d64, rtol=1e-5)
    assert rel_l1(c32[:, 0], c64[:, 0]) <= MIXED_L1
    for j in range(5):
        assert rel_l1(t32[:, j], t64[:, j]) <= MIXED_L1, j
        assert rel_l1(e32[:, j], e64[:, j]) <= MIXED_L1, j
    frozen = (stickers & 1) == 1
    exact(c32[frozen], cells[frozen].astype(np.float32).astype(np.float64))


def test_unsupported_combinations_and_readiness():
    mesh, cells, tr, _ = big_case(16, "rigid", seed=1)
    with richgpu.Handle(gamma=5 / 3, order=2, ghost_kind=0, device=0, precision=1) as h:
        h.set_tracer_config(2)                           # FP32-mixed hdsim::TimeAdvance carries tracers
    with richgpu.Handle(gamma=5 / 3, order=2, ghost_kind=0, device=0, precision=1, time_integrator=1) as h:
        with pytest.raises(richgpu.RichError) as ei:
            h.set_tracer_config(2)                       # not the FP32-mixed fused TimeAdvance2Heun
        assert ei.value.status == 1
    with richgpu.Handle(gamma=5 / 3, order=2, ghost_kind=0, device=0, time_integrator=1) as h:
        h.set_tracer_config(0, frozen_sticker=0)          # TimeAdvance2Heun carries tracers and stickers
    with richgpu.Handle(gamma=5 / 3, order=2, ghost_kind=0, device=0) as h:
        h.upload_mesh(mesh)
        with pytest.raises(richgpu.RichError):
            h.set_tracer_config(9)                       # more than RG_MAX_TRACERS
        with pytest.raises(richgpu.RichError):
            h.set_tracer_config(2, entropy=2)            # entropy index out of range
        h.set_tracer_config(5, limited=[0])
        h.set_cells(cells)
        h.init_extensives()
        h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
        with pytest.raises(richgpu.RichError) as ei:
            h.step()                                     # tracers not set
        assert ei.value.status == 3
        h.set_tracers(tr)
        h.init_extensives()
        h.step()
        h.set_problems([0, mesh.n_cells], [5 / 3])       # a batch of one problem carries tracers too
        h.step()
        h.set_tracer_config(0)
        h.step()                                         # tracers off again
