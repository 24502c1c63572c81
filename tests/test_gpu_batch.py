"""Batched form: independent problems of uneven size in one handle, each with
its own gamma and SimpleCFL dt, advanced by one launch per phase or (FP32-mixed,
RG_STEP_PERSISTENT) by one cooperative launch for the whole run.  Every
problem of a batch must evolve exactly as it does alone (FP64: bit-for-bit,
and the same for the FP32-mixed path, whose kernels are per cell and per
face too), and a CUDA-graph replay must equal rg_run."""
import numpy as np
import pytest

import oracle
import richgpu
import synthetic
from test_oracle_golden import accumulate, exact

pytestmark = pytest.mark.gpu


def small_batch(seed=5, n=12):
    return synthetic.riemann_batch(n, seed=seed, min_cells=64, max_cells=2500)


def init_ext(mesh, cells, offsets, gammas):
    ext = np.empty_like(cells)
    for p in range(len(gammas)):
        a, b = offsets[p], offsets[p + 1]
        sub = oracle.init_extensives(mesh, cells, gammas[p])
        ext[a:b] = sub[a:b]
    return ext


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("heun", [0, 1])
def test_batch_equals_problems_alone(precision, heun):
    """hdsim::TimeAdvance, and TimeAdvance2Heun (each problem's dt held for
    both halves), of a batch equal every problem's solo run."""
    mesh, off, gam, cells, meshes = small_batch()
    ext = init_ext(mesh, cells, off, gam)
    steps = 15
    with richgpu.Handle(gamma=1.4, order=2, ghost_kind=0, precision=precision, device=0,
                        time_integrator=heun) as h:
        h.upload_mesh(mesh)
        h.set_problems(off, gam)
        h.set_cells(cells)
        h.set_extensives(ext)
        h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
        h.run(steps)
        bc, be = h.get_cells(), h.get_extensives()
        times, last = h.problem_times()
    for p, m in enumerate(meshes):
        a, b = off[p], off[p + 1]
        with richgpu.Handle(gamma=gam[p], order=2, ghost_kind=0, precision=precision, device=0,
                            time_integrator=heun) as h:
            h.upload_mesh(m)
            h.set_cells(cells[a:b])
            h.set_extensives(ext[a:b])
            h.set_edge_velocities(np.zeros((m.n_faces, 2)))
            dts = h.run(steps)
            exact(bc[a:b], h.get_cells())
            exact(be[a:b], h.get_extensives())
        assert times[p] == accumulate(0.0, dts)[-1]
        assert last[p] == dts[-1]


def test_batch_fp64_matches_oracle_per_problem():
    mesh, off, gam, cells, meshes = small_batch(seed=9, n=6)
    ext = init_ext(mesh, cells, off, gam)
    with richgpu.Handle(gamma=1.4, order=2, ghost_kind=0, device=0) as h:
        h.upload_mesh(mesh)
        h.set_problems(off, gam)
        h.set_cells(cells)
        h.set_extensives(ext)
        h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
        h.run(5)
        bc = h.get_cells()
    for p, m in enumerate(meshes):
        a, b = off[p], off[p + 1]
        oc, _, _ = oracle.run(m, cells[a:b], ext[a:b], np.zeros((m.n_faces, 2)), gam[p], 5, 0.3, 2,
                              oracle.lgi_params(0))
        exact(bc[a:b], oc)


@pytest.mark.parametrize("batch", [False, True])
def test_graph_replay_equals_run(batch):
    if batch:
        mesh, off, gam, cells, _ = small_batch(seed=2, n=8)
        ext = init_ext(mesh, cells, off, gam)
    else:
        mesh = synthetic.lattice_mesh(96, 96, (-1.0, 1.0, -1.0, 1.0), "rigid", seed=2)
        cells = synthetic.sedov_cells(mesh)
        ext = oracle.init_extensives(mesh, cells, 5 / 3)
    out = []
    for graph in (False, True):
        with richgpu.Handle(gamma=5 / 3, order=2, ghost_kind=0, device=0) as h:
            h.upload_mesh(mesh)
            if batch:
                h.set_problems(off, gam)
            h.set_cells(cells)
            h.set_extensives(ext)
            h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
            if graph:
                h.run_graph(12)
            else:
                h.run(12)
            out.append((h.get_cells(), h.get_extensives()))
    exact(out[0][0], out[1][0])
    exact(out[0][1], out[1][1])


def test_batch_rejects_face_between_problems():
    mesh = synthetic.lattice_mesh(16, 16, (0.0, 1.0, 0.0, 1.0), "rigid", seed=1)
    with richgpu.Handle(gamma=1.4, order=2, ghost_kind=0, device=0) as h:
        h.upload_mesh(mesh)
        with pytest.raises(richgpu.RichError) as ei:
            h.set_problems([0, 100, mesh.n_cells], [1.4, 1.4])   # cuts through the lattice
        assert ei.value.status == 1
        h.set_problems([0, mesh.n_cells], [1.4])
        with pytest.raises(richgpu.RichError):
            h.cfl_dt()                                       # not available in batch mode


def test_batch_init_extensives_per_problem_gamma():
    """hdsim's init_extensives on a batch, formed on the device with each
    problem's gamma, equals the oracle's per problem bit for bit."""
    mesh, off, gam, cells, meshes = small_batch(seed=9, n=9)
    with richgpu.Handle(gamma=1.4, order=2, ghost_kind=0, device=0) as h:
        h.upload_mesh(mesh)
        h.set_problems(off, gam)
        h.set_cells(cells)
        h.init_extensives()
        exact(h.get_extensives(), init_ext(mesh, cells, off, gam))


def test_batch_heun_fp64_matches_oracle_per_problem():
    """TimeAdvance2Heun on a batch against the oracle's Heun step per problem."""
    mesh, off, gam, cells, meshes = small_batch(seed=13, n=5)
    ext = init_ext(mesh, cells, off, gam)
    with richgpu.Handle(gamma=1.4, order=2, ghost_kind=0, device=0, time_integrator=1) as h:
        h.upload_mesh(mesh)
        h.set_problems(off, gam)
        h.set_cells(cells)
        h.set_extensives(ext)
        h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
        h.run(5)
        bc, be = h.get_cells(), h.get_extensives()
    for p, m in enumerate(meshes):
        a, b = off[p], off[p + 1]
        oc, oe, _ = oracle.run(m, cells[a:b], ext[a:b], np.zeros((m.n_faces, 2)), gam[p], 5, 0.3, 2,
                               oracle.lgi_params(0), heun=True)
        exact(bc[a:b], oc)
        exact(be[a:b], oe)


@pytest.mark.parametrize("heun", [0, 1])
def test_batch_with_tracers_equals_problems_alone(heun):
    """Tracers and stickers in a batch: three tracers (one limited, the
    entropy tracer with each problem's gamma), frozen and limiter-skipped
    cells; every problem's cells, extensives and tracers bit for bit as
    alone, with TimeAdvance and TimeAdvance2Heun."""
    mesh, off, gam, cells, meshes = small_batch(seed=21, n=7)
    rng = np.random.default_rng(21)
    n = mesh.n_cells
    tr = np.stack([rng.uniform(-1, 1, n), cells[:, 1], (rng.random(n) < 0.5).astype(float)], axis=1)
    st = (rng.random(n) < 0.03).astype(np.uint32) | ((rng.random(n) < 0.05).astype(np.uint32) << 1)
    steps = 8

    def configure(h, o, g, c, t, s):
        h.set_tracer_config(3, limited=[0], entropy=1, skip_sticker=1, frozen_sticker=0)
        if o is not None:
            h.set_problems(o, g)
        h.set_stickers(s)
        h.set_cells(c)
        h.set_tracers(t)
        h.init_extensives()

    with richgpu.Handle(gamma=1.4, order=2, ghost_kind=0, device=0, time_integrator=heun) as h:
        h.upload_mesh(mesh)
        configure(h, off, gam, cells, tr, st)
        h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
        h.run(steps)
        bc, be, bt, bte = h.get_cells(), h.get_extensives(), h.get_tracers(), h.get_extensive_tracers()
    for p, m in enumerate(meshes):
        a, b = off[p], off[p + 1]
        with richgpu.Handle(gamma=gam[p], order=2, ghost_kind=0, device=0, time_integrator=heun) as h:
            h.upload_mesh(m)
            configure(h, None, None, cells[a:b], tr[a:b], st[a:b])
            h.set_edge_velocities(np.zeros((m.n_faces, 2)))
            h.run(steps)
            exact(bc[a:b], h.get_cells())
            exact(be[a:b], h.get_extensives())
            exact(bt[a:b], h.get_tracers())
            exact(bte[a:b], h.get_extensive_tracers())


def batch_handle(mesh, off, gam, cells, ext, precision=1, heun=0):
    h = richgpu.Handle(gamma=1.4, order=2, ghost_kind=0, precision=precision, device=0, time_integrator=heun)
    h.upload_mesh(mesh)
    h.set_problems(off, gam)
    h.set_cells(cells)
    h.set_extensives(ext)
    h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
    return h


@pytest.mark.parametrize("seed,n", [(5, 12), (7, 40)])
def test_persistent_run_equals_per_phase_run(seed, n):
    """RG_STEP_PERSISTENT (the batch run in one cooperative launch, grid
    barriers between the phases) gives the per-phase launches' cells,
    extensives, problem times and dts bit for bit."""
    mesh, off, gam, cells, _ = synthetic.riemann_batch(n, seed=seed, min_cells=64, max_cells=2500)
    ext = init_ext(mesh, cells, off, gam)
    out = []
    for mode in (richgpu.STEP_PER_PHASE, richgpu.STEP_PERSISTENT):
        with batch_handle(mesh, off, gam, cells, ext) as h:
            h.set_step_mode(mode)
            dts = list(h.run(9))
            h.run_graph(4)
            dts += list(h.run(3))
            out.append((h.get_cells(), h.get_extensives(), np.array(dts)) + h.problem_times())
    for a, b in zip(out[0], out[1]):
        exact(a, b)


def test_persistent_mode_where_it_applies():
    mesh, off, gam, cells, _ = small_batch()
    ext = init_ext(mesh, cells, off, gam)
    with batch_handle(mesh, off, gam, cells, ext, precision=0) as h:
        with pytest.raises(richgpu.RichError):
            h.set_step_mode(richgpu.STEP_PERSISTENT)        # FP64 batches run one launch per phase
    with batch_handle(mesh, off, gam, cells, ext, heun=1) as h:
        with pytest.raises(richgpu.RichError):
            h.set_step_mode(richgpu.STEP_PERSISTENT)        # TimeAdvance only
    with batch_handle(mesh, off, gam, cells, ext) as h:
        with pytest.raises(richgpu.RichError):
            h.set_step_mode(2)
        h.set_step_mode(richgpu.STEP_PERSISTENT)
        h.set_tracer_config(0, n_stickers=1)
        with pytest.raises(richgpu.RichError) as ei:
            h.run(1)                                        # no stickers or tracers in the persistent form
        assert ei.value.status == 1
        h.set_tracer_config(0)
        h.run(2)
        h.set_step_mode(richgpu.STEP_PER_PHASE)
        h.run(1)


def test_grid_barrier_wait_runs_out_and_the_handle_stays_usable():
    """The persistent form's barrier with a block that never arrives: the
    bounded wait ends the launch with RG_ERR_TIMEOUT (about a second), and
    the next launches run normally."""
    mesh, off, gam, cells, _ = small_batch()
    ext = init_ext(mesh, cells, off, gam)
    with batch_handle(mesh, off, gam, cells, ext) as h:
        h.grid_barrier_check(0)
        with pytest.raises(richgpu.RichError) as ei:
            h.grid_barrier_check(1)
        assert ei.value.status == 16 and ei.value.phase == 7
        h.grid_barrier_check(0)
        h.set_step_mode(richgpu.STEP_PERSISTENT)
        h.run(3)
        assert np.all(np.isfinite(h.get_cells()))
