"""Launch shapes and the autotuner (rg_autotune / rg_set_launch_shapes).

Every per-step kernel computes each cell or face in one thread from the same
inputs and reduces only minima, so the results must be bit-identical for
every launch shape: one thread per item or a persistent grid striding over
the items, any block size.  The autotuner must leave the state unchanged.
"""
import numpy as np
import pytest

import oracle
import richgpu
import synthetic
from test_oracle_golden import exact

pytestmark = pytest.mark.gpu

SHAPES = [
    {"cfl": (64, 0), "slopes": (512, 0), "faces": (128, 0), "update": (512, 0)},
    {"cfl": (512, 152), "slopes": (64, 304), "faces": (256, 152), "update": (128, 608)},
    {"cfl": (32, 7), "slopes": (96, 5), "faces": (480, 3), "update": (64, 1)},
]
# the FP32-mixed slopes kernel's other builds (unrolled, register-capped) and the
# face kernel's two-threads-per-face build
MIXED_SHAPES = [{"slopes": (128, 0, 1)}, {"slopes": (256, 608, 2)}, {"slopes": (64, 0, 3)},
                {"slopes": (128, 0, 4)}, {"slopes": (256, 1216, 4)},
                {"update": (256, 0, 2)}, {"update": (128, 912, 3)},
                {"faces": (128, 0, 1)}, {"faces": (256, 608, 1)}, {"faces": (96, 5, 1)}]


# the FP64 slopes kernel's register-capped builds
FP64_SHAPES = [{"slopes": (256, 0, 2)}, {"slopes": (128, 608, 3)}]


def shapes_for(precision):
    return SHAPES + (MIXED_SHAPES if precision == 1 else FP64_SHAPES)


def sedov(n=160):
    mesh = synthetic.lattice_mesh(n, n, (-1.0, 1.0, -1.0, 1.0), "rigid", seed=4)
    cells = synthetic.sedov_cells(mesh, 5 / 3)
    return mesh, cells, oracle.init_extensives(mesh, cells, 5 / 3)


def run(mesh, cells, ext, precision, shapes, steps=12, heun=0, order=2):
    with richgpu.Handle(gamma=5 / 3, order=order, ghost_kind=0, precision=precision, device=0,
                        time_integrator=heun) as h:
        h.upload_mesh(mesh)
        if shapes:
            h.set_launch_shapes(shapes)
        h.set_cells(cells)
        h.set_extensives(ext)
        h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
        dts = h.run(steps)
        return h.get_cells(), h.get_extensives(), dts


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("order,heun", [(2, 0), (1, 0), (2, 1)])
def test_results_do_not_depend_on_the_launch_shape(precision, order, heun):
    mesh, cells, ext = sedov()
    ref = run(mesh, cells, ext, precision, None, heun=heun, order=order)
    for shapes in shapes_for(precision):
        got = run(mesh, cells, ext, precision, shapes, heun=heun, order=order)
        for a, b in zip(got, ref):
            exact(a, b)


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_results_do_not_depend_on_the_launch_shape(precision):
    mesh, off, gam, cells, _ = synthetic.riemann_batch(10, seed=3, min_cells=64, max_cells=3000)
    ext = np.empty_like(cells)
    for p in range(len(gam)):
        ext[off[p]:off[p + 1]] = oracle.init_extensives(mesh, cells, gam[p])[off[p]:off[p + 1]]
    outs = []
    for shapes in [None] + shapes_for(precision):
        with richgpu.Handle(gamma=1.4, order=2, ghost_kind=0, precision=precision, device=0) as h:
            h.upload_mesh(mesh)
            h.set_problems(off, gam)
            if shapes:
                h.set_launch_shapes(shapes)
            h.set_cells(cells)
            h.set_extensives(ext)
            h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
            h.run(10)
            outs.append((h.get_cells(), h.get_extensives()) + h.problem_times())
    for o in outs[1:]:
        for a, b in zip(o, outs[0]):
            exact(a, b)


@pytest.mark.parametrize("precision", [0, 1])
def test_autotune_keeps_the_state_and_the_results(precision):
    mesh, cells, ext = sedov(192)
    ref = run(mesh, cells, ext, precision, None)
    with richgpu.Handle(gamma=5 / 3, order=2, ghost_kind=0, precision=precision, device=0) as h:
        h.upload_mesh(mesh)
        h.set_cells(cells)
        h.set_extensives(ext)
        h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
        before = h.get_cells()  # FP32-mixed: the cells as stored (FP32)
        chosen = h.autotune(reps=3)
        exact(h.get_cells(), before)
        exact(h.get_extensives(), ext)
        kept = h.launch_shapes()
        for k, v in chosen.items():
            assert v["block"] in (64, 128, 256, 512) and v["ms"] > 0, (k, v)
            assert (kept[k]["block"], kept[k]["max_blocks"]) == (v["block"], v["max_blocks"])
        dts = h.run(12)
        exact(h.get_cells(), ref[0])
        exact(h.get_extensives(), ref[1])
        exact(dts, ref[2])


def test_autotune_in_batch_mode_keeps_problem_times():
    mesh, off, gam, cells, _ = synthetic.riemann_batch(8, seed=2, min_cells=64, max_cells=2000)
    ext = np.empty_like(cells)
    for p in range(len(gam)):
        ext[off[p]:off[p + 1]] = oracle.init_extensives(mesh, cells, gam[p])[off[p]:off[p + 1]]
    with richgpu.Handle(gamma=1.4, order=2, ghost_kind=0, precision=1, device=0) as h:
        h.upload_mesh(mesh)
        h.set_problems(off, gam)
        h.set_cells(cells)
        h.set_extensives(ext)
        h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
        h.run(3)
        t0, d0 = h.problem_times()
        c0, e0 = h.get_cells(), h.get_extensives()
        h.autotune(reps=2)
        t1, d1 = h.problem_times()
        exact(t1, t0)
        exact(d1, d0)
        exact(h.get_cells(), c0)
        exact(h.get_extensives(), e0)


def test_invalid_shapes_are_rejected():
    mesh, cells, ext = sedov(32)
    with richgpu.Handle(gamma=5 / 3, order=2, ghost_kind=0, device=0) as h:
        h.upload_mesh(mesh)
        for bad in ({"cfl": (48, 0)}, {"faces": (1024, 0)}, {"update": (0, 0)}, {"slopes": (64, -1)},
                    {"slopes": (128, 0, 1)}, {"slopes": (512, 0, 2)}, {"slopes": (128, 0, 4)},
                    {"faces": (128, 0, 1)}, {"update": (128, 0, 2)}):
            with pytest.raises(richgpu.RichError) as ei:
                h.set_launch_shapes(bad)
            assert ei.value.status == 1


@pytest.mark.parametrize("precision", [0, 1])
def test_fused_steps_equal_steps_with_a_cfl_pass(precision):
    """A fused step takes its dt from the previous step's update; a handle
    whose device buffers were handed out (fusion off) runs the CFL pass every
    step.  Both give the same states and dts bit for bit."""
    mesh, cells, ext = sedov(128)
    outs = []
    for external in (False, True):
        with richgpu.Handle(gamma=5 / 3, order=2, ghost_kind=0, precision=precision, device=0) as h:
            h.upload_mesh(mesh)
            if external:
                h.device_buffers()
            h.set_cells(cells)
            h.set_extensives(ext)
            h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
            dts = list(h.run(7))
            dts += [h.step() for _ in range(3)]
            h.run_graph(4)
            outs.append((h.get_cells(), h.get_extensives(), np.array(dts)))
    for a, b in zip(outs[0], outs[1]):
        exact(a, b)


def test_new_face_velocities_reach_the_next_dt():
    """Setting face velocities between fused steps: the next step's dt is the
    SimpleCFL dt of the new velocities (FP64, equal to the oracle's)."""
    mesh, cells, ext = sedov(96)
    rng = np.random.default_rng(8)
    with richgpu.Handle(gamma=5 / 3, order=2, ghost_kind=0, device=0) as h:
        h.upload_mesh(mesh)
        h.set_cells(cells)
        h.set_extensives(ext)
        h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
        h.run(3)
        ev = synthetic.face_velocities(mesh, rng.normal(0, 0.5, (mesh.n_cells, 2)))
        h.set_edge_velocities(ev)
        c3 = h.get_cells()
        dt = h.step()
    assert dt == oracle.cfl(mesh, c3, ev, 5 / 3)
