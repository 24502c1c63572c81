"""Differentiation form: rg_step_fwd / rg_step_bwd (adjoint with checkpoints)
and rg_step_tlm (tangent-linear) through the C ABI.

The map is n fixed-dt hdsim::TimeAdvance steps of periodic
LinearGaussImproved + Hllc from the initial cells W_0 to the final cells W_n;
the loss of the adjoint workload is the L2 distance of the final density to
a second seeded field.  Checks:
  * the forward is the plain FP64 step bit for bit (oracle composition);
  * the tangent-linear run carries the same values bit for bit;
  * dot-product test <Wbar, TLM dW> = <ADJ Wbar, dW> to round-off;
  * central finite differences (eps = 1e-6, random directions) of the oracle
    forward (small mesh) and of the GPU forward (the 256x256, 200-step
    workload, checkpoints every 20 steps) to 1e-6 relative where the map is
    smooth (limiter off), and, with the reference's limiter on, in the
    directions in which no limiter switch lies within eps;
  * a torch.autograd.Function wrapping the fwd/bwd pair.
"""
import numpy as np
import pytest

import oracle
import richgpu
import synthetic
from test_oracle_golden import exact

pytestmark = pytest.mark.gpu

GAMMA = 5 / 3


def problem(nx, ny, seed=3):
    mesh = synthetic.lattice_mesh(nx, ny, (0.0, 1.0, 0.0, 1.0), "periodic", seed=seed)
    cells = synthetic.bumps_cells(mesh)
    target = synthetic.bumps_cells(mesh, seed=11)[:, 0]
    return mesh, cells, target


def handle(mesh, **kw):
    h = richgpu.Handle(gamma=GAMMA, order=2, ghost_kind=1, device=0, **kw)
    h.upload_mesh(mesh)
    h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
    return h


def cfl_dt(h, cells):
    h.set_cells(cells)
    return h.cfl_dt()


def loss(cells_n, target):
    r = cells_n[:, 0] - target
    return float(r @ r)


def loss_seed(cells_n, target):
    wbar = np.zeros_like(cells_n)
    wbar[:, 0] = 2.0 * (cells_n[:, 0] - target)
    return wbar


def fwd(h, cells, steps, dt, every=20):
    h.set_cells(cells)
    h.step_fwd(steps, dt, every)
    return h.get_cells()


def test_forward_is_the_plain_fp64_step_bit_for_bit():
    mesh, cells, _ = problem(48, 40)
    with handle(mesh) as h:
        dt = cfl_dt(h, cells)
        wn = fwd(h, cells, 12, dt, every=5)
        en = h.get_extensives()
    oc, oe = oracle.run_fixed_dt(mesh, cells, GAMMA, 12, dt)
    exact(wn, oc)
    exact(en, oe)


def test_tangent_run_carries_the_forward_values_bit_for_bit():
    mesh, cells, _ = problem(64, 64)
    rng = np.random.default_rng(1)
    with handle(mesh) as h:
        dt = cfl_dt(h, cells)
        wn = fwd(h, cells, 15, dt)
        h.set_cells(cells)
        h.step_tlm(15, dt, rng.normal(size=cells.shape))
        exact(h.get_cells(), wn)


@pytest.mark.parametrize("steps,every", [(30, 7), (12, 20), (9, 1)])
def test_dot_product_adjoint_vs_tangent_linear(steps, every):
    mesh, cells, target = problem(96, 80)
    rng = np.random.default_rng(steps)
    with handle(mesh) as h:
        dt = cfl_dt(h, cells)
        wn = fwd(h, cells, steps, dt, every)
        wbar = rng.normal(size=cells.shape)
        g = h.step_bwd(wbar)
        dw = rng.normal(size=cells.shape)
        h.set_cells(cells)
        tl = h.step_tlm(steps, dt, dw)
    lhs, rhs = float(np.sum(wbar * tl)), float(np.sum(g * dw))
    assert abs(lhs - rhs) <= 1e-11 * max(abs(lhs), abs(rhs)), (lhs, rhs)
    assert np.all(np.isfinite(g)) and np.all(np.isfinite(wn))


def test_backward_is_deterministic_and_leaves_the_state():
    mesh, cells, target = problem(64, 48)
    with handle(mesh) as h:
        dt = cfl_dt(h, cells)
        wn = fwd(h, cells, 25, dt, every=6)
        seed = loss_seed(wn, target)
        g1 = h.step_bwd(seed)
        g2 = h.step_bwd(seed)
        exact(h.get_cells(), wn)
    assert np.array_equal(g1, g2)


def test_checkpoint_interval_does_not_change_the_gradient():
    mesh, cells, target = problem(64, 48)
    grads = []
    with handle(mesh) as h:
        dt = cfl_dt(h, cells)
        for every in (1, 4, 13, 40):
            wn = fwd(h, cells, 26, dt, every)
            grads.append(h.step_bwd(loss_seed(wn, target)))
    for g in grads[1:]:
        assert np.array_equal(g, grads[0])


def smooth_lp():
    """LinearGaussImproved without its slope limiter: the step is then a
    smooth map away from HLLC wave-speed switches."""
    return oracle.lgi_params(1, slf=0)


def test_adjoint_vs_central_differences_of_the_oracle():
    """Small mesh, limiter off: the GPU adjoint against central differences
    of the CPU oracle forward (which is pinned to the reference)."""
    mesh, cells, target = problem(20, 16)
    steps, eps = 10, 1e-6
    rng = np.random.default_rng(7)
    with handle(mesh, slope_limiter=0) as h:
        dt = cfl_dt(h, cells)
        wn = fwd(h, cells, steps, dt, every=4)
        exact(wn, oracle.run_fixed_dt(mesh, cells, GAMMA, steps, dt, smooth_lp())[0])
        g = h.step_bwd(loss_seed(wn, target))
    for _ in range(6):
        d = rng.normal(size=cells.shape)
        lp = loss(oracle.run_fixed_dt(mesh, cells + eps * d, GAMMA, steps, dt, smooth_lp())[0], target)
        lm = loss(oracle.run_fixed_dt(mesh, cells - eps * d, GAMMA, steps, dt, smooth_lp())[0], target)
        fd = (lp - lm) / (2 * eps)
        ad = float(np.sum(g * d))
        assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)


def test_limited_adjoint_vs_oracle_differences_away_from_switches():
    """Limiter on.  LinearGaussImproved's limiter switches discontinuously
    (the 5%/10%-of-range threshold, the sign test, the 1e-9 relative
    deadband), so a finite difference that steps over a switch measures
    the jump, not a derivative; between switches the map is smooth but
    strongly curved (psi is a ratio of small differences).  From an evolved
    (non-uniform) state, a direction in which the central differences at
    eps = 1e-6 and 1e-7 agree to 1e-7 has no switch within eps; there the
    central difference must match the adjoint to 1e-6."""
    mesh, cells, target = problem(20, 16)
    steps = 3
    with handle(mesh) as h:
        dt = cfl_dt(h, cells)
        base, _ = oracle.run_fixed_dt(mesh, cells, GAMMA, 8, dt)
        wn = fwd(h, base, steps, dt, every=2)
        g = h.step_bwd(loss_seed(wn, target))
    rng = np.random.default_rng(3)

    def central(d, eps):
        lp = loss(oracle.run_fixed_dt(mesh, base + eps * d, GAMMA, steps, dt)[0], target)
        lm = loss(oracle.run_fixed_dt(mesh, base - eps * d, GAMMA, steps, dt)[0], target)
        return (lp - lm) / (2 * eps)

    checked = 0
    for _ in range(12):
        d = rng.normal(size=cells.shape)
        f6, f7 = central(d, 1e-6), central(d, 1e-7)
        if abs(f6 - f7) > 1e-7 * abs(f6):
            continue  # a limiter switch lies within eps
        checked += 1
        ad = float(np.sum(g * d))
        assert abs(f6 - ad) <= 1e-6 * abs(ad), (f6, ad)
    assert checked >= 6, checked


def test_adjoint_workload_256_central_differences():
    """The adjoint workload with the limiter off: 256x256 periodic bumps,
    200 steps at the initial CFL-0.3 dt, checkpoints every 20 steps, 32
    random directions, eps = 1e-6."""
    mesh, cells, target = problem(256, 256)
    steps, eps = 200, 1e-6
    rng = np.random.default_rng(2024)
    errs = []
    with handle(mesh, slope_limiter=0) as h:
        dt = cfl_dt(h, cells)
        wn = fwd(h, cells, steps, dt, 20)
        g = h.step_bwd(loss_seed(wn, target))
        for _ in range(32):
            d = rng.normal(size=cells.shape)
            lp = loss(fwd(h, cells + eps * d, steps, dt), target)
            lm = loss(fwd(h, cells - eps * d, steps, dt), target)
            fd = (lp - lm) / (2 * eps)
            ad = float(np.sum(g * d))
            errs.append(abs(fd - ad) / abs(ad))
    assert max(errs) <= 1e-6, sorted(errs)[-5:]


def test_adjoint_workload_256_limited_dot_product_and_differences():
    """The adjoint workload as specified (limiter on).  The dot-product test
    holds to round-off; the central differences also cross limiter
    switches over 200 steps of 65,536 cells, so they are held to the size
    those jumps give (measured: median about 4e-4, max about 2e-2)."""
    mesh, cells, target = problem(256, 256)
    steps, eps = 200, 1e-6
    rng = np.random.default_rng(99)
    with handle(mesh) as h:
        dt = cfl_dt(h, cells)
        wn = fwd(h, cells, steps, dt, 20)
        g = h.step_bwd(loss_seed(wn, target))
        dw = rng.normal(size=cells.shape)
        h.set_cells(cells)
        tl = h.step_tlm(steps, dt, dw)
        wbar = loss_seed(wn, target)
        lhs, rhs = float(np.sum(wbar * tl)), float(np.sum(g * dw))
        assert abs(lhs - rhs) <= 1e-11 * abs(lhs), (lhs, rhs)
        errs = []
        for _ in range(8):
            d = rng.normal(size=cells.shape)
            fd = (loss(fwd(h, cells + eps * d, steps, dt), target) -
                  loss(fwd(h, cells - eps * d, steps, dt), target)) / (2 * eps)
            ad = float(np.sum(g * d))
            errs.append(abs(fd - ad) / abs(ad))
    assert np.median(errs) <= 2e-3 and max(errs) <= 5e-2, errs


def test_torch_autograd_function():
    torch = pytest.importorskip("torch")
    mesh, cells, target = problem(64, 64)
    with handle(mesh, slope_limiter=0) as h:
        dt = cfl_dt(h, cells)

        class Evolve(torch.autograd.Function):
            @staticmethod
            def forward(ctx, w0):
                h.set_cells(w0.detach().numpy())
                h.step_fwd(20, dt, 5)
                return torch.from_numpy(h.get_cells())

            @staticmethod
            def backward(ctx, wbar):
                return torch.from_numpy(h.step_bwd(wbar.contiguous().numpy()))

        w0 = torch.tensor(cells, dtype=torch.float64, requires_grad=True)
        t = torch.tensor(target)
        wn = Evolve.apply(w0)
        L = ((wn[:, 0] - t) ** 2).sum()
        L.backward()
        g = w0.grad.numpy()
        exact(wn.detach().numpy(), oracle.run_fixed_dt(mesh, cells, GAMMA, 20, dt, smooth_lp())[0])
        assert np.array_equal(g, h.step_bwd(loss_seed(wn.detach().numpy(), target)))
        eps = 1e-6
        d = np.random.default_rng(5).normal(size=cells.shape)
        fd = (loss(fwd(h, cells + eps * d, 20, dt), target) - loss(fwd(h, cells - eps * d, 20, dt), target)) / (2 * eps)
    ad = float(np.sum(g * d))
    assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)


def test_unsupported_configurations_are_rejected():
    mesh, cells, _ = problem(32, 32)
    wall = synthetic.lattice_mesh(32, 32, (0.0, 1.0, 0.0, 1.0), "rigid", seed=3)
    for kw, m in [(dict(ghost_kind=0), wall), (dict(ghost_kind=1, order=1), mesh),
                  (dict(ghost_kind=1, time_integrator=1), mesh)]:
        kw.setdefault("order", 2)
        with richgpu.Handle(gamma=GAMMA, device=0, **kw) as h:
            h.upload_mesh(m)
            h.set_cells(cells if m is mesh else synthetic.bumps_cells(m))
            with pytest.raises(richgpu.RichError) as ei:
                h.step_fwd(3, 1e-4, 2)
            assert ei.value.status == 1
    with handle(mesh) as h:
        h.set_cells(cells)
        with pytest.raises(richgpu.RichError) as ei:
            h.step_bwd(np.zeros_like(cells))
        assert ei.value.status == 3
        with pytest.raises(richgpu.RichError):
            h.step_fwd(0, 1e-4, 2)
    with handle(mesh, precision=1) as h:            # the tangent-linear model is FP64 only
        h.set_cells(cells)
        with pytest.raises(richgpu.RichError):
            h.step_tlm(3, 1e-4, np.zeros_like(cells))


# ---------------------------------------------------------------- FP32-mixed adjoint

def mixed_and_fp64_gradients(nx, steps, every, seed=3, slf=1):
    mesh, cells, target = problem(nx, nx, seed)
    out = {}
    with handle(mesh, slope_limiter=slf) as h:
        dt = cfl_dt(h, cells)
    for precision in (0, 1):
        with handle(mesh, precision=precision, slope_limiter=slf) as h:
            wn = fwd(h, cells, steps, dt, every)
            out[precision] = (wn, h.step_bwd(loss_seed(wn, target)))
    return mesh, cells, target, dt, out


def test_mixed_adjoint_equals_the_fp64_gradient_on_the_smooth_map():
    """Limiter off (the map is smooth): the FP32-mixed adjoint (FP32
    reconstruction and Hllc reverse, FP64 gathers and cell update, along the
    FP32-mixed trajectory) against the FP64 adjoint: 128^2, 40 steps,
    checkpoints every 10.  Measured 1.2e-6 relative."""
    _, _, _, _, out = mixed_and_fp64_gradients(128, 40, 10, slf=0)
    (_, g64), (_, g32) = out[0], out[1]
    rel = np.linalg.norm(g32 - g64) / np.linalg.norm(g64)
    assert rel < 1e-5, rel


def test_mixed_adjoint_tracks_the_fp64_gradient():
    """Limiter on: the FP32-mixed map is the derivative of FP32 limiter
    decisions.  Where FP32 rounding flips a limiter branch the two maps'
    derivatives differ by construction: the initial pressure is uniform,
    its FP32 naive slope is rounding noise the limiter cuts to zero while
    the FP64 one passes, so the pressure component of the gradient differs
    most.  Measured: 1.3e-3 relative overall, 1 - cos 8e-7."""
    _, _, _, _, out = mixed_and_fp64_gradients(128, 40, 10)
    (w64, g64), (w32, g32) = out[0], out[1]
    l1 = np.abs(w32[:, 0] - w64[:, 0]).sum() / np.abs(w64[:, 0]).sum()
    assert l1 < 1e-5, l1
    rel = np.linalg.norm(g32 - g64) / np.linalg.norm(g64)
    cos = float((g32 * g64).sum() / (np.linalg.norm(g32) * np.linalg.norm(g64)))
    rel_d = np.linalg.norm(g32[:, 0] - g64[:, 0]) / np.linalg.norm(g64[:, 0])
    assert rel < 5e-3 and cos > 1 - 1e-5 and rel_d < 1e-3, (rel, cos, rel_d)


def test_mixed_adjoint_directional_derivatives_vs_fp64_tangent():
    """Smooth map (limiter off): <dL/dW0 (FP32-mixed adjoint), v> against the
    FP64 tangent-linear directional derivative for random directions v."""
    mesh, cells, target, dt, out = mixed_and_fp64_gradients(96, 30, 10, seed=5, slf=0)
    w64, _ = out[0]
    _, g32 = out[1]
    rng = np.random.default_rng(2)
    with handle(mesh, slope_limiter=0) as h:
        for _ in range(4):
            v = rng.normal(size=cells.shape) * np.abs(cells).mean(axis=0)
            h.set_cells(cells)
            dwn = h.step_tlm(30, dt, v)
            tl = float((loss_seed(w64, target) * dwn).sum())
            ad = float((g32 * v).sum())
            assert abs(ad - tl) <= 1e-4 * abs(tl), (ad, tl)  # measured up to 1.1e-5


def test_mixed_adjoint_is_deterministic_and_keeps_the_state():
    mesh, cells, target = problem(64, 64)
    with handle(mesh, precision=1) as h:
        dt = cfl_dt(h, cells)
        wn = fwd(h, cells, 12, dt, 5)
        g1 = h.step_bwd(loss_seed(wn, target))
        g2 = h.step_bwd(loss_seed(wn, target))
        exact(g1, g2)
        exact(h.get_cells(), wn)
