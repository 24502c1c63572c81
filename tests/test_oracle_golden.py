"""Pins the C restatement (oracle/rich_oracle.c) to the reference itself.

The fixtures in tests/golden/ were written by the reference RICH sources
(oracle/ref/ref_dump.cpp, generated by tests/golden/make_golden.py).  Every
comparison is exact: the oracle repeats the reference's operations in the
reference's order, so any difference is a restatement bug.
"""
import numpy as np
import pytest

import oracle


def exact(a, b):
    """Bit-for-bit equality up to the sign of zero (IEEE ==), NaN-free."""
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape
    assert np.all(np.isfinite(a)) and np.all(np.isfinite(b))
    bad = np.argwhere(a != b)
    assert bad.size == 0, f"{len(bad)} mismatches, first at {bad[0]}: {a[tuple(bad[0])]!r} vs {b[tuple(bad[0])]!r}"


def accumulate(t0, dts):
    """hdsim's time_ += dt sequence (hdsim2d.cpp:238)."""
    out = []
    t = t0
    for dt in dts:
        t = t + dt
        out.append(t)
    return np.array(out)


def lp_of(g):
    return oracle.lgi_params(ghost_kind=g["ghost_kind"])


def test_cfl(golden):
    g = golden
    dt = oracle.cfl(g["mesh"], g["cells0"], g["ev_cfl"], g["gamma"], 0.3)
    assert dt == g["dt"]


def flux_rules(g):
    """The case's condition/action flux rules, or None (Simple/ModularFluxCalculator)."""
    return g.get("flux_rules")


def stickers_of(g):
    return g["tr_stickers"].astype(np.uint32) if "tr_stickers" in g else None


def lagrangian(g):
    """LagrangianExtensiveUpdater around SimpleExtensiveUpdater (its
    LagrangianFlux's ws_ / edge_vel_ are in lag_ws / lag_ev)."""
    return "lagrangian_updater" in g


def test_fluxes(golden):
    g = golden
    if flux_rules(g) is not None:
        f = oracle.cas_flux(g["mesh"], g["cells0"], g["ev_flux"], g["gamma"], g["order"], lp_of(g), flux_rules(g),
                            stickers_of(g))
    elif g["order"] == 1:
        f = oracle.simple_flux(g["mesh"], g["cells0"], g["ev_flux"], g["gamma"])
    else:
        f = oracle.modular_flux(g["mesh"], g["cells0"], g["ev_flux"], g["gamma"], lp_of(g))
    exact(f, g["fluxes"])


def test_lgi_slopes_and_interp(golden):
    g = golden
    if g["order"] != 2:
        pytest.skip("first-order case")
    slopes, interp = oracle.lgi(g["mesh"], g["cells0"], g["gamma"], lp_of(g))
    exact(slopes, g["slopes"])
    exact(interp, g["interp"])


def cylindrical(g):
    return int(g["geometry"][0]) == 1


def areas_of(g):
    """CacheData face areas: None for SlabSymmetry (the edge lengths the
    oracle computes), CylindricalSymmetry's otherwise."""
    if not cylindrical(g):
        return None
    return oracle.cyl_geometry(g["mesh"], g["geometry"][1:3], g["geometry"][3:5])[0]


def test_extensive_update(golden):
    g = golden
    if cylindrical(g):
        ext1 = oracle.extensive_update_areas(g["mesh"], g["fluxes"], areas_of(g), g["dt"], g["ext0"])
    else:
        ext1 = oracle.extensive_update(g["mesh"], g["fluxes"], g["dt"], g["ext0"])
    if lagrangian(g):
        ext1 = oracle.lagrangian_update(g["mesh"], g["lag_ws"], g["lag_ev"], g["dt"], ext1)
    exact(ext1, g["ext1"])


def test_lagrangian_flux_ws_and_face_speeds(golden):
    """LagrangianFlux's per-face outputs: LagrangianHLLC's transferred energy
    (the contact speed for massflux = false) where WallsMassFlux holds, 0
    elsewhere, and every face's speed along its normal."""
    g = golden
    if not lagrangian(g):
        pytest.skip("no LagrangianFlux in this case")
    _, ws, lev = oracle.cas_flux(g["mesh"], g["cells0"], g["ev_flux"], g["gamma"], g["order"], lp_of(g),
                                 flux_rules(g), stickers_of(g), lagrangian=True)
    exact(ws, g["lag_ws"])
    exact(lev, g["lag_ev"])


def test_cell_update(golden):
    g = golden
    if flux_rules(g) is not None and stickers_of(g) is not None:
        # obstacle cells keep their state (HasSticker + SkipUpdate)
        ts = oracle.TracerSetup(0, frozen_sticker=0, stickers=stickers_of(g))
        cells, _, _ = oracle.cell_update_tr(g["mesh"], g["ext1"], np.zeros((g["mesh"].n_cells, 0)), g["cells0"],
                                            np.zeros((g["mesh"].n_cells, 0)), g["gamma"], ts)
        exact(cells, g["cells1"])
        return
    exact(oracle.cell_update(g["mesh"], g["ext1"], g["gamma"]), g["cells1"])


def test_hdsim_run(golden):
    """N hdsim::TimeAdvance (or TimeAdvance2Heun) steps on a mesh that hdsim
    rebuilt unchanged."""
    g = golden
    if "run_cells" not in g:
        pytest.skip("no multi-step run in this case")
    assert "run_mesh_unchanged" in g
    steps = int(g["case_params"][3])
    ev = np.zeros((g["mesh"].n_faces, 2))
    if flux_rules(g) is not None:
        st = stickers_of(g)
        cells, ext, dts = oracle.run_cas(g["mesh"], g["cells0"], g["ext0"], ev, g["gamma"], steps, g["order"],
                                         lp_of(g), flux_rules(g), st, 1 if st is not None else 0,
                                         lagrangian_update=lagrangian(g))
    else:
        cells, ext, dts = oracle.run(g["mesh"], g["cells0"], g["ext0"], ev, g["gamma"], steps,
                                     0.3, g["order"], lp_of(g), heun=g["heun"], areas=areas_of(g))
    exact(accumulate(float(g["time0"][0]), dts), g["run_times"])
    exact(ext, g["run_ext"])
    exact(cells, g["run_cells"])


def test_init_extensives(golden):
    """hdsim's init_extensives on the initial state (cases that start at step 0)."""
    g = golden
    if int(g["case_params"][2]) != 0:
        pytest.skip("state is not the initial one")
    exact(oracle.init_extensives(g["mesh"], g["cells0"], g["gamma"]), g["ext0"])


def oracle_pass(g, cells, ext, ev, steps=1, heun=None):
    """hdsim::TimeAdvance (TimeAdvance2Heun with heun) steps of the case's own
    plugins on the fixture mesh; heun=None takes the fixture's."""
    heun = g["heun"] if heun is None else heun
    if flux_rules(g) is not None:
        st = stickers_of(g)
        return oracle.run_cas(g["mesh"], cells, ext, ev, g["gamma"], steps, g["order"], lp_of(g), flux_rules(g), st,
                              1 if st is not None else 0, lagrangian_update=lagrangian(g))
    return oracle.run(g["mesh"], cells, ext, ev, g["gamma"], steps, 0.3, g["order"], lp_of(g), heun=heun,
                      areas=areas_of(g))


def motion_of(g):
    """The case's PointMotion / EdgeVelocityCalculator as recorded by the dump."""
    k, edges, chi, eta, cold, fix = g["motion"]
    return oracle.motion(k, edges, chi, eta, cold, fix, tuple(g["outer_box"]))


def test_cell_geometry(golden):
    """Tessellation::GetVolume, CalcCellCM (with the ghosts' reflected or
    shifted CMs) and the PhysicalGeometry's CacheData volumes and areas
    (SlabSymmetry, CylindricalSymmetry) from points and face vertices."""
    g = golden
    m = g["mesh"]
    vol, cm, cdv = oracle.cell_geometry(m, g["ghost_kind"], g["outer_box"])
    exact(vol, m.volume)
    exact(cm, m.cm_xy)
    if cylindrical(g):
        areas, cdv = oracle.cyl_geometry(m, g["geometry"][1:3], g["geometry"][3:5])
        exact(areas, g["mesh_cd_area"])
    else:
        # SlabSymmetry::calcArea = |first - second| (physical_geometry.cpp:8-11)
        d = m.face_vertices[:, 0:2] - m.face_vertices[:, 2:4]
        exact(np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]), g["mesh_cd_area"])
    exact(cdv, m.cd_volume)


def test_point_motion_and_edge_velocities(golden):
    """PointMotion (Eulerian, Lagrangian, RoundCells hot and cold with
    CorrectPointsOverShoot), ApplyFix and the edge velocities both times
    hdsim::TimeAdvance computes them."""
    g = golden
    mo = motion_of(g)
    pv = oracle.point_velocities(g["mesh"], g["cells0"], g["gamma"], mo)
    exact(pv, g["pv_cfl"])
    exact(oracle.edge_velocities(g["mesh"], mo, pv), g["ev_cfl"])
    pv = oracle.apply_fix(g["mesh"], g["cells0"], g["gamma"], mo, g["dt"], pv)
    exact(pv, g["pv_flux"])
    exact(oracle.edge_velocities(g["mesh"], mo, pv), g["ev_flux"])
