"""Pins the oracle's condition/action flux calculators with tracers
(ro_cas_flux_tr, ro_step_cas_tr in oracle/rich_oracle.c) to the reference
itself: the fixtures in tests/golden/cas_tracers/ (oracle/ref/ref_dump.cpp's
cas*_tracers forms: ConditionActionSequence with free-flow walls,
ConditionActionSequence2 with rigid walls and an obstacle, its Ratchet, and
LagrangianFlux with LagrangianExtensiveUpdater; tracers {"A" in
calc_tracers, "Z"}).  Every comparison is exact."""
import os

import numpy as np
import pytest

import oracle
from conftest import load_golden
from test_cpu_cas_tracer_fixtures import CASES
from test_oracle_golden import accumulate, exact


def case(name):
    g = load_golden(os.path.join("cas_tracers", name))
    obstacle = bool(np.any(g["tr_stickers"] & 1))
    g["ts"] = oracle.TracerSetup(2, limited=0b01, frozen_sticker=0 if obstacle else -1, stickers=g["tr_stickers"])
    g["lp"] = oracle.lgi_params(ghost_kind=g["ghost_kind"])
    g["lag"] = "lagrangian_updater" in g
    return g


@pytest.mark.parametrize("name", CASES)
def test_one_pass(name):
    g = case(name)
    m, ts = g["mesh"], g["ts"]
    fl, tfl, ws, lev = oracle.cas_flux_tr(m, g["cells0"], g["tr_cells0"], g["ev_flux"], g["gamma"], g["order"],
                                          g["lp"], g["flux_rules"], ts, lagrangian=True)
    exact(fl, g["fluxes"])
    exact(tfl, g["tr_fluxes"])
    if g["lag"]:
        exact(ws, g["lag_ws"])
        exact(lev, g["lag_ev"])
    if g["order"] == 2:
        exact(oracle.lgi_tr(m, g["cells0"], g["tr_cells0"], g["gamma"], g["lp"], ts)[2], g["tr_slopes"])
    ext1 = oracle.extensive_update(m, fl, g["dt"], g["ext0"])
    tr_ext1 = oracle.extensive_update_tr(m, tfl, g["dt"], g["tr_ext0"])
    if g["lag"]:
        ext1, tr_ext1 = oracle.lagrangian_update_tr(m, ws, lev, g["dt"], ext1, tr_ext1)
    exact(ext1, g["ext1"])
    exact(tr_ext1, g["tr_ext1"])
    cells1, tr1, tr_ext1b = oracle.cell_update_tr(m, ext1, tr_ext1, g["cells0"], g["tr_cells0"], g["gamma"], ts)
    exact(cells1, g["cells1"])
    exact(tr1, g["tr_cells1"])
    exact(tr_ext1b, g["tr_ext1b"])


@pytest.mark.parametrize("name", CASES)
def test_hdsim_run(name):
    g = case(name)
    steps = int(g["case_params"][3])
    cells, ext, tr, tr_ext, dts = oracle.run_cas_tr(g["mesh"], g["cells0"], g["ext0"], g["tr_cells0"], g["tr_ext0"],
                                                    np.zeros((g["mesh"].n_faces, 2)), g["gamma"], steps, g["order"],
                                                    g["lp"], g["flux_rules"], g["ts"], lagrangian_update=g["lag"])
    exact(accumulate(float(g["time0"][0]), dts), g["run_times"])
    exact(ext, g["run_ext"])
    exact(cells, g["run_cells"])
    exact(tr_ext, g["tr_run_ext"])
    exact(tr, g["tr_run_cells"])


@pytest.mark.parametrize("name", CASES)
def test_unit_tracers_carry_the_mass_flux(name):
    """Tracers that are 1 everywhere move the mass flux across every face,
    whichever side each action takes: exactly from cell values (first
    order); from LinearGaussImproved's face values to rounding (the naive
    slope of a constant is a sum of stencil vectors that cancels only to
    rounding)."""
    g = case(name)
    m = g["mesh"]
    ones = np.ones((m.n_cells, 2))
    fl, tfl = oracle.cas_flux_tr(m, g["cells0"], ones, g["ev_flux"], g["gamma"], g["order"], g["lp"],
                                 g["flux_rules"], g["ts"])
    for j in range(2):
        if g["order"] == 1:
            exact(tfl[:, j], fl[:, 0])
        else:
            np.testing.assert_allclose(tfl[:, j], fl[:, 0], rtol=1e-12, atol=1e-15 * np.abs(fl[:, 0]).max())
