"""Pins the oracle's tracer and sticker handling to the reference itself.

Fixtures in tests/golden/tracers/ come from oracle/ref/ref_dump.cpp's
<case>_tracers forms (tests/golden/make_golden.py): tracers named
{"A", "Entropy", "Z"} (sorted, as hdsim sorts them), "A" in
LinearGaussImproved's calc_tracers, "Entropy" recomputed by SimpleCellUpdater;
stickers {"frozen", "skip"}: HasSticker("frozen") + SkipUpdate in the cell
updater's sequence and "skip" as LinearGaussImproved's skip_key.  Every
comparison is exact.
"""
import glob
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, load_golden
from test_oracle_golden import accumulate, exact

TRACER_CASES = sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, "tracers", "*.npz")))


def load_tracers(name):
    g = load_golden(os.path.join("tracers", name))
    g["ts"] = oracle.TracerSetup(3, limited=0b001, entropy=1, skip_sticker=1, frozen_sticker=0,
                                 stickers=g["tr_stickers"])
    return g


@pytest.fixture(params=TRACER_CASES)
def tg(request):
    return load_tracers(request.param)


def lp_of(g):
    return oracle.lgi_params(ghost_kind=g["ghost_kind"])


def test_case_uses_every_feature(tg):
    st = tg["tr_stickers"]
    assert np.any(st & 1) and np.any(st & 2)


def test_init_extensives(tg):
    if int(tg["case_params"][2]) != 0:
        pytest.skip("state is not the initial one")
    exact(oracle.init_extensives_tr(tg["mesh"], tg["cells0"], tg["tr_cells0"]), tg["tr_ext0"])


def test_lgi_slopes_and_interp(tg):
    g = tg
    if g["order"] != 2:
        pytest.skip("first-order case")
    slopes, interp, tsl, tip = oracle.lgi_tr(g["mesh"], g["cells0"], g["tr_cells0"], g["gamma"], lp_of(g), g["ts"])
    exact(slopes, g["slopes"])
    exact(interp, g["interp"])
    exact(tsl, g["tr_slopes"])
    exact(tip, g["tr_interp"])


def test_fluxes(tg):
    g = tg
    fl, tfl = oracle.flux_tr(g["mesh"], g["cells0"], g["tr_cells0"], g["ev_flux"], g["gamma"], g["order"],
                             lp_of(g), g["ts"])
    exact(fl, g["fluxes"])
    exact(tfl, g["tr_fluxes"])


def test_extensive_and_cell_update(tg):
    g = tg
    exact(oracle.extensive_update(g["mesh"], g["fluxes"], g["dt"], g["ext0"]), g["ext1"])
    exact(oracle.extensive_update_tr(g["mesh"], g["tr_fluxes"], g["dt"], g["tr_ext0"]), g["tr_ext1"])
    cells, tr, tr_ext = oracle.cell_update_tr(g["mesh"], g["ext1"], g["tr_ext1"], g["cells0"], g["tr_cells0"],
                                              g["gamma"], g["ts"])
    exact(cells, g["cells1"])
    exact(tr, g["tr_cells1"])
    exact(tr_ext, g["tr_ext1b"])


def test_frozen_cells_keep_their_state(tg):
    g = tg
    fr = (g["tr_stickers"] & 1) == 1
    exact(g["cells1"][fr], g["cells0"][fr])
    exact(g["tr_cells1"][fr], g["tr_cells0"][fr])


def test_hdsim_run(tg):
    g = tg
    if "run_cells" not in g:
        pytest.skip("no multi-step run in this case")
    steps = int(g["case_params"][3])
    ev = np.zeros((g["mesh"].n_faces, 2))
    cells, ext, tr, tr_ext, dts = oracle.run_tr(g["mesh"], g["cells0"], g["ext0"], g["tr_cells0"], g["tr_ext0"], ev,
                                                g["gamma"], steps, g["ts"], 0.3, g["order"], lp_of(g), heun=g["heun"])
    exact(accumulate(float(g["time0"][0]), dts), g["run_times"])
    exact(ext, g["run_ext"])
    exact(cells, g["run_cells"])
    exact(tr_ext, g["tr_run_ext"])
    exact(tr, g["tr_run_cells"])
