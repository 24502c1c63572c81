"""The condition/action tracer fixtures (tests/golden/cas_tracers/, written by
the reference through oracle/ref/ref_dump.cpp's cas*_tracers forms) hold
what the GPU tests read: the rule table, two tracers per cell, the sticker
masks, one pass of every plugin and a 10-step hdsim run, with tracer mass
moving across the faces."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden

CASES = sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, "cas_tracers", "*.npz")))
KEYS = ("flux_rules", "tr_stickers", "tr_cells0", "tr_ext0", "tr_fluxes", "tr_ext1", "tr_cells1", "tr_ext1b",
        "tr_run_ext", "tr_run_cells", "fluxes", "ext1", "cells1", "run_ext", "run_cells", "run_times")


def test_four_cases():
    assert CASES == ["cas2_lag_tracers_o2", "cas2_ratchet_tracers_o2", "cas2_wall_tracers_o2",
                     "cas_free_tracers_o1"]


@pytest.mark.parametrize("name", CASES)
def test_fixture_contents(name):
    g = load_golden(os.path.join("cas_tracers", name))
    n, e = g["mesh"].n_cells, g["mesh"].n_faces
    for k in KEYS:
        assert k in g, k
    assert g["tr_cells0"].shape == (n, 2) and g["tr_fluxes"].shape == (e, 2)
    assert g["flux_rules"].shape[1] == 6
    # tracer mass crosses a good share of the faces, and the run moves it
    assert np.count_nonzero(g["tr_fluxes"]) > e // 4
    assert not np.array_equal(g["tr_run_ext"], g["tr_ext0"])
    # tracer "A" (index 0) is LinearGaussImproved's calc_tracers entry: the
    # second-order cases carry its slopes, "Z" (index 1) gets none
    if g["order"] == 2:
        s = g["tr_slopes"]                      # {x_A, x_Z, y_A, y_Z} per cell
        assert s.shape == (n, 4)
        assert np.count_nonzero(s[:, [0, 2]]) > n // 2 and not np.any(s[:, [1, 3]])
    # Lagrangian case: LagrangianExtensiveUpdater's per-face data
    assert ("lag_ws" in g) == (name == "cas2_lag_tracers_o2")
