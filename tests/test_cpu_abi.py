"""CPU checks of the C-ABI library: it loads and exports every entry point the
header declares; calls that need no GPU behave as documented."""
import ctypes as C
import os
import re
import subprocess

import pytest

import richgpu
from meshview import RgConfig

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "rich_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:rg_status|void|const char\*)\s+(rg3?_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(richgpu.LIB_PATH):
        import rg_build
        rg_build.build()
    return richgpu.load()


def test_header_matches_binding_list():
    assert declared_functions() == sorted(richgpu.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", richgpu.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\sT\s(rg3?_\w+)$", out, re.M))
    missing = set(declared_functions()) - exported
    assert not missing, missing
    for name in declared_functions():
        assert hasattr(lib, name)


def test_default_config_is_reference_defaults(lib):
    cfg = RgConfig()
    lib.rg_default_config(C.byref(cfg))
    assert cfg.gamma == 5.0 / 3.0 and cfg.cfl == 0.3 and cfg.order == 2
    assert (cfg.delta_v, cfg.theta, cfg.delta_p) == (0.2, 0.5, 0.7)  # LinearGaussImproved.hpp:31-40
    assert cfg.slope_limiter == 1 and cfg.precision == 0


def test_status_strings_are_reference_messages(lib):
    lib.rg_status_string.restype = C.c_char_p
    assert lib.rg_status_string(10) == b"Negative density"
    assert lib.rg_status_string(11) == b"Negative thermal energy"
    assert lib.rg_status_string(13) == b"Invalid wave speeds in hllc solver"
    assert lib.rg_status_string(14) == b"Singular matrix"


def test_invalid_config_rejected_without_gpu(lib):
    cfg = RgConfig()
    lib.rg_default_config(C.byref(cfg))
    cfg.order = 3
    h = C.c_void_p()
    assert lib.rg_create(C.byref(cfg), C.byref(h)) == 1  # RG_ERR_INVALID_ARGUMENT
    assert lib.rg_destroy(None) == 0
