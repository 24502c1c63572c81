"""The committed fixtures are what the reference writes: regenerating every
2D fixture (base, tracer and condition/action tracer cases) with the reference
build (oracle/_ref/<arch>/ref_dump, made by build() from the staged
reference sources) reproduces every array bit for bit.  The recipe is
tests/golden/make_golden.py's; scratch files go under oracle/_ref.  Skipped
where the reference build is absent."""
import glob
import os
import platform
import subprocess
import sys
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SCRATCH = os.path.join(ROOT, "oracle", "_ref", platform.machine())
REF_DUMP = os.path.join(SCRATCH, "ref_dump")
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, GOLDEN)
import make_golden  # noqa: E402

pytestmark = pytest.mark.skipif(not os.path.exists(REF_DUMP), reason="ref_dump not built here")

ADDED = {"case_params", "time_integrator", "run_mesh_unchanged"}  # written by make_golden itself


def regenerate(case, nx, ny, warm, run, heun=False):
    with tempfile.TemporaryDirectory(dir=SCRATCH) as d:
        subprocess.run([REF_DUMP, case, d, str(nx), str(ny), str(warm), str(run)] + (["heun"] if heun else []),
                       check=True, capture_output=True, timeout=600)
        return {os.path.basename(f)[:-4]: np.load(f) for f in glob.glob(os.path.join(d, "*.npy"))}


CASES = [(n, s, "cas_tracers") for n, s in sorted(make_golden.CASES_CAS_TRACERS.items())]
CASES += [(n, s, "tracers") for n, s in sorted(make_golden.CASES_TRACERS.items())]
CASES += [(n, s, "") for n, s in sorted(make_golden.CASES.items())]


@pytest.mark.parametrize("name,spec,sub", CASES, ids=[c[0] for c in CASES])
def test_fixture_regenerates_bitwise(name, spec, sub):
    case, nx, ny, warm, run = spec[:5]
    heun = len(spec) > 5 and spec[5] == "heun"
    got = regenerate(case, nx, ny, warm, run, heun)
    want = np.load(os.path.join(GOLDEN, sub, name + ".npz"))
    keys = set(want.files) - ADDED
    if "run_mesh_unchanged" in want.files:
        got = {k: v for k, v in got.items() if not k.startswith("runmesh_")}
    assert keys == set(got), sorted(keys ^ set(got))
    for k in sorted(keys):
        a, b = got[k], want[k]
        assert a.shape == b.shape and a.dtype == b.dtype, k
        assert a.tobytes() == b.tobytes(), k


REF_DUMP3D = os.path.join(SCRATCH, "ref_dump3d")


@pytest.mark.skipif(not os.path.exists(REF_DUMP3D), reason="ref_dump3d not built here")
@pytest.mark.parametrize("name", sorted(make_golden.CASES3D))
def test_3d_fixture_regenerates_bitwise(name):
    case, nx, ny, nz, run = make_golden.CASES3D[name]
    with tempfile.TemporaryDirectory(dir=SCRATCH) as d:
        subprocess.run([REF_DUMP3D, case, d, str(nx), str(ny), str(nz), str(run)], check=True, capture_output=True,
                       timeout=600)
        got = {os.path.basename(f)[:-4]: np.load(f) for f in glob.glob(os.path.join(d, "*.npy"))}
    want = np.load(os.path.join(GOLDEN, "3d", name + ".npz"))
    keys = set(want.files) - ADDED
    assert keys == set(got), sorted(keys ^ set(got))
    for k in sorted(keys):
        assert got[k].tobytes() == want[k].tobytes() and got[k].shape == want[k].shape, k


@pytest.mark.parametrize("name", sorted(make_golden.MESH_PINS))
def test_mesh_pin_regenerates_bitwise(name):
    """The reference's VoronoiMesh of synthetic.lattice_mesh's points, packed
    by ref_dump, as tests/golden/mesh/ holds it."""
    sys.path.insert(0, os.path.join(ROOT, "huji-rich_gb300"))
    import synthetic
    nx, ny, box, boundary, seed = make_golden.MESH_PINS[name]
    px, py = synthetic.jittered_points(nx, ny, *box, seed)
    with tempfile.TemporaryDirectory(dir=SCRATCH) as d:
        np.stack([px.ravel(), py.ravel()], 1).astype("<f8").tofile(os.path.join(d, "points.f64"))
        np.array(box, dtype="<f8").tofile(os.path.join(d, "box.f64"))
        subprocess.run([REF_DUMP, "mesh_" + boundary, d, str(nx), str(ny), "0", "0"], check=True,
                       capture_output=True, timeout=600)
        got = {os.path.basename(f)[:-4]: np.load(f) for f in glob.glob(os.path.join(d, "*.npy"))}
    want = np.load(os.path.join(GOLDEN, "mesh", name + ".npz"))
    keys = set(want.files) - {"case_params", "box"}
    assert keys == set(got), sorted(keys ^ set(got))
    for k in sorted(keys):
        assert got[k].tobytes() == want[k].tobytes() and got[k].shape == want[k].shape, k
