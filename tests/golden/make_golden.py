"""Regenerate the golden fixtures in this directory from the reference itself.

Builds the reference RICH hot path from its own sources (oracle/ref/Makefile,
outputs only under oracle/_ref/), runs oracle/ref/ref_dump.cpp on each case
and bundles the .npy arrays it writes into ``<case>.npz``.

Usage (needs the reference source tree; not available at test time):

    python tests/golden/make_golden.py [--ref /path/to/huji-rich] [case ...]

Each fixture holds the packed mesh (``mesh_*``), the state (``cells0``,
``ext0``), the edge velocities, and the reference's own outputs of one
hot-path pass (``dt``, ``fluxes``, ``slopes``/``interp`` for second order,
``ext1``, ``cells1``); cases with ``run > 0`` also hold the state after that
many ``hdsim::TimeAdvance`` steps (``run_cells``, ``run_ext``, ``run_dts``).
"""
import argparse
import glob
import os
import platform
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

# name: (ref_dump case, nx, ny, warm steps, run steps[, "heun"])
CASES = {
    # 2D Sod, first order, Eulerian: one pass + 20 hdsim steps
    "sod_o1": ("sod", 50, 10, 0, 20),
    # the full 200x40 Sod tube of the first benchmark configuration, 200 steps
    "sod_full_o1": ("sod", 200, 40, 0, 200),
    # first order with moving (Lagrangian) faces after 3 steps
    "sod_lagrangian_o1": ("sod_lagrangian", 50, 10, 3, 0),
    # Sedov, LinearGaussImproved + rigid walls, RoundCells motion, after 3 steps
    "sedov_o2": ("sedov", 24, 24, 3, 0),
    # Sedov on a fixed mesh: one pass + 10 hdsim steps
    "sedov_eulerian_o2": ("sedov_eulerian", 24, 24, 2, 10),
    # periodic box, LinearGaussImproved + periodic ghosts, Eulerian: one pass + 10 steps
    "periodic_o2": ("periodic", 16, 16, 2, 10),
    # periodic box with Lagrangian faces after 2 steps
    "periodic_lagrangian_o2": ("periodic_lagrangian", 16, 16, 2, 0),
    # hdsim::TimeAdvance2Heun on fixed meshes
    "sod_heun_o1": ("sod", 50, 10, 0, 20, "heun"),
    "sedov_eulerian_heun_o2": ("sedov_eulerian", 24, 24, 2, 10, "heun"),
    "periodic_heun_o2": ("periodic", 16, 16, 2, 10, "heun"),
    # RoundCells(Lagrangian, cold) with the box as its outer boundary, flow
    # into the walls: ApplyFix's calc_dw(dt) and CorrectPointsOverShoot act
    "wallflow_cold_o2": ("wallflow_cold", 24, 24, 2, 0),
    # CylindricalSymmetry (axis x = 0) face areas and cell volumes: one pass + 10 steps
    "cyl_blast_o2": ("cyl_blast", 24, 24, 2, 10),
    # condition/action flux schemes: free-flow walls (first order), rigid
    # walls and a rigid obstacle of "obstacle"-sticker cells, outflow ratchets
    "cas_free_o1": ("cas_free", 24, 24, 2, 10),
    "cas2_wall_o2": ("cas2_wall", 24, 24, 2, 10),
    "cas2_ratchet_o2": ("cas2_ratchet", 24, 24, 2, 10),
    # LagrangianFlux (LagrangianHLLC pair, WallsMassFlux) + LagrangianExtensiveUpdater:
    # Eulerian with 10 hdsim steps, and one pass on Lagrangian-moving faces
    "cas2_lag_o2": ("cas2_lag", 24, 24, 2, 10),
    "cas2_lag_move_o2": ("cas2_lag_move", 24, 24, 2, 0),
}

# Tracers and stickers (ref_dump's <case>_tracers forms), written to
# tracers/<name>.npz: tracers {"A" (in calc_tracers), "Entropy", "Z"},
# stickers {"frozen" (HasSticker + SkipUpdate), "skip" (LinearGaussImproved's
# skip_key)}; name: (ref_dump case, nx, ny, warm steps, run steps)
CASES_TRACERS = {
    "sod_tracers_o1": ("sod_tracers", 50, 10, 0, 20),
    "sedov_eulerian_tracers_o2": ("sedov_eulerian_tracers", 24, 24, 2, 10),
    "periodic_tracers_o2": ("periodic_tracers", 16, 16, 2, 10),
    # RoundCells motion after 3 steps: one pass with moving faces
    "sedov_tracers_o2": ("sedov_tracers", 24, 24, 3, 0),
    # TimeAdvance2Heun with tracers, stickers (frozen cells) and the entropy tracer
    "sedov_eulerian_heun_tracers_o2": ("sedov_eulerian_tracers", 24, 24, 2, 10, "heun"),
    "periodic_heun_tracers_o2": ("periodic_tracers", 16, 16, 2, 10, "heun"),
}

# The condition/action cases with tracers (ref_dump's cas*_tracers forms),
# written to cas_tracers/<name>.npz: tracers {"A" (in calc_tracers), "Z"},
# the cases' own stickers; name: (ref_dump case, nx, ny, warm steps, run steps)
CASES_CAS_TRACERS = {
    "cas_free_tracers_o1": ("cas_free_tracers", 24, 24, 2, 10),
    "cas2_wall_tracers_o2": ("cas2_wall_tracers", 24, 24, 2, 10),
    "cas2_ratchet_tracers_o2": ("cas2_ratchet_tracers", 24, 24, 2, 10),
    "cas2_lag_tracers_o2": ("cas2_lag_tracers", 24, 24, 2, 10),
}

# 3D first-order path (oracle/ref/ref_dump3d.cpp), written to 3d/<name>.npz:
# name: (ref_dump3d case, nx, ny, nz, run steps)
CASES3D = {
    # seeded density, pressure and velocity per cell: every HLLC branch, tangential flow
    "cube_random": ("random", 6, 5, 4, 8),
    # a Sod tube along x at rest
    "cube_sod": ("sod", 24, 4, 3, 30),
    # uniform gas with a sheared velocity field
    "cube_shear": ("shear", 8, 8, 6, 15),
}


# The tessellator of the test and benchmark meshes (synthetic.lattice_mesh)
# pinned to the reference's VoronoiMesh of the same points, written to
# mesh/<name>.npz: name: (nx, ny, box, boundary, seed)
MESH_PINS = {
    "lattice64_rigid": (64, 64, (-1.0, 1.0, -1.0, 1.0), "rigid", 2),
    "lattice64_periodic": (64, 64, (0.0, 1.0, 0.0, 1.0), "periodic", 3),
    "lattice48x16_rigid": (48, 16, (0.0, 1.0, 0.0, 0.2), "rigid", 1),
}


def mesh_pins(exe, scratch, names):
    sys.path.insert(0, os.path.join(ROOT, "huji-rich_gb300"))
    import synthetic
    os.makedirs(os.path.join(HERE, "mesh"), exist_ok=True)
    for name in [c for c in (names or sorted(MESH_PINS)) if c in MESH_PINS]:
        nx, ny, box, boundary, seed = MESH_PINS[name]
        px, py = synthetic.jittered_points(nx, ny, *box, seed)
        with tempfile.TemporaryDirectory(dir=scratch) as d:
            np.stack([px.ravel(), py.ravel()], 1).astype("<f8").tofile(os.path.join(d, "points.f64"))
            np.array(box, dtype="<f8").tofile(os.path.join(d, "box.f64"))
            subprocess.check_call([exe, "mesh_" + boundary, d, str(nx), str(ny), "0", "0"])
            arrays = {os.path.basename(f)[:-4]: np.load(f) for f in glob.glob(os.path.join(d, "*.npy"))}
        arrays["case_params"] = np.array([nx, ny, seed], dtype=np.int64)
        arrays["box"] = np.array(box)
        out = os.path.join(HERE, "mesh", name + ".npz")
        np.savez_compressed(out, **arrays)
        print(f"{name}: {len(arrays)} arrays, {os.path.getsize(out) / 1024:.0f} KiB", file=sys.stderr)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("RICH_REFERENCE"),
                    help="reference source tree (default: oracle/ref/Makefile's REF)")
    ap.add_argument("cases", nargs="*")
    a = ap.parse_args()
    mk = ["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle", "ref")]
    subprocess.check_call(mk + ["stage"] + (["REF=" + a.ref] if a.ref else []))
    subprocess.check_call(mk + ["all"])
    scratch = os.path.join(ROOT, "oracle", "_ref", platform.machine())
    exe = os.path.join(scratch, "ref_dump")
    exe3 = os.path.join(scratch, "ref_dump3d")
    mesh_pins(exe, scratch, a.cases)
    os.makedirs(os.path.join(HERE, "3d"), exist_ok=True)
    for name in [c for c in (a.cases or sorted(CASES3D)) if c in CASES3D]:
        case, nx, ny, nz, run = CASES3D[name]
        with tempfile.TemporaryDirectory(dir=scratch) as d:
            subprocess.check_call([exe3, case, d, str(nx), str(ny), str(nz), str(run)])
            arrays = {os.path.basename(f)[:-4]: np.load(f) for f in glob.glob(os.path.join(d, "*.npy"))}
        arrays["case_params"] = np.array([nx, ny, nz, run], dtype=np.int64)
        out = os.path.join(HERE, "3d", name + ".npz")
        np.savez_compressed(out, **arrays)
        print(f"{name}: {len(arrays)} arrays, {os.path.getsize(out) / 1024:.0f} KiB", file=sys.stderr)
    os.makedirs(os.path.join(HERE, "tracers"), exist_ok=True)
    todo = [(c, CASES[c], HERE) for c in (a.cases or sorted(CASES)) if c in CASES]
    todo += [(c, CASES_TRACERS[c], os.path.join(HERE, "tracers"))
             for c in (a.cases or sorted(CASES_TRACERS)) if c in CASES_TRACERS]
    os.makedirs(os.path.join(HERE, "cas_tracers"), exist_ok=True)
    todo += [(c, CASES_CAS_TRACERS[c], os.path.join(HERE, "cas_tracers"))
             for c in (a.cases or sorted(CASES_CAS_TRACERS)) if c in CASES_CAS_TRACERS]
    for name, spec, outdir in todo:
        case, nx, ny, warm, run = spec[:5]
        scheme = spec[5] if len(spec) > 5 else "first"
        with tempfile.TemporaryDirectory(dir=scratch) as d:
            subprocess.check_call([exe, case, d, str(nx), str(ny), str(warm), str(run)] +
                                  (["heun"] if scheme == "heun" else []))
            arrays = {os.path.basename(f)[:-4]: np.load(f) for f in glob.glob(os.path.join(d, "*.npy"))}
        run_keys = [k for k in arrays if k.startswith("runmesh_")]
        if run_keys and all(np.array_equal(arrays[k], arrays["mesh_" + k[8:]]) for k in run_keys):
            # hdsim rebuilt an identical tessellation every step (Eulerian):
            # the run continued on mesh_* itself
            for k in run_keys:
                del arrays[k]
            arrays["run_mesh_unchanged"] = np.array(1)
        arrays["case_params"] = np.array([nx, ny, warm, run], dtype=np.int64)
        arrays["time_integrator"] = np.array(1 if scheme == "heun" else 0)
        out = os.path.join(outdir, name + ".npz")
        np.savez_compressed(out, **arrays)
        print(f"{name}: {len(arrays)} arrays, {os.path.getsize(out) / 1024:.0f} KiB", file=sys.stderr)


if __name__ == "__main__":
    main()
