#!/usr/bin/env python3
"""Benchmark of RICH's per-step hydro hot path on GB300.

Workload (the headline configuration): 2D Sedov-Taylor on [-1,1]^2, a
512x512 lattice of mesh points jittered by +-1e-3 of a cell (seeded), rigid
walls, LinearGaussImproved second-order reconstruction, Hllc, IdealGas
gamma=5/3, CFL 0.3, energy 1 deposited as pressure in r<0.02.  A step is one
pass of the hot path: SimpleCFL dt, LinearGaussImproved + Hllc face fluxes,
SimpleExtensiveUpdater gather, SimpleCellUpdater -- hdsim::TimeAdvance's
plugin work with the mesh held fixed (the Voronoi rebuild is host code and
out of scope).

value  the FP32-mixed form (reconstruction, HLLC and CFL in FP32; geometry,
       volumes, extensive accumulation and the internal energy in FP64), with
       its density L1 error against the plain FP64 path stated; the plain FP64
       path (bit-identical to the reference) is measured in the same run and
       reported under "fp64".  Device-resident inputs; each step timed with
       CUDA events on the library's stream, L2 flushed (256 MiB write) before
       every timed step.
e2e    the same steps through the C ABI with host buffers, as a moving-mesh
       caller drives it: upload of the packed tessellation and the face
       velocities, the step, download of cells and extensives; "link" times
       one pinned copy each way of the same byte counts, the floor of the
       step's copies.
e2e_hdsim  the same Sedov problem advanced by the reference's own hdsim
       (tests/hdsim_dropin.cpp, linked with the reference built by
       oracle/ref/Makefile) with the GPU plugins, RoundCells moving the points
       and the host rebuilding the Voronoi mesh every step, beside hdsim with
       the reference's own plugins: what a RICH user sees per step.
batch  the batched form (512 independent Riemann problems, one launch per
       phase, CUDA graph), FP32-mixed and FP64, with its own roofline.
--impl reference   the reference's own CPU implementation of the path
       (oracle/ref/ref_bench.cpp: SimpleCFL, ModularFluxCalculator(
       LinearGaussImproved, Hllc), SimpleExtensiveUpdater, SimpleCellUpdater
       on the same mesh points, initial state and RoundCells face velocities)
       on all host cores, one independent simulation per core; where the
       reference could not be built, the C restatement oracle/rich_oracle.c.

Multi-GPU: replicas only (one independent simulation per rank); value sums
the cells all ranks updated over the slowest rank's time.
"""
import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "huji-rich_gb300")
ORACLE_DIR = os.path.join(ROOT, "oracle")
for _p in (PKG, ORACLE_DIR):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "cell-updates/s on 1 GB300: FP32-mixed vs FP64 at stated L1 error; adjoint/fwd cost"
UNIT = "cell-updates/s"
NX = NY = 512
GAMMA = 5.0 / 3.0
SEED = 2
FLUSH_BYTES = 256 << 20
# the reference built for this machine by oracle/ref/Makefile (through build())
REF_BIN = os.path.join(ROOT, "oracle", "_ref", platform.machine())


def reference_mesh(nx, ny, box, boundary, seed):
    """The reference's own tessellation of the jittered lattice: VoronoiMesh
    of synthetic.jittered_points in input order, packed by rich_pack.hpp
    (oracle/ref/ref_dump.cpp, mesh_rigid / mesh_periodic), or None where the
    reference was not built."""
    exe = os.path.join(REF_BIN, "ref_dump")
    if not os.path.exists(exe):
        return None
    import synthetic
    from meshview import MESH_FIELDS, PackedMesh
    px, py = synthetic.jittered_points(nx, ny, *box, seed)
    with tempfile.TemporaryDirectory() as d:
        np.stack([px.ravel(), py.ravel()], 1).astype("<f8").tofile(os.path.join(d, "points.f64"))
        np.array(box, dtype="<f8").tofile(os.path.join(d, "box.f64"))
        r = subprocess.run([exe, "mesh_" + boundary, d, str(nx), str(ny), "0", "0"], capture_output=True, text=True)
        if r.returncode != 0:
            return None
        return PackedMesh(**{k: np.load(os.path.join(d, "mesh_" + k + ".npy")) for k in MESH_FIELDS})


_WORKLOAD = {}


def workload():
    """The Sedov workload's mesh and initial cells: the reference's own
    VoronoiMesh of the jittered lattice where the reference is built here,
    else the same mesh from synthetic.lattice_mesh (the same cells, faces and
    ghosts up to a renumbering, geometry equal to rounding:
    tests/test_cpu_mesh_pin.py)."""
    if "mesh" not in _WORKLOAD:
        import synthetic
        box = (-1.0, 1.0, -1.0, 1.0)
        mesh = reference_mesh(NX, NY, box, "rigid", SEED)
        _WORKLOAD["source"] = "reference VoronoiMesh (oracle/ref/ref_dump.cpp mesh_rigid, input order)"
        if mesh is None:
            mesh = synthetic.lattice_mesh(NX, NY, box, "rigid", seed=SEED)
            _WORKLOAD["source"] = "synthetic.lattice_mesh (the reference was not built here)"
        _WORKLOAD["mesh"] = mesh
    mesh = _WORKLOAD["mesh"]
    import synthetic
    return mesh, synthetic.sedov_cells(mesh, GAMMA)


def config_block(mesh):
    """The workload, the same for both arms (implementation notes are kept
    out of it: see impl_notes)."""
    return {"workload": f"sedov2d_{NX}x{NY}_lgi_hllc", "cells": mesh.n_cells,
            "faces": mesh.n_faces, "ghosts": mesh.n_ghosts, "order": 2,
            "reconstruction": "LinearGaussImproved(slf, delta_v=0.2, theta=0.5, delta_P=0.7)",
            "riemann": "Hllc", "eos": "IdealGas(5/3)", "cfl": 0.3,
            "mesh": f"Voronoi mesh of a {NX}x{NY} lattice jittered +-1e-3 cell (seed {SEED}), rigid walls",
            "initial": "rho 1, p 1e-6, energy 1 deposited as pressure in r < 0.02",
            "point_motion": "RoundCells(Lagrangian, chi 0.15, eta 0.02) + StationaryBox face velocities, formed "
                            "once before timing; every timed flux pass reads them",
            "step": "SimpleCFL dt, LinearGaussImproved + Hllc fluxes, SimpleExtensiveUpdater, SimpleCellUpdater "
                    "on a fixed mesh",
            "l2": "flushed before every timed step (256 MiB write)", "parallelism": "replicas"}


IMPL_NOTES = {
    "geometry": "volumes and CMs computed on the device from points and face vertices",
    "face_velocities": "RoundCells point velocities and StationaryBox face velocities computed on the device",
    "e2e_step": "upload points + topology + face vertices (pinned), RoundCells motion, face velocities, dt, "
                "ApplyFix, fluxes and extensive update on the device (rg_advance_begin, point velocities "
                "read back), cell update (rg_cell_update), cells and extensives read back "
                "(rg_get_state_async: the copy overlaps the next step's mesh upload; the host waits for "
                "it before the next step's computation)"}


# ------------------------------------------------------------------ clocks

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.count(",") >= 8]
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].strip() == "Active"})
        power = [float(r[3]) for r in rows if r[3].strip().replace(".", "").isdigit()]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max(power) if power else None}


# ------------------------------------------------------------------ roofline

def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel):
    """dram bytes per launch of `kernel` from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "roofline_traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        parts = line.split()
        if len(parts) >= 2 and parts[0] == kernel and not line.startswith("#"):
            return float(parts[1])
    return None


def algorithmic_bytes(mesh, precision=0):
    """Compulsory bytes per launch of each kernel of a step (order 2).
    Geometry-only terms the design precomputes per mesh upload and the
    intermediates (slopes, fluxes) are not algorithmic.  The FP32-mixed path
    keeps primitives in FP32 (16 instead of 32 bytes per cell)."""
    n, f = mesh.n_cells, mesh.n_faces
    m = int(mesh.cell_face_offset[-1])
    if precision == 1:
        return {"cfl": 28 * n + 4 * m + 16 * f, "slopes": 60 * n + 4 * m, "faces": 56 * f,
                "update": 92 * n + 8 * m}
    return {
        # cells in 32 + width 8 + CSR offset 4 per cell; face id 4 per CSR entry;
        # face velocity 16 per face
        "cfl": 44 * n + 4 * m + 16 * f,
        # cells in 32, CM 16, mesh point 16, volume 8, CSR offset 4 per cell;
        # neighbour id 4 per CSR entry
        "slopes": 76 * n + 4 * m,
        # face cell pair 8, vertex pair 32, face velocity 16 per face
        "faces": 56 * f,
        # extensive in 32 + out 32, cells out 32, cd volume 8, CSR offset 4 per
        # cell; face id + side 8 per CSR entry
        "update": 108 * n + 8 * m,
    }


# ------------------------------------------------------------------ CPU

def roundcells_face_velocities(mesh, cells):
    """RoundCells(Lagrangian, chi 0.15, eta 0.02) point velocities through
    StationaryBox, as the C restatement computes them (the GPU arm forms the
    same on the device)."""
    import oracle
    mo = oracle.motion(kind=2, edges=0, chi=0.15, eta=0.02, box=(-1.0, 1.0, -1.0, 1.0))
    pv = oracle.point_velocities(mesh, cells, GAMMA, mo)
    return oracle.edge_velocities(mesh, mo, pv)


def write_workload(mesh, cells, d):
    """The mesh points and initial cells the reference's own driver reads."""
    pts = os.path.join(d, "points.f64")
    cel = os.path.join(d, "cells.f64")
    np.ascontiguousarray(mesh.point_xy[:mesh.n_cells], dtype="<f8").tofile(pts)
    np.ascontiguousarray(cells, dtype="<f8").tofile(cel)
    return pts, cel


def ref_bench(mesh, cells, procs, warm, steps):
    """Runs `procs` copies of the reference's own hot path
    (oracle/ref/ref_bench.cpp), one simulation per process, at the same
    time; returns their JSON records, or None where it was not built."""
    exe = os.path.join(REF_BIN, "ref_bench")
    if not os.path.exists(exe):
        return None
    with tempfile.TemporaryDirectory() as d:
        pts, cel = write_workload(mesh, cells, d)
        ps = [subprocess.Popen([exe, pts, cel, str(NX), str(NY), str(warm), str(steps)],
                               stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
              for _ in range(procs)]
        out = [p.communicate() for p in ps]
    if any(p.returncode != 0 for p in ps):
        raise RuntimeError("ref_bench failed: " + out[0][1][-500:])
    return [json.loads(o[0].strip().splitlines()[-1]) for o in out]


def cpu_steps(mesh, cells, ext, budget_s=10.0, max_steps=60):
    import oracle
    ev = roundcells_face_velocities(mesh, cells)
    lp = oracle.lgi_params(0)
    c, e = cells, ext
    c, e, _ = oracle.step(mesh, c, e, ev, GAMMA, 0.3, 2, lp)  # warm
    t0 = time.perf_counter()
    k = 0
    while k < max_steps and (time.perf_counter() - t0 < budget_s or k < 3):
        c, e, _ = oracle.step(mesh, c, e, ev, GAMMA, 0.3, 2, lp)
        k += 1
    return k, time.perf_counter() - t0


def cpu_baseline_block(mesh, cells, ext):
    """One host core: the reference's own code where it was built, else the C
    restatement; a sample of about 5-10 s of the same workload."""
    n = mesh.n_cells
    res = ref_bench(mesh, cells, 1, 1, 10)
    if res is not None:
        r = res[0]
        return {"value": n * r["steps"] / r["seconds"], "unit": UNIT, "cores": 1, "kind": "reference",
                "sample": f"{r['steps']} steps (after 1 warm-up) of the same {NX}x{NY} workload (FP64), one "
                          "process: the reference's SimpleCFL, ModularFluxCalculator(LinearGaussImproved, Hllc), "
                          "SimpleExtensiveUpdater, SimpleCellUpdater (oracle/ref/ref_bench.cpp, g++ -O2)",
                "ms_per_step": r["ms_per_step"]}
    kc, tc = cpu_steps(mesh, cells, ext)
    return {"value": n * kc / tc, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{kc} steps of the same {NX}x{NY} workload (FP64), one thread, C restatement "
                      "oracle/rich_oracle.c (gcc -O2); the reference itself is serial"}


def _reference_worker(args):
    steps, warmup = args
    import oracle
    mesh, cells = workload()
    ext = oracle.init_extensives(mesh, cells, GAMMA)
    ev = roundcells_face_velocities(mesh, cells)
    lp = oracle.lgi_params(0)
    c, e = cells, ext
    for _ in range(warmup):
        c, e, _ = oracle.step(mesh, c, e, ev, GAMMA, 0.3, 2, lp)
    t0 = time.perf_counter()
    for _ in range(steps):
        c, e, _ = oracle.step(mesh, c, e, ev, GAMMA, 0.3, 2, lp)
    return time.perf_counter() - t0, mesh.n_cells


def run_reference(args, world, rank):
    """The reference arm: the reference's own CPU hot path on every host core
    (one simulation per core), on this arm's workload, steps and warm-up."""
    if rank != 0:
        return
    cores = min(os.cpu_count() or 1, 64)
    steps = max(1, min(args.steps, 30))
    warm = max(3, min(args.warmup, 10))
    mesh, cells = workload()
    res = ref_bench(mesh, cells, cores, warm, steps)
    if res is not None:
        t = max(r["seconds"] for r in res)
        kind = "reference"
        sample = (f"{cores} independent {NX}x{NY} simulations, one process per core, {warm} warm-up + {steps} "
                  "timed steps each: the reference's own SimpleCFL, ModularFluxCalculator(LinearGaussImproved, "
                  "Hllc), SimpleExtensiveUpdater and SimpleCellUpdater (oracle/ref/ref_bench.cpp, compiled from "
                  "the reference's sources with g++ -O2 on this machine), RoundCells face velocities")
    else:
        import multiprocessing as mp
        import oracle
        oracle.build()
        ctx = mp.get_context("spawn")
        with ctx.Pool(cores) as pool:
            out = pool.map(_reference_worker, [(steps, warm)] * cores)
        t = max(r[0] for r in out)
        kind = "port"
        sample = (f"{cores} independent {NX}x{NY} simulations, one per core, {warm} warm-up + {steps} timed steps "
                  "each (C restatement oracle/rich_oracle.c, gcc -O2; the reference could not be built here), "
                  "RoundCells face velocities")
    n = mesh.n_cells
    value = cores * n * steps / t
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": steps, "warmup": warm, "ms_per_step": 1e3 * t / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_block(mesh),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU

KERNELS = ["cfl", "slopes", "faces", "update"]
KERNEL_NAMES = {0: {"cfl": "k_cfl", "slopes": "k_slopes", "faces": "k_faces_lgi", "update": "k_update"},
                1: {"cfl": "k_cfl32", "slopes": "k_slopes32", "faces": "k_faces32_lgi", "update": "k_update_mixed"}}


def device_extensives(mesh, cells, local_rank, offsets=None, gammas=None):
    """hdsim's init_extensives of the cells, formed by the library on the
    device (the FP64 path; per-problem gamma for a batch)."""
    import richgpu
    with richgpu.Handle(gamma=GAMMA, order=2, ghost_kind=0, device=local_rank) as h:
        h.upload_mesh(mesh)
        if offsets is not None:
            h.set_problems(offsets, gammas)
        h.set_cells(cells)
        h.init_extensives()
        return h.get_extensives()


def measure(precision, mesh, cells, ext, args, local_rank, barrier, max_over_ranks):
    """Warm-up + timed steps of one precision; returns the timing record and
    the final cells (for the accuracy comparison)."""
    import torch
    import richgpu

    h = richgpu.Handle(gamma=GAMMA, order=2, ghost_kind=0, precision=precision, device=local_rank)
    h.set_outer_box(-1.0, 1.0, -1.0, 1.0)
    h.upload_mesh(mesh, flags=richgpu.MESH_DEVICE_GEOMETRY)
    # RoundCells(Lagrangian) with StationaryBox face velocities, as the Sedov
    # configuration moves its mesh; the face velocities are computed on the
    # device and every timed kernel reads them
    h.set_point_motion(kind=2, edges=0, chi=0.15, eta=0.02)
    h.set_cells(cells)
    h.set_extensives(ext)
    h.point_velocities()
    # launch shapes of the per-step kernels chosen by the library's autotuner
    # on this mesh and state (before the warm-up; the state is unchanged)
    shapes = h.launch_shapes() if args.no_tune else h.autotune(reps=5)
    warm = max(args.warmup, 3)
    for _ in range(warm):
        h.step()
    stream = torch.cuda.ExternalStream(h.stream())
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    clocks = ClockSampler(local_rank)
    kms = []
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    wall0 = time.perf_counter()
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        _, k = h.step_timed()
        kms.append(k)
    torch.cuda.synchronize()
    barrier()
    wall = time.perf_counter() - wall0
    clock = clocks.stop()
    final_cells = h.get_cells()
    kms = np.array(kms)
    total_ms = max_over_ranks(float(kms.sum()))

    # end to end through the C ABI with host buffers (moving-mesh data flow):
    # each step uploads the tessellation the host would have rebuilt (points,
    # topology, face vertices, from pinned memory), runs hdsim::TimeAdvance's
    # first half on the device (rg_advance_begin) and the cell update, and
    # reads the cells, extensives and point velocities back into pinned memory
    pmesh, ppv, pcells, pext = pinned_io(mesh, np.zeros((mesh.n_cells, 2)), torch)
    ke = max(1, min(args.steps, 30))
    upload_ms = []
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(ke):
        h.upload_mesh(pmesh, flags=richgpu.MESH_DEVICE_GEOMETRY)
        upload_ms.append(h.last_upload_ms())
        if k:
            # the previous step's cells and extensives, copied while this
            # step's mesh went up
            h.wait_state()
        h.advance_begin(out=ppv)
        h.cell_update()
        h.get_state_async(pcells, pext)
    h.wait_state()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    h.close()
    del flush
    return {"kernel_ms": kms.mean(0), "total_ms": total_ms, "wall": wall, "clock": clock,
            "e2e_s": e2e_s, "e2e_steps": ke, "upload_ms": float(np.mean(upload_ms)),
            "warmup": warm, "shapes": shapes}, final_cells


def fixed_mesh_l1(mesh, cells, ext, steps, local_rank):
    """Density L1 (relative) of the FP32-mixed path against the FP64 path
    after `steps` steps of the timed workload from the same initial state
    (the fixed mesh with RoundCells face velocities, dt from SimpleCFL on
    each path)."""
    import richgpu
    out = []
    for precision in (0, 1):
        with richgpu.Handle(gamma=GAMMA, order=2, ghost_kind=0, precision=precision, device=local_rank) as h:
            h.set_outer_box(-1.0, 1.0, -1.0, 1.0)
            h.upload_mesh(mesh, flags=richgpu.MESH_DEVICE_GEOMETRY)
            h.set_point_motion(kind=2, edges=0, chi=0.15, eta=0.02)
            h.set_cells(cells)
            h.set_extensives(ext)
            h.point_velocities()
            h.run(steps)
            out.append(h.get_cells())
    c64, c32 = out
    return float(np.abs(c32[:, 0] - c64[:, 0]).sum() / np.abs(c64[:, 0]).sum())


def pinned_io(mesh, ev, torch):
    """Copies of the per-step inputs and outputs in pinned (page-locked) host memory."""
    from meshview import MESH_FIELDS, PackedMesh

    def pin(a):
        t = torch.empty(a.shape, dtype=getattr(torch, str(a.dtype)), pin_memory=True)
        out = t.numpy()
        out[...] = a
        return out
    pm = PackedMesh(**{k: pin(getattr(mesh, k)) for k in MESH_FIELDS})
    return (pm, pin(ev), pin(np.zeros((mesh.n_cells, 4))), pin(np.zeros((mesh.n_cells, 4))))


def link_floor(h2d, d2h, reps=20):
    """Host<->device link speed for the e2e step's byte counts: one pinned
    copy each way of the same size, timed with CUDA events (the e2e copies
    cannot be faster than this)."""
    import torch
    out = {}
    for name, nbytes in (("h2d", h2d), ("d2h", d2h)):
        host = torch.empty(int(nbytes), dtype=torch.uint8, pin_memory=True)
        dev = torch.empty(int(nbytes), dtype=torch.uint8, device="cuda")
        src, dst = (host, dev) if name == "h2d" else (dev, host)
        for _ in range(3):
            dst.copy_(src, non_blocking=True)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        for _ in range(reps):
            dst.copy_(src, non_blocking=True)
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / reps
        out[name + "_ms"] = ms
        out[name + "_gbs"] = nbytes / (ms * 1e-3) / 1e9
    out["copy_floor_ms"] = out["h2d_ms"] + out["d2h_ms"]
    return out


def roofline(rec, mesh, precision):
    alg = algorithmic_bytes(mesh, precision)
    dom = int(np.argmax(rec["kernel_ms"]))
    name = KERNELS[dom]
    peak, peak_kind = measured_peaks()
    achieved = alg[name] / (rec["kernel_ms"][dom] * 1e-3) / 1e9
    kname = KERNEL_NAMES[precision][name]
    step_alg = (172 if precision == 0 else 140) * mesh.n_cells + 64 * mesh.n_faces
    step_ms = float(rec["kernel_ms"].sum())
    return {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)",
            "traffic": ncu_traffic(kname), "algorithmic_bytes_per_launch": alg[name],
            "kernel_ms_mean": {KERNEL_NAMES[precision][k]: float(v) for k, v in zip(KERNELS, rec["kernel_ms"])},
            "step_algorithmic_bytes": step_alg, "step_achieved_gbs": step_alg / (step_ms * 1e-3) / 1e9}


def run_gpu(args, world, rank, local_rank):
    import torch

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()

    def max_over_ranks(x):
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    mesh, cells = workload()
    ext = device_extensives(mesh, cells, local_rank)
    r64, c64 = measure(0, mesh, cells, ext, args, local_rank, barrier, max_over_ranks)
    r32, c32 = measure(1, mesh, cells, ext, args, local_rank, barrier, max_over_ranks)
    l1 = float(np.abs(c32[:, 0] - c64[:, 0]).sum() / np.abs(c64[:, 0]).sum())
    l1_500 = fixed_mesh_l1(mesh, cells, ext, 500, local_rank) if rank == 0 else None
    n, k = mesh.n_cells, args.steps
    value32 = world * n * k / (r32["total_ms"] * 1e-3)
    value64 = world * n * k / (r64["total_ms"] * 1e-3)
    h2d = mesh.topology_nbytes()
    d2h = 2 * 32 * n + 16 * n + 8

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline_block(mesh, cells, ext)
    adjoint = adjoint_block() if rank == 0 and not args.no_adjoint else None
    sedov3d = sedov3d_block(cpu=not args.no_cpu) if rank == 0 and not args.no_3d else None
    tracers = tracers_block(r64["total_ms"] / k) if rank == 0 and not args.no_tracers else None
    batch = batch_block(cpu=not args.no_cpu) if rank == 0 and world == 1 and not args.no_batch else None
    hdsim = hdsim_block() if rank == 0 and world == 1 and not args.no_hdsim else None
    accuracy = accuracy_block() if rank == 0 and world == 1 and not args.no_hdsim else None
    if rank == 0:
        line = {"metric": METRIC, "value": value32, "unit": UNIT, "n_gpus": world, "steps": k,
                "warmup": r32["warmup"], "ms_per_step": r32["total_ms"] / k, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
                "data": "synthetic", "config": config_block(mesh),
                "impl_notes": dict(IMPL_NOTES, mesh_source=_WORKLOAD.get("source")),
                "precision": "FP32-mixed: reconstruction, HLLC, CFL in FP32 (FP32 geometry from FP64 "
                             "coordinate differences); volumes, CMs, motion, extensive accumulation, "
                             "E/m - v^2/2 in FP64",
                "l1_density_vs_fp64": l1, "l1_after_steps": r32["warmup"] + k,
                "l1_density_vs_fp64_500_steps": l1_500,
                "roofline": roofline(r32, mesh, 1),
                "cpu_baseline": cpu,
                "e2e": {"value": world * n * r32["e2e_steps"] / r32["e2e_s"], "unit": UNIT,
                        "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                        "steps": r32["e2e_steps"], "ms_per_step": r32["e2e_s"] * 1e3 / r32["e2e_steps"],
                        "upload_ms_mean": r32["upload_ms"], "link": link_floor(h2d, d2h)},
                "gpu_launches": 4 * k, "clocks": r32["clock"],
                "launch_shapes": {kk: [v["block"], v["max_blocks"], v["variant"]] for kk, v in r32["shapes"].items()},
                "faces_per_s": world * mesh.n_faces * k / (r32["total_ms"] * 1e-3),
                "fp64": {"value": value64, "ms_per_step": r64["total_ms"] / k, "dtype": "f64",
                         "parity": "bit-exact to the reference (tests/test_gpu_parity.py)", "roofline": roofline(r64, mesh, 0),
                         "note": "plain FP64 path: bound by GB300's FP64 pipe (2 DFMA/clk/SM), not HBM",
                         "launch_shapes": {kk: [v["block"], v["max_blocks"], v["variant"]] for kk, v in r64["shapes"].items()},
                         "e2e": {"value": world * n * r64["e2e_steps"] / r64["e2e_s"], "unit": UNIT,
                                 "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
                         "clocks": r64["clock"]},
                "speedup_fp32mixed_vs_fp64": value32 / value64,
                "adjoint": adjoint,
                "sedov3d": sedov3d,
                "tracers": tracers,
                "batch": batch,
                "e2e_hdsim": hdsim,
                "accuracy_hdsim_moving_mesh": accuracy,
                "accuracy_hdsim_512x500": recorded_accuracy(),
                "wall_s_timed_region": r32["wall"] + r64["wall"]}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


# ------------------------------------------------------------------ tracers

def tracers_block(fp64_ms_per_step, steps=20, warmup=3):
    """The FP64 step of the same 512^2 Sedov workload with three tracers
    ("A" limited by LinearGaussImproved, "Entropy" recomputed by the cell
    updater, "Z" piecewise constant) and two stickers (HasSticker +
    SkipUpdate on 1% of the cells, LinearGaussImproved's skip_key on 2%, all
    outside r = 0.5): ms per step and the cost over the tracer-free step.
    Bit-identical to the reference (the entropy tracer to a few ulp)."""
    import torch
    import richgpu
    mesh, cells = workload()
    rng = np.random.default_rng(17)
    n = mesh.n_cells
    xy = mesh.point_xy[:n]
    r = np.hypot(xy[:, 0], xy[:, 1])
    tr = np.stack([xy[:, 0], cells[:, 1] * cells[:, 0] ** -GAMMA, (r < 0.3).astype(float)], axis=1)
    far = r > 0.5
    stickers = ((rng.random(n) < 0.01) & far).astype(np.uint32) | \
        (((rng.random(n) < 0.02) & far).astype(np.uint32) << 1)
    with richgpu.Handle(gamma=GAMMA, order=2, ghost_kind=0, device=0) as h:
        h.upload_mesh(mesh)
        h.set_tracer_config(3, limited=[0], entropy=1, skip_sticker=1, frozen_sticker=0)
        h.set_stickers(stickers)
        h.set_cells(cells)
        h.set_tracers(tr)
        h.init_extensives()
        h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
        for _ in range(warmup):
            h.step()
        stream = torch.cuda.ExternalStream(h.stream())
        flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device="cuda")
        kms = []
        torch.cuda.synchronize()
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            _, k = h.step_timed()
            kms.append(k)
        torch.cuda.synchronize()
        del flush
    kms = np.array(kms).mean(0)
    ms = float(kms.sum())
    return {"workload": "sedov2d_512x512_lgi_hllc_fp64_3tracers_2stickers", "n_tracers": 3,
            "ms_per_step": ms, "value": n / (ms * 1e-3), "unit": UNIT, "steps": steps, "warmup": warmup,
            "phase_ms": {"cfl": float(kms[0]), "slopes+tracer_slopes": float(kms[1]),
                         "faces+tracer_faces": float(kms[2]), "update+tracer_update": float(kms[3])},
            "cost_vs_tracer_free_fp64": ms / fp64_ms_per_step,
            "gpu_launches_per_step": 7, "l2": "flushed before every timed step (256 MiB write)"}


# ------------------------------------------------------------------ 3D

def sedov3d_block(steps=20, warmup=3, cpu=True):
    """3D first-order path on the 3D configuration's size: Sedov-Taylor on a
    96^3 CubeGrid over [-0.5, 0.5]^3 (884,736 cells, 2,681,856 faces; rho 1,
    p 1e-6, E = 1 in r < 0.04, gamma 5/3, CFL 0.3), HDSim3D's step with
    FirstOrderHydroFlux(Hllc), update_extensive, DefaultCellUpdater (FP64,
    bit-identical to the reference).  The reference has no LinearGauss3D /
    Hllc3D / Voronoi3D; CubeGrid first order is its 3D path.  Each step is
    timed with CUDA events per kernel; its working set (about 400 MB) is
    larger than L2."""
    import richgpu
    import synthetic
    n = 96
    box = dict(lo=(-0.5, -0.5, -0.5), hi=(0.5, 0.5, 0.5))
    mesh = synthetic.cube_grid(n, n, n, **box)
    cells = synthetic.cube_sedov_cells(n, GAMMA)
    def timed(precision):
        with richgpu.Handle3(gamma=GAMMA, device=0, precision=precision) as h:
            h.upload_mesh(mesh)
            h.set_cells(cells)
            h.init_extensives()
            for _ in range(warmup):
                h.step()
            k = np.array([h.step_timed()[1] for _ in range(steps)])
            return k, h.get_cells()

    kms, c64 = timed(0)
    kms32, c32 = timed(1)
    N, F = mesh.n_cells, mesh.n_faces
    ms = float(kms.sum(1).mean())
    # algorithmic bytes per launch (220 N + 96 F per step in total):
    # faces: neighbour pair 8 + normal 24 + area 8 + flux out 40 per face, the cells once (40 per cell)
    faces_bytes = F * (8 + 24 + 8 + 40) + N * 40
    kf = float(kms[:, 1].mean())
    peak = measured_peaks()
    rec = {"workload": "sedov3d_cubegrid_96^3_first_order_hllc_fp64", "cells": N, "faces": F, "steps": steps,
           "ms_per_step": ms, "cell_updates_per_s": N / (ms * 1e-3), "faces_per_s": F / (ms * 1e-3),
           "kernel_ms_mean": {"k3_cfl": float(kms[:, 0].mean()), "k3_faces": kf, "k3_update": float(kms[:, 2].mean())},
           "parity": "bit-exact to the reference's HDSim3D (tests/test_gpu_3d.py)",
           "roofline": {"bound": "hbm", "kernel": "k3_faces", "achieved": faces_bytes / (kf * 1e-3) / 1e9,
                        "peak": peak[0], "unit": "GB/s", "frac": faces_bytes / (kf * 1e-3) / 1e9 / peak[0],
                        "traffic": ncu_traffic("k3_faces"), "algorithmic_bytes_per_launch": faces_bytes,
                        "note": "FP64 Hllc per face: bound by GB300's FP64 pipe"}}
    ms32 = float(kms32.sum(1).mean())
    kf32 = float(kms32[:, 1].mean())
    faces_bytes32 = F * (8 + 16 + 4 + 20) + N * 20  # FP32 normal, area, flux out; FP32 cells
    rec["fp32_mixed"] = {
        "ms_per_step": ms32, "cell_updates_per_s": N / (ms32 * 1e-3),
        "kernel_ms_mean": {"k3m_cfl": float(kms32[:, 0].mean()), "k3m_faces": kf32,
                           "k3m_update": float(kms32[:, 2].mean())},
        "l1_density_vs_fp64": float(np.abs(c32[:, 0] - c64[:, 0]).sum() / np.abs(c64[:, 0]).sum()),
        "l1_after_steps": warmup + steps,
        "roofline": {"bound": "hbm", "kernel": "k3m_faces", "achieved": faces_bytes32 / (kf32 * 1e-3) / 1e9,
                     "peak": peak[0], "unit": "GB/s", "frac": faces_bytes32 / (kf32 * 1e-3) / 1e9 / peak[0],
                     "traffic": ncu_traffic("k3m_faces"), "algorithmic_bytes_per_launch": faces_bytes32}}
    if cpu:
        import oracle
        ext = oracle.init_extensives3(mesh, cells, GAMMA)
        t0 = time.perf_counter()
        k = 0
        c, e = cells, ext
        while k < 3 and (k == 0 or time.perf_counter() - t0 < 10):
            c, e, _ = oracle.run3(mesh, c, e, GAMMA, 1)
            k += 1
        tc = time.perf_counter() - t0
        rec["cpu_baseline"] = {"value": N * k / tc, "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": f"{k} steps of the same 96^3 workload, one thread, oracle/rich_oracle.c ro3_step"}
    return rec


# ------------------------------------------------------------------ adjoint

def adjoint_block(reps=3):
    """Differentiation form on its own workload: 256x256 periodic lattice,
    rho = 1 + 8 Gaussian bumps, p = 1, velocity from 16 Fourier modes,
    gamma 5/3, LinearGaussImproved + Hllc, 200 steps at the initial CFL-0.3
    dt, loss = L2 of the final density against a second seeded field,
    checkpoints every 20 steps.  Forward = rg_step_fwd, backward =
    rg_step_bwd (seed upload, recomputation, reverse sweep, gradient
    download), each a synchronous C-ABI call timed on the host; the cost
    ratio is backward over forward.  The dot-product residual compares the
    adjoint with one tangent-linear run."""
    import richgpu
    import synthetic
    mesh = synthetic.lattice_mesh(256, 256, (0.0, 1.0, 0.0, 1.0), "periodic", seed=3)
    cells = synthetic.bumps_cells(mesh)
    target = synthetic.bumps_cells(mesh, seed=11)[:, 0]
    steps, every = 200, 20
    with richgpu.Handle(gamma=GAMMA, order=2, ghost_kind=1, device=0) as h:
        h.upload_mesh(mesh)
        h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
        h.set_cells(cells)
        dt = h.cfl_dt()
        fwd_ms, bwd_ms = [], []
        for _ in range(reps + 1):
            h.set_cells(cells)
            t0 = time.perf_counter()
            h.step_fwd(steps, dt, every)
            t1 = time.perf_counter()
            wn = h.get_cells()
            seed = np.zeros_like(wn)
            seed[:, 0] = 2.0 * (wn[:, 0] - target)
            t2 = time.perf_counter()
            g = h.step_bwd(seed)
            t3 = time.perf_counter()
            fwd_ms.append((t1 - t0) * 1e3)
            bwd_ms.append((t3 - t2) * 1e3)
        fwd_ms, bwd_ms = fwd_ms[1:], bwd_ms[1:]
        dw = np.random.default_rng(1).normal(size=cells.shape)
        h.set_cells(cells)
        tl = h.step_tlm(steps, dt, dw)
        lhs, rhs = float(np.sum(seed * tl)), float(np.sum(g * dw))
    f, b = statistics.median(fwd_ms), statistics.median(bwd_ms)
    # the FP32-mixed step's adjoint on the same problem and dt
    with richgpu.Handle(gamma=GAMMA, order=2, ghost_kind=1, device=0, precision=1) as h:
        h.upload_mesh(mesh)
        h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
        fwd32, bwd32 = [], []
        for _ in range(reps + 1):
            h.set_cells(cells)
            t0 = time.perf_counter()
            h.step_fwd(steps, dt, every)
            t1 = time.perf_counter()
            wn32 = h.get_cells()
            seed32 = np.zeros_like(wn32)
            seed32[:, 0] = 2.0 * (wn32[:, 0] - target)
            t2 = time.perf_counter()
            g32 = h.step_bwd(seed32)
            t3 = time.perf_counter()
            fwd32.append((t1 - t0) * 1e3)
            bwd32.append((t3 - t2) * 1e3)
    f32, b32 = statistics.median(fwd32[1:]), statistics.median(bwd32[1:])
    return {"workload": "periodic_bumps_256x256_lgi_hllc_fp64_200steps_fixed_dt", "cells": mesh.n_cells,
            "steps": steps, "checkpoint_every": every, "fwd_ms": f, "bwd_ms": b, "adjoint_over_fwd": b / f,
            "fwd_cell_updates_per_s": mesh.n_cells * steps / (f * 1e-3),
            "dot_product_rel": abs(lhs - rhs) / abs(lhs),
            "fp32_mixed": {"fwd_ms": f32, "bwd_ms": b32, "adjoint_over_fwd": b32 / f32,
                           "bwd_speedup_vs_fp64": b / b32,
                           "gradient_rel_l2_vs_fp64": float(np.linalg.norm(g32 - g) / np.linalg.norm(g)),
                           "final_density_l1_vs_fp64": float(np.abs(wn32[:, 0] - wn[:, 0]).sum()
                                                             / np.abs(wn[:, 0]).sum()),
                           "note": "FP32-mixed step forward; reverse with FP32 reconstruction, limiter and "
                                   "Hllc and FP64 gathers and cell update"},
            "timing": "host wall clock around synchronous C-ABI calls, median of %d" % reps}


# ------------------------------------------------------------------ batch

def _batch_cpu_worker(args):
    problems, steps = args
    import oracle
    import synthetic
    done, t = 0, 0.0
    for p in problems:
        m, c, g = synthetic.riemann_problem(p, BATCH_SEED)
        e = oracle.init_extensives(m, c, g)
        ev = np.zeros((m.n_faces, 2))
        t0 = time.perf_counter()
        oracle.run(m, c, e, ev, g, steps, 0.3, 2, oracle.lgi_params(0))
        t += time.perf_counter() - t0
        done += m.n_cells * steps
    return done, t


BATCH_SEED = 11


def batch_measure(lo, hi, steps, warmup, tune, local_rank, barrier=lambda: None):
    """Generates problems [lo, hi) of the batched workload and times `steps`
    steps of both precisions (CUDA events per kernel, then a CUDA graph of one
    step replayed `steps` times).  Returns the per-precision records, the
    batch mesh and the generation time."""
    import torch
    import richgpu
    import synthetic
    t0 = time.perf_counter()
    mesh, off, gam, cells, _ = synthetic.riemann_batch_range(range(lo, hi), seed=BATCH_SEED)
    gen_s = time.perf_counter() - t0
    ext = device_extensives(mesh, cells, local_rank, off, gam)
    res = {}
    for precision in (0, 1):
        h = richgpu.Handle(gamma=1.4, order=2, ghost_kind=0, precision=precision, device=local_rank)
        h.upload_mesh(mesh)
        h.set_problems(off, gam)
        h.set_cells(cells)
        h.set_extensives(ext)
        h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
        shapes = h.autotune(reps=3) if tune else h.launch_shapes()
        for _ in range(max(warmup, 3)):
            h.step()
        kms = []
        barrier()
        torch.cuda.synchronize()
        for _ in range(steps):
            _, k = h.step_timed()
            kms.append(k)
        torch.cuda.synchronize()
        barrier()
        kms = np.array(kms)
        stream = torch.cuda.ExternalStream(h.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        h.run_graph(1)
        with torch.cuda.stream(stream):
            e0.record()
        h.run_graph(steps)
        with torch.cuda.stream(stream):
            e1.record()
        torch.cuda.synchronize()
        graph_ms = e0.elapsed_time(e1) / steps
        times, _ = h.problem_times()
        res[precision] = {"ms_per_step": float(kms.sum(1).mean()), "kernel_ms": kms.mean(0).tolist(),
                          "graph_ms_per_step": graph_ms, "final_cells": h.get_cells(),
                          "launch_shapes": {kk: [v["block"], v["max_blocks"], v["variant"]] for kk, v in shapes.items()},
                          "time_min": float(times.min()), "time_max": float(times.max())}
        if precision == 1:
            # the same steps as one cooperative launch (RG_STEP_PERSISTENT)
            h.set_step_mode(richgpu.STEP_PERSISTENT)
            h.run(1)
            with torch.cuda.stream(stream):
                e0.record()
            h.run(steps)
            with torch.cuda.stream(stream):
                e1.record()
            torch.cuda.synchronize()
            res[precision]["persistent_ms_per_step"] = e0.elapsed_time(e1) / steps
        h.close()
    return res, mesh, gen_s


def batch_cpu_baseline(problems):
    import multiprocessing as mp
    cores = min(os.cpu_count() or 1, 64)
    sample = list(range(0, problems, max(1, problems // (2 * cores))))[:2 * cores]
    chunks = [sample[k::cores] for k in range(cores)]
    with mp.get_context("spawn").Pool(cores) as pool:
        out = pool.map(_batch_cpu_worker, [(c, 2) for c in chunks if c])
    t_wall = max(o[1] for o in out)
    return {"value": sum(o[0] for o in out) / t_wall, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{len(sample)} of the {problems} problems, 2 steps each, one process per core "
                      "(C restatement oracle/rich_oracle.c; the reference has no batched driver)"}


def batch_roofline(res, mesh):
    """The dominant kernel of the FP32-mixed batch step against HBM: the
    single-problem byte counts (every problem's cells and faces once) plus the
    per-point problem index (4 B) the batch kernels read."""
    alg = algorithmic_bytes(mesh, 1)
    n = mesh.n_cells
    kms = np.array(res[1]["kernel_ms"])
    dom = int(np.argmax(kms))
    name = KERNELS[dom]
    nbytes = alg[name] + 4 * n
    peak, peak_kind = measured_peaks()
    achieved = nbytes / (kms[dom] * 1e-3) / 1e9
    return {"bound": "hbm", "kernel": KERNEL_NAMES[1][name] + "<batch>", "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)",
            "algorithmic_bytes_per_launch": nbytes,
            "kernel_ms_mean": {KERNEL_NAMES[1][k]: float(v) for k, v in zip(KERNELS, kms)}}


def batch_block(steps=20, warmup=3, problems=512, tune=True, cpu=True):
    """The batched form inside the default benchmark run: all `problems`
    problems on this GPU, both precisions, graph replay, roofline and a CPU
    sample."""
    res, mesh, gen_s = batch_measure(0, problems, steps, warmup, tune, 0)
    c32, c64 = res[1].pop("final_cells"), res[0].pop("final_cells")
    n = mesh.n_cells
    return {"workload": f"riemann_batch_{problems}", "problems": problems, "cells": n, "faces": mesh.n_faces,
            "steps": steps, "warmup": max(warmup, 3), "value": n / (res[1]["ms_per_step"] * 1e-3), "unit": UNIT,
            "ms_per_step": res[1]["ms_per_step"], "dtype": "f32+f64",
            "graph_value": n / (res[1]["graph_ms_per_step"] * 1e-3),
            "persistent_value": n / (res[1]["persistent_ms_per_step"] * 1e-3),
            "l1_density_vs_fp64": float(np.abs(c32[:, 0] - c64[:, 0]).sum() / np.abs(c64[:, 0]).sum()),
            "fp32mixed": res[1], "fp64": {"value": n / (res[0]["ms_per_step"] * 1e-3), **res[0]},
            "roofline": batch_roofline(res, mesh),
            "cpu_baseline": batch_cpu_baseline(problems) if cpu else None,
            "generation_s": gen_s, "gpu_launches_per_step": 4,
            "launch": "one launch per phase for all problems, per-problem dt; graph of one step replayed; "
                      "persistent: the whole run in one cooperative launch (RG_STEP_PERSISTENT)"}


def run_batch(args, world, rank, local_rank):
    """512 independent 2D Riemann problems (cell counts log-uniform in
    [1024, 65536], rigid walls, LinearGaussImproved + Hllc, gamma 1.4 or 5/3)
    advanced together: one launch per phase for all problems, per-problem
    dt; also replayed from a CUDA graph of one step.  With N ranks each rank
    advances a contiguous range of the problems holding about 1/N of the
    cells (sharding.problem_shard): no collective on the data path, the
    timing is the maximum over ranks and `value` counts every rank's cells."""
    import torch
    import synthetic
    from sharding import problem_shard

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def reduce(x, op):
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=op)
        return float(t.item())

    counts = [synthetic.riemann_problem_cells(p, BATCH_SEED) for p in range(args.problems)]
    lo, hi = problem_shard(counts, world, rank)
    if hi <= lo:
        raise SystemExit(f"rank {rank}: no problems in its shard ({args.problems} problems, {world} ranks)")
    res, mesh, gen_s = batch_measure(lo, hi, args.steps, args.warmup, not args.no_tune, local_rank,
                                     barrier=(dist.barrier if dist is not None else lambda: None))
    c32, c64 = res[1].pop("final_cells"), res[0].pop("final_cells")
    l1 = float(np.abs(c32[:, 0] - c64[:, 0]).sum() / np.abs(c64[:, 0]).sum())
    roof = batch_roofline(res, mesh)
    # every rank's cells over the slowest rank's step time
    if dist is not None:
        from torch.distributed import ReduceOp
        l1 = reduce(l1, ReduceOp.MAX)
        for r in res.values():
            for key in ("ms_per_step", "graph_ms_per_step", "persistent_ms_per_step"):
                if key in r:
                    r[key] = reduce(r[key], ReduceOp.MAX)
    n = int(reduce(float(mesh.n_cells), dist.ReduceOp.SUM if dist is not None else None))
    n_faces = int(reduce(float(mesh.n_faces), dist.ReduceOp.SUM if dist is not None else None))
    if rank != 0:
        dist.destroy_process_group()
        return
    cpu = batch_cpu_baseline(args.problems) if (not args.no_cpu and world == 1) else None
    line = {"metric": METRIC, "value": n / (res[1]["ms_per_step"] * 1e-3), "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": max(args.warmup, 3),
            "ms_per_step": res[1]["ms_per_step"], "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": f"riemann_batch_{args.problems}", "problems": args.problems, "cells": n,
                       "faces": n_faces, "order": 2, "reconstruction": "LinearGaussImproved",
                       "riemann": "Hllc", "gamma": "1.4 or 5/3 per problem", "dt": "per problem (SimpleCFL 0.3)",
                       "launch": "one launch per phase for all problems; graph of one step replayed",
                       "parallelism": f"problems sharded over {world} rank(s), contiguous ranges of ~equal cells",
                       "rank0_problems": [lo, hi], "generation_s": gen_s},
            "l1_density_vs_fp64": l1, "roofline": roof,
            "fp32mixed": {k: v for k, v in res[1].items()},
            "fp64": {"value": n / (res[0]["ms_per_step"] * 1e-3), **res[0]},
            "graph_value_fp32mixed": n / (res[1]["graph_ms_per_step"] * 1e-3),
            "persistent_value_fp32mixed": n / (res[1]["persistent_ms_per_step"] * 1e-3),
            "cpu_baseline": cpu, "gpu_launches": 4 * args.steps}
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


# ------------------------------------------------------------------ hdsim

def accuracy_block(n=128, steps=200):
    """Accuracy on the moving-mesh Sedov configuration through hdsim: the
    GPU FP64 and FP32-mixed plugins in lockstep and the reference's own
    plugins at the same time in another process (tests/hdsim_dropin.cpp,
    `accuracy` mode), RoundCells moving the points and the host rebuilding
    the Voronoi mesh every step.  Density L1 (relative) after `steps` steps,
    and whether the FP64 plugins' state equalled the stock one's after every
    step."""
    exe = os.path.join(REF_BIN, "hdsim_dropin")
    if not os.path.exists(exe):
        return {"unavailable": "hdsim_dropin was not built (the reference's sources are not staged)"}
    r = subprocess.run([exe, "accuracy", "sedov", str(n), str(steps), "stock"], capture_output=True, text=True,
                       timeout=7200)
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    if r.returncode != 0 or not lines:
        return {"failed": r.stderr[-500:]}
    d = json.loads(lines[-1])
    return {"workload": f"hdsim::TimeAdvance sedov {n}x{n}, RoundCells(Lagrangian), host VoronoiMesh rebuild "
                        f"every step, {steps} steps",
            "l1_density_fp32mixed_vs_fp64": d["l1_density_fp32mixed_vs_fp64"],
            "l1_density_fp64_vs_stock": d["l1_density_fp64_vs_stock"],
            "l1_density_fp32mixed_vs_stock": d["l1_density_fp32mixed_vs_stock"],
            "fp64_equal_to_stock_every_step": d["fp64_equal_to_stock"],
            "first_differing_step": d["first_differing_step"], "unmatched_cells": d["unmatched"],
            "time": {"stock": d["time_stock"], "fp64": d["time_fp64"], "fp32_mixed": d["time_fp32mixed"]},
            "ms_per_step": {"stock": d["stock"]["ms_per_step"], "fp64": d["gpu_fp64"]["ms_per_step"],
                            "fp32_mixed": d["gpu_fp32mixed"]["ms_per_step"]}}


def recorded_accuracy():
    """The 512^2 x 500-step record of accuracy_block (bench.py --workload
    accuracy), kept in profiles/accuracy_sedov512.md: its run takes minutes,
    longer than a default benchmark run."""
    p = os.path.join(ROOT, "profiles", "accuracy_sedov512.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("{") and '"l1_density_fp32mixed_vs_fp64"' in line:
            rec = json.loads(line)
            rec["source"] = "recorded: profiles/accuracy_sedov512.md (python bench.py --workload accuracy)"
            return rec
    return None



def hdsim_block(n=NX, steps=5, stock_steps=2):
    """hdsim::TimeAdvance of the Sedov problem (n x n, RoundCells(Lagrangian),
    LinearGaussImproved + Hllc) with the GPU plugins and with the
    reference's own plugins, the host moving the points and rebuilding the
    Voronoi mesh every step (tests/hdsim_dropin.cpp, `time` mode): ms per
    step, the part spent in the four plugin calls and the host's rest."""
    exe = os.path.join(REF_BIN, "hdsim_dropin")
    if not os.path.exists(exe):
        return {"unavailable": "hdsim_dropin was not built (the reference's sources are not staged)"}
    rec = {"workload": f"hdsim::TimeAdvance sedov {n}x{n}, RoundCells(Lagrangian), StationaryBox, "
                       "LinearGaussImproved + Hllc, host VoronoiMesh rebuild every step",
           "note": "each step: host point motion and face velocities, GPU plugins (CFL, fluxes, extensive and "
                   "cell update through rich_gpu_adapters.hpp, C ABI), host MoveMeshPoints + VoronoiMesh rebuild"}
    for name, set_, k in (("fp32_mixed", "gpu32", steps), ("fp64", "gpu", steps), ("stock", "stock", stock_steps)):
        r = subprocess.run([exe, "time", "sedov", str(n), str(k), set_], capture_output=True, text=True,
                           timeout=900)
        lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
        if r.returncode != 0 or not lines:
            rec[name] = {"failed": r.stderr[-300:]}
            continue
        d = json.loads(lines[-1])
        t = d[set_]
        rec[name] = {"ms_per_step": t["ms_per_step"], "cell_updates_per_s": d["cells"] / (t["ms_per_step"] * 1e-3),
                     "plugin_ms_per_step": t["plugin_ms_per_step"], "host_rest_ms_per_step": t["host_rest_ms_per_step"],
                     "steps": k, "plugins_ms": {kk: t[kk] for kk in ("cfl_ms", "flux_ms", "extensive_update_ms",
                                                                       "cell_update_ms")}}
    if all("ms_per_step" in rec.get(k, {}) for k in ("fp32_mixed", "fp64", "stock")):
        rec["value"] = rec["fp32_mixed"]["cell_updates_per_s"]
        rec["unit"] = UNIT
        rec["speedup_vs_stock_fp32_mixed"] = rec["stock"]["ms_per_step"] / rec["fp32_mixed"]["ms_per_step"]
        rec["speedup_vs_stock_fp64"] = rec["stock"]["ms_per_step"] / rec["fp64"]["ms_per_step"]
        rec["plugin_speedup_vs_stock_fp64"] = rec["stock"]["plugin_ms_per_step"] / rec["fp64"]["plugin_ms_per_step"]
    return rec


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint cost measurement")
    ap.add_argument("--no-tune", action="store_true", help="default launch shapes instead of the autotuner's")
    ap.add_argument("--no-tracers", action="store_true", help="skip the tracer-path measurement")
    ap.add_argument("--no-3d", action="store_true", help="skip the 3D first-order measurement")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-form measurement")
    ap.add_argument("--no-hdsim", action="store_true", help="skip hdsim driven through the GPU plugins")
    ap.add_argument("--workload", default="sedov", choices=["sedov", "riemann_batch", "sedov3d", "accuracy"])
    ap.add_argument("--accuracy-n", type=int, default=512)
    ap.add_argument("--accuracy-steps", type=int, default=500)
    ap.add_argument("--problems", type=int, default=512)
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload == "accuracy":
        if rank == 0:
            print(json.dumps(accuracy_block(args.accuracy_n, args.accuracy_steps)), flush=True)
    elif args.workload == "riemann_batch":
        run_batch(args, world, rank, local_rank)
    elif args.workload == "sedov3d":
        if rank == 0:
            rec = sedov3d_block(steps=args.steps, warmup=max(args.warmup, 3), cpu=not args.no_cpu)
            line = {"metric": "cell-updates/s, 3D first-order path (FP64)", "value": rec["cell_updates_per_s"],
                    "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3),
                    "ms_per_step": rec["ms_per_step"], "higher_is_better": True, "scaling": "weak",
                    "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                    "config": {"workload": rec["workload"], "cells": rec["cells"], "faces": rec["faces"]},
                    "roofline": rec["roofline"], "cpu_baseline": rec.get("cpu_baseline"),
                    "gpu_launches": 6 * args.steps, "fp32_mixed": rec["fp32_mixed"],
                    "kernel_ms_mean": rec["kernel_ms_mean"]}
            print(json.dumps(line), flush=True)
    else:
        run_gpu(args, world, rank, local_rank)


if __name__ == "__main__":
    main()
