"""ctypes binding of librich_gb300.so (the C ABI in include/rich_gb300.h).

This is the reference-facing boundary as a Python caller sees it: every call
goes through the exported ``rg_*`` functions with host (numpy) buffers, or
with device buffers through :meth:`Handle.device_buffers`.  There is no CPU
fallback: loading fails loudly when the library is missing.
"""
import ctypes as C
import os

import numpy as np

from meshview import (REFERENCE_MESSAGES, STATUS_NAMES, PackedMesh, RgConfig, RgError, RgMeshView,
                      dptr, make_config)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librich_gb300.so")

# every entry point include/rich_gb300.h declares
EXPORTS = ("rg_default_config", "rg_create", "rg_destroy", "rg_status_string", "rg_last_error",
           "rg_upload_mesh", "rg_last_upload_ms", "rg_set_cells", "rg_get_cells",
           "rg_set_extensives", "rg_get_extensives", "rg_get_state_async", "rg_wait_state",
           "rg_set_edge_velocities",
           "rg_device_buffers", "rg_init_extensives", "rg_cfl_dt", "rg_flux", "rg_set_fluxes",
           "rg_extensive_update", "rg_cell_update", "rg_step", "rg_run", "rg_step_async",
           "rg_synchronize", "rg_step_timed", "rg_cfl_dt_noalloc", "rg_set_problems",
           "rg_get_problem_times", "rg_run_graph", "rg_step_fwd", "rg_step_bwd", "rg_step_tlm",
           "rg_autotune", "rg_set_launch_shapes", "rg_get_launch_shapes", "rg_stream",
           "rg3_create", "rg3_destroy", "rg3_last_error", "rg3_upload_mesh", "rg3_set_cells", "rg3_get_cells",
           "rg3_set_extensives", "rg3_get_extensives", "rg3_set_face_velocities", "rg3_init_extensives",
           "rg3_cfl_dt", "rg3_flux", "rg3_extensive_update", "rg3_cell_update", "rg3_step", "rg3_run",
           "rg3_step_timed", "rg_set_tracer_config", "rg_set_tracers", "rg_get_tracers",
           "rg_set_extensive_tracers", "rg_get_extensive_tracers", "rg_set_stickers",
           "rg_get_tracer_fluxes", "rg_get_tracer_slopes", "rg_set_outer_box", "rg_set_point_motion",
           "rg_point_velocities", "rg_apply_fix", "rg_get_edge_velocities", "rg_get_geometry",
           "rg_advance_begin", "rg_set_physical_geometry", "rg_set_tracer_fluxes", "rg_set_flux_rules",
           "rg_set_lagrangian_updater", "rg_get_lagrangian_faces", "rg_set_lagrangian_faces",
           "rg_set_step_mode", "rg_grid_barrier_check")

MESH_DEVICE_GEOMETRY = 2  # RG_MESH_DEVICE_GEOMETRY
STEP_PER_PHASE, STEP_PERSISTENT = 0, 1  # rg_step_mode

KERNELS = ("cfl", "slopes", "faces", "update")


class RgLaunchShapes(C.Structure):
    _fields_ = [("block", C.c_int32 * 4), ("max_blocks", C.c_int32 * 4), ("variant", C.c_int32 * 4),
                ("ms", C.c_float * 4)]


class RgTracerConfig(C.Structure):
    _fields_ = [("n_tracers", C.c_int32), ("n_stickers", C.c_int32), ("limited_mask", C.c_uint32),
                ("entropy_tracer", C.c_int32), ("skip_sticker", C.c_int32), ("frozen_sticker", C.c_int32)]


class RgFluxRule(C.Structure):
    _fields_ = [("sequence", C.c_int32), ("condition", C.c_int32), ("sticker", C.c_int32), ("action", C.c_int32),
                ("ratchet_in", C.c_int32), ("massflux", C.c_int32)]


class RgPointMotion(C.Structure):
    _fields_ = [("kind", C.c_int32), ("edges", C.c_int32), ("chi", C.c_double), ("eta", C.c_double),
                ("cold", C.c_int32), ("correct_overshoot", C.c_int32)]


class RgPhysicalGeometry(C.Structure):
    _fields_ = [("kind", C.c_int32), ("origin", C.c_double * 2), ("direction", C.c_double * 2),
                ("unit", C.c_int32)]


class RgDeviceView(C.Structure):
    _fields_ = [("cells", C.c_void_p), ("extensives", C.c_void_p),
                ("edge_velocities", C.c_void_p), ("fluxes", C.c_void_p), ("stream", C.c_void_p)]


class RichError(RuntimeError):
    """A failure reported by the library; for physical failures the message is
    the reference's UniversalError text."""

    def __init__(self, status, err=None):
        self.status = status
        self.phase = err.phase if err else 0
        self.index = err.index if err else -1
        self.value = err.value if err else 0.0
        msg = REFERENCE_MESSAGES.get(status, STATUS_NAMES.get(status, f"status {status}"))
        super().__init__(f"{msg} (phase {self.phase}, index {self.index}, value {self.value!r})")


_lib = None


def load(path=LIB_PATH):
    """Loads the library (no fallback: raises if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError(f"{path} is missing: build it with huji-rich_gb300/rg_build.py")
    lib = C.CDLL(path)
    vp = C.c_void_p
    dp = C.POINTER(C.c_double)
    lib.rg_create.argtypes = [C.POINTER(RgConfig), C.POINTER(vp)]
    lib.rg_destroy.argtypes = [vp]
    lib.rg_status_string.restype = C.c_char_p
    lib.rg_last_error.argtypes = [vp, C.POINTER(RgError)]
    lib.rg_upload_mesh.argtypes = [vp, C.POINTER(RgMeshView), C.c_uint32]
    lib.rg_last_upload_ms.argtypes = [vp, dp]
    for f in ("rg_set_cells", "rg_get_cells", "rg_set_extensives", "rg_get_extensives",
              "rg_set_edge_velocities", "rg_set_fluxes"):
        getattr(lib, f).argtypes = [vp, dp]
    lib.rg_device_buffers.argtypes = [vp, C.POINTER(RgDeviceView)]
    lib.rg_get_state_async.argtypes = [vp, dp, dp]
    lib.rg_wait_state.argtypes = [vp]
    lib.rg_init_extensives.argtypes = [vp]
    lib.rg_cfl_dt.argtypes = [vp, dp]
    lib.rg_flux.argtypes = [vp, C.c_double, dp]
    lib.rg_extensive_update.argtypes = [vp, C.c_double]
    lib.rg_cell_update.argtypes = [vp]
    lib.rg_step.argtypes = [vp, dp]
    lib.rg_run.argtypes = [vp, C.c_int32, dp]
    lib.rg_step_async.argtypes = [vp]
    lib.rg_synchronize.argtypes = [vp, dp]
    lib.rg_step_timed.argtypes = [vp, dp, C.POINTER(C.c_float)]
    lib.rg_cfl_dt_noalloc.argtypes = [C.c_int32, vp, vp, vp, vp, vp, C.c_double, C.c_double, vp, vp]
    lib.rg_set_problems.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32), dp]
    lib.rg_get_problem_times.argtypes = [vp, dp, dp]
    lib.rg_run_graph.argtypes = [vp, C.c_int32]
    lib.rg_set_step_mode.argtypes = [vp, C.c_int32]
    lib.rg_grid_barrier_check.argtypes = [vp, C.c_int32]
    lib.rg_step_fwd.argtypes = [vp, C.c_int32, C.c_double, C.c_int32]
    lib.rg_step_bwd.argtypes = [vp, dp, dp]
    lib.rg_step_tlm.argtypes = [vp, C.c_int32, C.c_double, dp, dp]
    lib.rg_autotune.argtypes = [vp, C.c_int32, C.POINTER(RgLaunchShapes)]
    lib.rg_stream.argtypes = [vp, C.POINTER(vp)]
    from meshview import RgMesh3DView
    lib.rg3_create.argtypes = [C.POINTER(RgConfig), C.POINTER(vp)]
    lib.rg3_destroy.argtypes = [vp]
    lib.rg3_last_error.argtypes = [vp, C.POINTER(RgError)]
    lib.rg3_upload_mesh.argtypes = [vp, C.POINTER(RgMesh3DView)]
    for f in ("rg3_set_cells", "rg3_get_cells", "rg3_set_extensives", "rg3_get_extensives",
              "rg3_set_face_velocities", "rg3_flux", "rg3_cfl_dt", "rg3_step"):
        getattr(lib, f).argtypes = [vp, dp]
    lib.rg3_init_extensives.argtypes = [vp]
    lib.rg3_extensive_update.argtypes = [vp, C.c_double]
    lib.rg3_cell_update.argtypes = [vp]
    lib.rg3_run.argtypes = [vp, C.c_int32, dp]
    lib.rg3_step_timed.argtypes = [vp, dp, C.POINTER(C.c_float)]
    lib.rg_set_tracer_config.argtypes = [vp, C.POINTER(RgTracerConfig)]
    for f in ("rg_set_tracers", "rg_get_tracers", "rg_set_extensive_tracers", "rg_get_extensive_tracers",
              "rg_get_tracer_fluxes", "rg_get_tracer_slopes", "rg_set_tracer_fluxes"):
        getattr(lib, f).argtypes = [vp, dp]
    lib.rg_set_stickers.argtypes = [vp, C.POINTER(C.c_uint32)]
    lib.rg_set_flux_rules.argtypes = [vp, C.c_int32, C.POINTER(RgFluxRule)]
    lib.rg_set_lagrangian_updater.argtypes = [vp, C.c_int32]
    lib.rg_get_lagrangian_faces.argtypes = [vp, dp, dp]
    lib.rg_set_lagrangian_faces.argtypes = [vp, dp, dp]
    lib.rg_set_outer_box.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double]
    lib.rg_set_point_motion.argtypes = [vp, C.POINTER(RgPointMotion)]
    lib.rg_point_velocities.argtypes = [vp, dp]
    lib.rg_apply_fix.argtypes = [vp, C.c_double, dp]
    lib.rg_get_edge_velocities.argtypes = [vp, dp]
    lib.rg_get_geometry.argtypes = [vp, dp, dp, dp, dp]
    lib.rg_set_physical_geometry.argtypes = [vp, C.POINTER(RgPhysicalGeometry)]
    lib.rg_advance_begin.argtypes = [vp, dp, dp]
    lib.rg_set_launch_shapes.argtypes = [vp, C.POINTER(RgLaunchShapes)]
    lib.rg_get_launch_shapes.argtypes = [vp, C.POINTER(RgLaunchShapes)]
    _lib = lib
    return lib


class Handle:
    """One rg_handle: a simulation's device state on one GPU."""

    def __init__(self, config=None, **kw):
        self.lib = load()
        self.config = config or make_config(**kw)
        h = C.c_void_p()
        st = self.lib.rg_create(C.byref(self.config), C.byref(h))
        if st:
            raise RichError(st)
        self.h = h
        self.mesh = None

    def close(self):
        if self.h:
            self.lib.rg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st):
        if st:
            err = RgError()
            self.lib.rg_last_error(self.h, C.byref(err))
            raise RichError(st, err)

    def last_error(self):
        err = RgError()
        self.lib.rg_last_error(self.h, C.byref(err))
        return err

    # mesh / state -------------------------------------------------------
    def upload_mesh(self, mesh: PackedMesh, flags=0):
        """flags & MESH_DEVICE_GEOMETRY: only points, topology and face
        vertices are sent; volumes and CMs are computed on the device."""
        view = mesh.topology_view() if flags & MESH_DEVICE_GEOMETRY else mesh.view()
        self._check(self.lib.rg_upload_mesh(self.h, C.byref(view), flags))
        self.mesh = mesh

    def last_upload_ms(self):
        v = C.c_double()
        self.lib.rg_last_upload_ms(self.h, C.byref(v))
        return v.value

    def set_cells(self, cells):
        a = np.ascontiguousarray(cells, dtype=np.float64)
        assert a.size == 4 * self.mesh.n_cells
        self._check(self.lib.rg_set_cells(self.h, dptr(a)))

    def get_cells(self, out=None):
        out = np.empty((self.mesh.n_cells, 4)) if out is None else out
        assert out.dtype == np.float64 and out.size == 4 * self.mesh.n_cells and out.flags.c_contiguous
        self._check(self.lib.rg_get_cells(self.h, dptr(out)))
        return out

    def set_extensives(self, ext):
        a = np.ascontiguousarray(ext, dtype=np.float64)
        assert a.size == 4 * self.mesh.n_cells
        self._check(self.lib.rg_set_extensives(self.h, dptr(a)))

    def get_extensives(self, out=None):
        out = np.empty((self.mesh.n_cells, 4)) if out is None else out
        assert out.dtype == np.float64 and out.size == 4 * self.mesh.n_cells and out.flags.c_contiguous
        self._check(self.lib.rg_get_extensives(self.h, dptr(out)))
        return out

    def get_state_async(self, cells_out, ext_out):
        """Starts copying the cells and extensives into the given (pinned)
        arrays without waiting; read them after wait_state()."""
        for o in (cells_out, ext_out):
            assert o.dtype == np.float64 and o.size == 4 * self.mesh.n_cells and o.flags.c_contiguous
        self._check(self.lib.rg_get_state_async(self.h, dptr(cells_out), dptr(ext_out)))

    def wait_state(self):
        self._check(self.lib.rg_wait_state(self.h))

    def set_edge_velocities(self, ev):
        a = np.ascontiguousarray(ev, dtype=np.float64)
        assert a.size == 2 * self.mesh.n_faces
        self._check(self.lib.rg_set_edge_velocities(self.h, dptr(a)))

    def set_fluxes(self, fl):
        a = np.ascontiguousarray(fl, dtype=np.float64)
        assert a.size == 4 * self.mesh.n_faces
        self._check(self.lib.rg_set_fluxes(self.h, dptr(a)))

    def device_buffers(self):
        v = RgDeviceView()
        self._check(self.lib.rg_device_buffers(self.h, C.byref(v)))
        return v

    def stream(self):
        """The handle's CUDA stream (an integer handle), without handing out state."""
        v = C.c_void_p()
        self._check(self.lib.rg_stream(self.h, C.byref(v)))
        return v.value

    def init_extensives(self):
        self._check(self.lib.rg_init_extensives(self.h))

    # plugin operations ----------------------------------------------------
    def cfl_dt(self):
        dt = C.c_double()
        self._check(self.lib.rg_cfl_dt(self.h, C.byref(dt)))
        return dt.value

    def flux(self, dt=0.0, download=True):
        out = np.empty((self.mesh.n_faces, 4)) if download else None
        self._check(self.lib.rg_flux(self.h, C.c_double(dt), dptr(out) if download else None))
        return out

    def extensive_update(self, dt):
        self._check(self.lib.rg_extensive_update(self.h, C.c_double(dt)))

    def cell_update(self):
        self._check(self.lib.rg_cell_update(self.h))

    def step(self):
        dt = C.c_double()
        self._check(self.lib.rg_step(self.h, C.byref(dt)))
        return dt.value

    def run(self, n_steps):
        dts = np.empty(max(n_steps, 1))
        self._check(self.lib.rg_run(self.h, n_steps, dptr(dts)))
        return dts[:n_steps]

    def step_timed(self):
        """One fused step; returns (dt, [cfl, slopes, faces, update] kernel ms)."""
        dt = C.c_double()
        ms = (C.c_float * 4)()
        self._check(self.lib.rg_step_timed(self.h, C.byref(dt), ms))
        return dt.value, list(ms)

    # point motion on the device ------------------------------------------------
    def set_outer_box(self, left, right, down, up):
        self._check(self.lib.rg_set_outer_box(self.h, left, right, down, up))

    def set_point_motion(self, kind=0, edges=0, chi=0.15, eta=0.02, cold=False, correct_overshoot=False):
        """kind 0 Eulerian, 1 Lagrangian, 2 RoundCells(Lagrangian); edges 0
        StationaryBox, 1 PeriodicEdgeVelocities."""
        pm = RgPointMotion(int(kind), int(edges), chi, eta, int(cold), int(correct_overshoot))
        self._check(self.lib.rg_set_point_motion(self.h, C.byref(pm)))

    def point_velocities(self):
        out = np.empty((self.mesh.n_cells, 2))
        self._check(self.lib.rg_point_velocities(self.h, dptr(out)))
        return out

    def apply_fix(self, dt):
        out = np.empty((self.mesh.n_cells, 2))
        self._check(self.lib.rg_apply_fix(self.h, C.c_double(dt), dptr(out)))
        return out

    def edge_velocities(self):
        out = np.empty((self.mesh.n_faces, 2))
        self._check(self.lib.rg_get_edge_velocities(self.h, dptr(out)))
        return out

    def geometry(self, areas=False):
        """(volume, cm_xy of all points, cd_volume[, CacheData face areas]) of
        the mesh in use."""
        n, g = self.mesh.n_cells, self.mesh.n_ghosts
        vol, cm, cdv, ar = np.empty(n), np.empty((n + g, 2)), np.empty(n), np.empty(self.mesh.n_faces)
        self._check(self.lib.rg_get_geometry(self.h, dptr(vol), dptr(cm), dptr(cdv), dptr(ar)))
        return (vol, cm, cdv, ar) if areas else (vol, cm, cdv)

    def set_physical_geometry(self, kind=0, origin=(0.0, 0.0), direction=(0.0, 1.0)):
        """0 SlabSymmetry, 1 CylindricalSymmetry about the axis through
        origin along direction; applies from the next upload."""
        pg = RgPhysicalGeometry(int(kind), (C.c_double * 2)(*origin), (C.c_double * 2)(*direction), 0)
        self._check(self.lib.rg_set_physical_geometry(self.h, C.byref(pg)))

    def advance_begin(self, download_pv=True, out=None):
        """hdsim::TimeAdvance up to MoveMeshPoints; returns (dt, point
        velocities), the latter into `out` when given."""
        dt = C.c_double()
        pv = out if out is not None else (np.empty((self.mesh.n_cells, 2)) if download_pv else None)
        if pv is not None:
            assert pv.dtype == np.float64 and pv.size == 2 * self.mesh.n_cells and pv.flags.c_contiguous
        self._check(self.lib.rg_advance_begin(self.h, C.byref(dt), dptr(pv) if pv is not None else None))
        return dt.value, pv

    # tracers and stickers --------------------------------------------------
    def set_tracer_config(self, n_tracers=0, limited=(), entropy=-1, skip_sticker=-1, frozen_sticker=-1,
                          n_stickers=0):
        """Tracer count, the tracers in LinearGaussImproved's calc_tracers
        (indices), the "Entropy" tracer, the skip_key sticker bit and the
        HasSticker + SkipUpdate sticker bit (-1: none); n_stickers keeps
        stickers for the flux rules."""
        mask = 0
        for j in limited:
            mask |= 1 << j
        c = RgTracerConfig(n_tracers, n_stickers, mask, entropy, skip_sticker, frozen_sticker)
        self._check(self.lib.rg_set_tracer_config(self.h, C.byref(c)))
        self.n_tracers = n_tracers

    def _tr_io(self, fn, arr, cols):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        assert a.size == cols * self.mesh.n_cells
        self._check(fn(self.h, dptr(a)))

    def set_tracers(self, tr):
        self._tr_io(self.lib.rg_set_tracers, tr, self.n_tracers)

    def get_tracers(self):
        out = np.empty((self.mesh.n_cells, self.n_tracers))
        self._check(self.lib.rg_get_tracers(self.h, dptr(out)))
        return out

    def set_extensive_tracers(self, tr):
        self._tr_io(self.lib.rg_set_extensive_tracers, tr, self.n_tracers)

    def get_extensive_tracers(self):
        out = np.empty((self.mesh.n_cells, self.n_tracers))
        self._check(self.lib.rg_get_extensive_tracers(self.h, dptr(out)))
        return out

    def set_stickers(self, stickers):
        a = np.ascontiguousarray(stickers, dtype=np.uint32)
        assert a.size == self.mesh.n_cells
        self._check(self.lib.rg_set_stickers(self.h, a.ctypes.data_as(C.POINTER(C.c_uint32))))

    def tracer_fluxes(self):
        out = np.empty((self.mesh.n_faces, self.n_tracers))
        self._check(self.lib.rg_get_tracer_fluxes(self.h, dptr(out)))
        return out

    def tracer_slopes(self):
        out = np.empty((self.mesh.n_cells, 2 * self.n_tracers))
        self._check(self.lib.rg_get_tracer_slopes(self.h, dptr(out)))
        return out

    def set_flux_rules(self, rules):
        """Condition/action flux rules: rows (sequence, condition, sticker,
        action, ratchet_in[, LagrangianFlux massflux bits]); an empty list
        restores the default flux calculator."""
        a = np.asarray(rules, dtype=np.int64)
        a = a.reshape(-1, a.shape[-1] if a.size else 6)
        if a.shape[1] == 5:
            a = np.concatenate([a, np.zeros((len(a), 1), np.int64)], axis=1)
        rows = [tuple(int(x) for x in r) for r in a]
        arr = (RgFluxRule * max(len(rows), 1))(*[RgFluxRule(*r) for r in rows])
        self._check(self.lib.rg_set_flux_rules(self.h, len(rows), arr))

    def set_lagrangian_updater(self, on=True):
        """LagrangianExtensiveUpdater around SimpleExtensiveUpdater."""
        self._check(self.lib.rg_set_lagrangian_updater(self.h, 1 if on else 0))

    def lagrangian_faces(self):
        """(ws_, edge_vel_) of the last flux pass's LagrangianFlux."""
        ws, ev = np.empty(self.mesh.n_faces), np.empty(self.mesh.n_faces)
        self._check(self.lib.rg_get_lagrangian_faces(self.h, dptr(ws), dptr(ev)))
        return ws, ev

    def set_lagrangian_faces(self, ws, edge_vel):
        """LagrangianFlux's ws_ / edge_vel_ from the host (with set_fluxes)."""
        a = np.ascontiguousarray(ws, dtype=np.float64)
        b = np.ascontiguousarray(edge_vel, dtype=np.float64)
        assert a.size == b.size == self.mesh.n_faces
        self._check(self.lib.rg_set_lagrangian_faces(self.h, dptr(a), dptr(b)))

    # batches ---------------------------------------------------------------
    def set_problems(self, offsets, gammas):
        """Declare the uploaded mesh a batch (problem p owns cells
        offsets[p]:offsets[p+1]) with per-problem gamma."""
        off = np.ascontiguousarray(offsets, dtype=np.int32)
        g = np.ascontiguousarray(gammas, dtype=np.float64)
        assert off.size == g.size + 1
        self.n_problems = int(g.size)
        self._check(self.lib.rg_set_problems(self.h, g.size, off.ctypes.data_as(C.POINTER(C.c_int32)),
                                             dptr(g)))

    def problem_times(self):
        t = np.empty(self.n_problems)
        d = np.empty(self.n_problems)
        self._check(self.lib.rg_get_problem_times(self.h, dptr(t), dptr(d)))
        return t, d

    def run_graph(self, n_steps):
        self._check(self.lib.rg_run_graph(self.h, n_steps))

    def set_step_mode(self, mode):
        """STEP_PER_PHASE (0) or STEP_PERSISTENT (1): a batch run in one
        cooperative launch."""
        self._check(self.lib.rg_set_step_mode(self.h, mode))

    def grid_barrier_check(self, missing_blocks=0):
        """The persistent form's grid barrier alone, expecting missing_blocks
        more blocks than run (RG_ERR_TIMEOUT after its bounded wait)."""
        self._check(self.lib.rg_grid_barrier_check(self.h, missing_blocks))

    def step_async(self):
        self._check(self.lib.rg_step_async(self.h))

    def synchronize(self):
        dt = C.c_double()
        self._check(self.lib.rg_synchronize(self.h, C.byref(dt)))
        return dt.value

    # differentiation (fixed dt, periodic LinearGaussImproved + Hllc, FP64)
    def step_fwd(self, n_steps, dt, checkpoint_every=20):
        """n_steps fixed-dt steps from the handle's cells, recorded for step_bwd."""
        self._check(self.lib.rg_step_fwd(self.h, n_steps, dt, checkpoint_every))

    def step_bwd(self, cells_bar):
        """dL/d(initial cells) from dL/d(final cells) of the last step_fwd."""
        a = np.ascontiguousarray(cells_bar, dtype=np.float64)
        assert a.size == 4 * self.mesh.n_cells
        out = np.empty((self.mesh.n_cells, 4))
        self._check(self.lib.rg_step_bwd(self.h, dptr(a), dptr(out)))
        return out

    def step_tlm(self, n_steps, dt, dcells0):
        """Tangent of the final cells along dcells0 (the handle ends at W_n)."""
        a = np.ascontiguousarray(dcells0, dtype=np.float64)
        assert a.size == 4 * self.mesh.n_cells
        out = np.empty((self.mesh.n_cells, 4))
        self._check(self.lib.rg_step_tlm(self.h, n_steps, dt, dptr(a), dptr(out)))
        return out

    # launch shapes of the per-step kernels
    @staticmethod
    def _shapes_dict(r):
        return {k: {"block": r.block[i], "max_blocks": r.max_blocks[i], "variant": r.variant[i], "ms": r.ms[i]}
                for i, k in enumerate(KERNELS)}

    def autotune(self, reps=5):
        """Times every candidate launch shape per kernel and keeps the fastest."""
        r = RgLaunchShapes()
        self._check(self.lib.rg_autotune(self.h, reps, C.byref(r)))
        return self._shapes_dict(r)

    def launch_shapes(self):
        r = RgLaunchShapes()
        self._check(self.lib.rg_get_launch_shapes(self.h, C.byref(r)))
        return self._shapes_dict(r)

    def set_launch_shapes(self, shapes):
        """shapes: {kernel: (block, max_blocks[, variant])} for some of KERNELS."""
        r = RgLaunchShapes()
        self._check(self.lib.rg_get_launch_shapes(self.h, C.byref(r)))
        for k, shape in shapes.items():
            i = KERNELS.index(k)
            r.block[i], r.max_blocks[i] = shape[0], shape[1]
            r.variant[i] = shape[2] if len(shape) > 2 else 0
        self._check(self.lib.rg_set_launch_shapes(self.h, C.byref(r)))


class Handle3:
    """A 3D first-order handle (rg3_*): HDSim3D's step on a packed 3D mesh.
    Cells (n, 5) {density, pressure, vx, vy, vz}; extensives and fluxes (n, 5)
    {mass, px, py, pz, energy}."""

    def __init__(self, config=None, **kw):
        self.lib = load()
        self.cfg = config or make_config(**kw)
        h = C.c_void_p()
        st = self.lib.rg3_create(C.byref(self.cfg), C.byref(h))
        if st:
            raise RichError(st)
        self.h = h
        self.mesh = None

    def close(self):
        if getattr(self, "h", None):
            self.lib.rg3_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st):
        if st:
            err = RgError()
            self.lib.rg3_last_error(self.h, C.byref(err))
            raise RichError(st, err)

    def upload_mesh(self, mesh):
        self.mesh = mesh
        self._check(self.lib.rg3_upload_mesh(self.h, C.byref(mesh.view())))

    def _put(self, fn, a, rows):
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.size == 5 * rows
        self._check(fn(self.h, dptr(a)))

    def _get(self, fn, rows):
        out = np.empty((rows, 5))
        self._check(fn(self.h, dptr(out)))
        return out

    def set_cells(self, c):
        self._put(self.lib.rg3_set_cells, c, self.mesh.n_cells)

    def get_cells(self):
        return self._get(self.lib.rg3_get_cells, self.mesh.n_cells)

    def set_extensives(self, e):
        self._put(self.lib.rg3_set_extensives, e, self.mesh.n_cells)

    def get_extensives(self):
        return self._get(self.lib.rg3_get_extensives, self.mesh.n_cells)

    def set_face_velocities(self, fv):
        if fv is None:
            self._check(self.lib.rg3_set_face_velocities(self.h, None))
            return
        a = np.ascontiguousarray(fv, dtype=np.float64)
        assert a.size == 3 * self.mesh.n_faces
        self._check(self.lib.rg3_set_face_velocities(self.h, dptr(a)))

    def init_extensives(self):
        self._check(self.lib.rg3_init_extensives(self.h))

    def cfl_dt(self):
        v = C.c_double()
        self._check(self.lib.rg3_cfl_dt(self.h, C.byref(v)))
        return v.value

    def flux(self, download=True):
        if not download:
            self._check(self.lib.rg3_flux(self.h, None))
            return None
        return self._get(self.lib.rg3_flux, self.mesh.n_faces)

    def extensive_update(self, dt):
        self._check(self.lib.rg3_extensive_update(self.h, dt))

    def cell_update(self):
        self._check(self.lib.rg3_cell_update(self.h))

    def step(self):
        v = C.c_double()
        self._check(self.lib.rg3_step(self.h, C.byref(v)))
        return v.value

    def step_timed(self):
        """One step; returns (dt, [cfl, faces, update] kernel ms)."""
        v = C.c_double()
        k = (C.c_float * 3)()
        self._check(self.lib.rg3_step_timed(self.h, C.byref(v), k))
        return v.value, list(k)

    def run(self, n_steps):
        out = np.empty(n_steps)
        self._check(self.lib.rg3_run(self.h, n_steps, dptr(out) if n_steps else None))
        return out
