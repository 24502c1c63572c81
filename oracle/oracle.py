"""ctypes binding of the C parity oracle (rich_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, as the checker.  Never used by the product.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "liboracle.so")


def build(force=False):
    """Compile rich_oracle.c with gcc (no FMA contraction)."""
    src = os.path.join(HERE, "rich_oracle.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "rich_oracle.h"))):
        return LIB
    subprocess.check_call(["gcc", "-O2", "-std=c99", "-ffp-contract=off", "-fno-fast-math",
                           "-fPIC", "-shared", "-Wall", "-I" + os.path.join(ROOT, "include"),
                           src, "-o", LIB + ".tmp", "-lm"])
    os.replace(LIB + ".tmp", LIB)
    return LIB


class RoError(C.Structure):
    _fields_ = [("status", C.c_int32), ("phase", C.c_int32), ("index", C.c_int64),
                ("value", C.c_double)]


class RoLgiParams(C.Structure):
    _fields_ = [("ghost_kind", C.c_int32), ("slf", C.c_int32), ("delta_v", C.c_double),
                ("theta", C.c_double), ("delta_p", C.c_double)]


class OracleError(RuntimeError):
    def __init__(self, err):
        self.status, self.phase, self.index, self.value = err.status, err.phase, err.index, err.value
        super().__init__(f"oracle status {err.status} phase {err.phase} index {err.index} value {err.value}")


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
    return _lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a if shape is None else a.reshape(shape)


def _check(st, err):
    if st:
        raise OracleError(err)


def lgi_params(ghost_kind=0, slf=1, delta_v=0.2, theta=0.5, delta_p=0.7):
    return RoLgiParams(ghost_kind, slf, delta_v, theta, delta_p)


def cfl(mesh, cells, ev, gamma, cfl_number=0.3):
    cells, ev = _f64(cells), _f64(ev)
    dt = C.c_double()
    err = RoError()
    _check(lib().ro_cfl(C.byref(mesh.view()), _d(cells), _d(ev), C.c_double(gamma),
                        C.c_double(cfl_number), C.byref(dt), C.byref(err)), err)
    return dt.value


def simple_flux(mesh, cells, ev, gamma):
    out = np.zeros((mesh.n_faces, 4))
    err = RoError()
    cells, ev = _f64(cells), _f64(ev)
    _check(lib().ro_simple_flux(C.byref(mesh.view()), _d(cells), _d(ev), C.c_double(gamma),
                                _d(out), C.byref(err)), err)
    return out


def lgi(mesh, cells, gamma, lp):
    slopes = np.zeros((mesh.n_cells, 8))
    interp = np.zeros((mesh.n_faces, 8))
    err = RoError()
    cells = _f64(cells)
    _check(lib().ro_lgi(C.byref(mesh.view()), _d(cells), C.c_double(gamma), C.byref(lp),
                        _d(slopes), _d(interp), C.byref(err)), err)
    return slopes, interp


def modular_flux(mesh, cells, ev, gamma, lp):
    out = np.zeros((mesh.n_faces, 4))
    err = RoError()
    cells, ev = _f64(cells), _f64(ev)
    _check(lib().ro_modular_flux(C.byref(mesh.view()), _d(cells), _d(ev), C.c_double(gamma),
                                 C.byref(lp), _d(out), C.byref(err)), err)
    return out


def extensive_update(mesh, fluxes, dt, ext):
    ext = _f64(ext).copy()
    err = RoError()
    fluxes = _f64(fluxes)
    _check(lib().ro_extensive_update(C.byref(mesh.view()), _d(fluxes), C.c_double(dt), _d(ext),
                                     C.byref(err)), err)
    return ext


def cell_update(mesh, ext, gamma):
    out = np.zeros((mesh.n_cells, 4))
    err = RoError()
    ext = _f64(ext)
    _check(lib().ro_cell_update(C.byref(mesh.view()), _d(ext), C.c_double(gamma), _d(out),
                                C.byref(err)), err)
    return out


def init_extensives(mesh, cells, gamma):
    out = np.zeros((mesh.n_cells, 4))
    cells = _f64(cells)
    lib().ro_init_extensives(C.byref(mesh.view()), _d(cells), C.c_double(gamma), _d(out))
    return out


def step(mesh, cells, ext, ev, gamma, cfl_number=0.3, order=2, lp=None, heun=False, areas=None):
    """One fixed-mesh hot-path pass (hdsim::TimeAdvance, or TimeAdvance2Heun
    with heun=True); returns (cells, ext, dt).  areas: CacheData face areas
    of a non-slab PhysicalGeometry (the mesh's cd_volume holds its volumes)."""
    cells = _f64(cells).copy()
    ext = _f64(ext).copy()
    ev = _f64(ev)
    lp = lp or lgi_params()
    dt = C.c_double()
    err = RoError()
    if areas is not None:
        assert not heun
        _check(lib().ro_step_areas(C.byref(mesh.view()), _d(cells), _d(ext), _d(ev), C.c_double(gamma),
                                   C.c_double(cfl_number), C.c_int(order), C.byref(lp), _d(_f64(areas)),
                                   C.byref(dt), C.byref(err)), err)
        return cells, ext, dt.value
    fn = lib().ro_step_heun if heun else lib().ro_step
    _check(fn(C.byref(mesh.view()), _d(cells), _d(ext), _d(ev), C.c_double(gamma),
              C.c_double(cfl_number), C.c_int(order), C.byref(lp), C.byref(dt), C.byref(err)), err)
    return cells, ext, dt.value


def run(mesh, cells, ext, ev, gamma, steps, cfl_number=0.3, order=2, lp=None, heun=False, areas=None):
    dts = []
    for _ in range(steps):
        cells, ext, dt = step(mesh, cells, ext, ev, gamma, cfl_number, order, lp, heun, areas)
        dts.append(dt)
    return cells, ext, np.array(dts)


def run_fixed_dt(mesh, cells, gamma, steps, dt, lp=None):
    """hdsim::TimeAdvance with a fixed dt on a mesh at rest, composed from
    the plugin operations (init_extensives, ModularFluxCalculator with
    LinearGaussImproved, SimpleExtensiveUpdater, SimpleCellUpdater); returns
    (cells, ext).  The map the adjoint differentiates."""
    lp = lp or lgi_params(1)
    ev = np.zeros((mesh.n_faces, 2))
    ext = init_extensives(mesh, cells, gamma)
    for _ in range(steps):
        fl = modular_flux(mesh, cells, ev, gamma, lp)
        ext = extensive_update(mesh, fl, dt, ext)
        cells = cell_update(mesh, ext, gamma)
    return cells, ext


# ---------------------------------------------------------------- condition/action flux schemes

class RoFluxRule(C.Structure):
    _fields_ = [("seq", C.c_int32), ("cond", C.c_int32), ("sticker", C.c_int32), ("action", C.c_int32),
                ("in_", C.c_int32), ("massflux", C.c_int32)]


def _rules(rows):
    """Rule rows (sequence, condition, sticker, action, ratchet in[, LagrangianFlux massflux bits])."""
    rows = np.atleast_2d(np.asarray(rows, dtype=np.int32))
    if rows.shape[1] == 5:
        rows = np.concatenate([rows, np.zeros((len(rows), 1), np.int32)], axis=1)
    arr = (RoFluxRule * len(rows))(*[RoFluxRule(*map(int, r)) for r in rows])
    return arr, len(rows)


def _stickers(st):
    if st is None:
        return None, None
    st = np.ascontiguousarray(st, dtype=np.uint32)
    return st, st.ctypes.data_as(C.POINTER(C.c_uint32))


def cas_flux(mesh, cells, ev, gamma, order, lp, rules, stickers=None, lagrangian=False):
    """Fluxes of ConditionActionSequence (order 1) / ConditionActionSequence2
    (order 2, LinearGaussImproved face states) with the given rule rows; with
    lagrangian=True also LagrangianFlux's per-face ws_ and edge_vel_."""
    out = np.zeros((mesh.n_faces, 4))
    ws, lev = np.zeros(mesh.n_faces), np.zeros(mesh.n_faces)
    arr, nr = _rules(rules)
    st, stp = _stickers(stickers)
    err = RoError()
    _check(lib().ro_cas_flux(C.byref(mesh.view()), _d(_f64(cells)), _d(_f64(ev)), C.c_double(gamma), C.c_int(order),
                             C.byref(lp), arr, C.c_int(nr), stp, _d(out), _d(ws), _d(lev), C.byref(err)), err)
    return (out, ws, lev) if lagrangian else out


def lagrangian_update(mesh, ws, lag_ev, dt, ext, areas=None):
    """LagrangianExtensiveUpdater's correction of extensives already updated by
    SimpleExtensiveUpdater (LagrangianExtensiveUpdater.cpp:8-80)."""
    out = _f64(ext).copy()
    lib().ro_lagrangian_update(C.byref(mesh.view()), _d(_f64(ws)), _d(_f64(lag_ev)), C.c_double(dt),
                               None if areas is None else _d(_f64(areas)), _d(out))
    return out


def run_cas(mesh, cells, ext, ev, gamma, steps, order, lp, rules, stickers=None, frozen_mask=0, cfl_number=0.3,
            lagrangian_update=False):
    cells, ext = _f64(cells).copy(), _f64(ext).copy()
    arr, nr = _rules(rules)
    st, stp = _stickers(stickers)
    dts = []
    for _ in range(steps):
        dt, err = C.c_double(), RoError()
        _check(lib().ro_step_cas(C.byref(mesh.view()), _d(cells), _d(ext), _d(_f64(ev)), C.c_double(gamma),
                                 C.c_double(cfl_number), C.c_int(order), C.byref(lp), arr, C.c_int(nr), stp,
                                 C.c_uint32(frozen_mask), C.c_int(1 if lagrangian_update else 0), C.byref(dt),
                                 C.byref(err)), err)
        dts.append(dt.value)
    return cells, ext, np.array(dts)


# ---------------------------------------------------------------- geometry and point motion

class RoMotion(C.Structure):
    _fields_ = [("kind", C.c_int32), ("edges", C.c_int32), ("chi", C.c_double), ("eta", C.c_double),
                ("cold", C.c_int32), ("correct_overshoot", C.c_int32), ("box", C.c_double * 4)]


def motion(kind=0, edges=0, chi=0.15, eta=0.02, cold=0, correct_overshoot=0, box=(0, 0, 0, 0)):
    """kind 0 Eulerian, 1 Lagrangian, 2 RoundCells(Lagrangian); edges 0
    StationaryBox, 1 PeriodicEdgeVelocities; box {left, right, down, up}."""
    return RoMotion(int(kind), int(edges), chi, eta, int(cold), int(correct_overshoot), (C.c_double * 4)(*box))


def _setup_geo():
    L = lib()
    if getattr(L, "_rogeo", False):
        return L
    dp = C.POINTER(C.c_double)
    mp = C.POINTER(RoMotion)
    L.ro_cell_geometry.restype = None
    L.ro_cell_geometry.argtypes = [C.c_void_p, C.c_int, dp, dp, dp, dp]
    for f in ("ro_point_velocities", "ro_edge_velocities", "ro_apply_fix"):
        getattr(L, f).restype = None
    L.ro_point_velocities.argtypes = [C.c_void_p, dp, C.c_double, mp, dp]
    L.ro_apply_fix.argtypes = [C.c_void_p, dp, C.c_double, mp, C.c_double, dp]
    L.ro_edge_velocities.argtypes = [C.c_void_p, mp, dp, dp]
    L.ro_cyl_geometry.restype = None
    L.ro_cyl_geometry.argtypes = [C.c_void_p, dp, dp, dp, dp]
    L.ro_extensive_update_areas.restype = None
    L.ro_extensive_update_areas.argtypes = [C.c_void_p, dp, dp, C.c_double, dp]
    L._rogeo = True
    return L


def cell_geometry(mesh, ghost_kind, box):
    """(volume, cm_xy of all points, cd_volume) from points and face vertices."""
    n, g = mesh.n_cells, mesh.n_ghosts
    vol, cm, cdv = np.zeros(n), np.zeros((n + g, 2)), np.zeros(n)
    b = _f64(box)
    _setup_geo().ro_cell_geometry(C.byref(mesh.view()), ghost_kind, _d(b), _d(vol), _d(cm), _d(cdv))
    return vol, cm, cdv


def cyl_geometry(mesh, origin, direction):
    """CylindricalSymmetry's CacheData face areas and cell volumes."""
    areas, vols = np.zeros(mesh.n_faces), np.zeros(mesh.n_cells)
    L = _setup_geo()
    L.ro_cyl_geometry(C.byref(mesh.view()), _d(_f64(origin)), _d(_f64(direction)), _d(areas), _d(vols))
    return areas, vols


def extensive_update_areas(mesh, fluxes, areas, dt, ext):
    ext = _f64(ext).copy()
    _setup_geo().ro_extensive_update_areas(C.byref(mesh.view()), _d(_f64(fluxes)), _d(_f64(areas)), dt, _d(ext))
    return ext


def point_velocities(mesh, cells, gamma, mo):
    pv = np.zeros((mesh.n_cells, 2))
    _setup_geo().ro_point_velocities(C.byref(mesh.view()), _d(_f64(cells)), gamma, C.byref(mo), _d(pv))
    return pv


def apply_fix(mesh, cells, gamma, mo, dt, pv):
    pv = _f64(pv).copy()
    _setup_geo().ro_apply_fix(C.byref(mesh.view()), _d(_f64(cells)), gamma, C.byref(mo), dt, _d(pv))
    return pv


def edge_velocities(mesh, mo, pv):
    ev = np.zeros((mesh.n_faces, 2))
    _setup_geo().ro_edge_velocities(C.byref(mesh.view()), C.byref(mo), _d(_f64(pv)), _d(ev))
    return ev


# ---------------------------------------------------------------- tracers and stickers

class RoTracers(C.Structure):
    _fields_ = [("n", C.c_int32), ("limited", C.c_uint32), ("entropy", C.c_int32),
                ("skip_mask", C.c_uint32), ("frozen_mask", C.c_uint32),
                ("stickers", C.POINTER(C.c_uint32))]


class TracerSetup:
    """Tracer count, calc_tracers mask, "Entropy" index, skip_key and
    SkipUpdate sticker bits (-1: none) and the per-cell sticker masks."""

    def __init__(self, n, limited=0, entropy=-1, skip_sticker=-1, frozen_sticker=-1, stickers=None):
        self.n, self.limited, self.entropy = n, limited, entropy
        self.skip_sticker, self.frozen_sticker = skip_sticker, frozen_sticker
        self.stickers = None if stickers is None else np.ascontiguousarray(stickers, dtype=np.uint32)

    def c(self):
        st = None if self.stickers is None else self.stickers.ctypes.data_as(C.POINTER(C.c_uint32))
        return RoTracers(self.n, self.limited, self.entropy,
                         (1 << self.skip_sticker) if self.skip_sticker >= 0 else 0,
                         (1 << self.frozen_sticker) if self.frozen_sticker >= 0 else 0, st)


def _setup_tr():
    L = lib()
    if getattr(L, "_rotr", False):
        return L
    dp = C.POINTER(C.c_double)
    L.ro_extensive_update_tr.restype = None
    L.ro_extensive_update_tr.argtypes = [C.c_void_p, dp, C.c_int, C.c_double, dp]
    L.ro_init_extensives_tr.restype = None
    L.ro_init_extensives_tr.argtypes = [C.c_void_p, dp, dp, C.c_int, dp]
    L._rotr = True
    return L


def lgi_tr(mesh, cells, tr, gamma, lp, ts):
    n, N, E = ts.n, mesh.n_cells, mesh.n_faces
    slopes, interp = np.zeros((N, 8)), np.zeros((E, 8))
    tsl, tip = np.zeros((N, 2 * n)), np.zeros((E, 2 * n))
    cells, tr = _f64(cells), _f64(tr)
    err, tc = RoError(), ts.c()
    _check(_setup_tr().ro_lgi_tr(C.byref(mesh.view()), _d(cells), _d(tr), C.c_double(gamma), C.byref(lp),
                                 C.byref(tc), _d(slopes), _d(interp), _d(tsl), _d(tip), C.byref(err)), err)
    return slopes, interp, tsl, tip


def flux_tr(mesh, cells, tr, ev, gamma, order, lp, ts):
    """(fluxes, tracer fluxes) of SimpleFluxCalculator (order 1) or
    ModularFluxCalculator with LinearGaussImproved (order 2)."""
    E = mesh.n_faces
    fl, tfl = np.zeros((E, 4)), np.zeros((E, max(ts.n, 1)))
    cells, tr, ev = _f64(cells), _f64(tr), _f64(ev)
    err, tc = RoError(), ts.c()
    L = _setup_tr()
    if order == 1:
        st = L.ro_simple_flux_tr(C.byref(mesh.view()), _d(cells), _d(tr), _d(ev), C.c_double(gamma), C.byref(tc),
                                 _d(fl), _d(tfl), C.byref(err))
    else:
        st = L.ro_modular_flux_tr(C.byref(mesh.view()), _d(cells), _d(tr), _d(ev), C.c_double(gamma), C.byref(lp),
                                  C.byref(tc), _d(fl), _d(tfl), C.byref(err))
    _check(st, err)
    return fl, tfl[:, :ts.n]


def extensive_update_tr(mesh, tfluxes, dt, tr_ext):
    tr_ext = _f64(tr_ext).copy()
    nt = tr_ext.shape[1]
    _setup_tr().ro_extensive_update_tr(C.byref(mesh.view()), _d(_f64(tfluxes)), nt, dt, _d(tr_ext))
    return tr_ext


def cell_update_tr(mesh, ext, tr_ext, old_cells, old_tr, gamma, ts):
    """SimpleCellUpdater with tracers; returns (cells, tracers, extensive tracers)."""
    N = mesh.n_cells
    cells, tr = np.zeros((N, 4)), np.zeros((N, ts.n))
    tr_ext = _f64(tr_ext).copy()
    err, tc = RoError(), ts.c()
    _check(_setup_tr().ro_cell_update_tr(C.byref(mesh.view()), _d(_f64(ext)), _d(tr_ext), _d(_f64(old_cells)),
                                         _d(_f64(old_tr)), C.c_double(gamma), C.byref(tc), _d(cells), _d(tr),
                                         C.byref(err)), err)
    return cells, tr, tr_ext


def init_extensives_tr(mesh, cells, tr):
    tr = _f64(tr)
    out = np.zeros_like(tr)
    _setup_tr().ro_init_extensives_tr(C.byref(mesh.view()), _d(_f64(cells)), _d(tr), tr.shape[1], _d(out))
    return out


def run_tr(mesh, cells, ext, tr, tr_ext, ev, gamma, steps, ts, cfl_number=0.3, order=2, lp=None, heun=False):
    """hdsim::TimeAdvance (TimeAdvance2Heun with heun) steps with tracers on a
    fixed mesh; returns (cells, ext, tracers, extensive tracers, dts)."""
    cells, ext = _f64(cells).copy(), _f64(ext).copy()
    tr, tr_ext = _f64(tr).copy(), _f64(tr_ext).copy()
    ev = _f64(ev)
    lp = lp or lgi_params()
    L = _setup_tr()
    dts = []
    for _ in range(steps):
        dt, err, tc = C.c_double(), RoError(), ts.c()
        fn = L.ro_step_heun_tr if heun else L.ro_step_tr
        _check(fn(C.byref(mesh.view()), _d(cells), _d(ext), _d(tr), _d(tr_ext), _d(ev), C.c_double(gamma),
                  C.c_double(cfl_number), C.c_int(order), C.byref(lp), C.byref(tc), C.byref(dt), C.byref(err)), err)
        dts.append(dt.value)
    return cells, ext, tr, tr_ext, np.array(dts)


def cas_flux_tr(mesh, cells, tr, ev, gamma, order, lp, rules, ts, lagrangian=False):
    """(fluxes, tracer fluxes[, ws_, edge_vel_]) of the condition/action flux
    calculators with tracers; the stickers come from ts."""
    E = mesh.n_faces
    fl, tfl = np.zeros((E, 4)), np.zeros((E, max(ts.n, 1)))
    ws, lev = np.zeros(E), np.zeros(E)
    arr, nr = _rules(rules)
    err, tc = RoError(), ts.c()
    _check(_setup_tr().ro_cas_flux_tr(C.byref(mesh.view()), _d(_f64(cells)), _d(_f64(tr)), _d(_f64(ev)),
                                      C.c_double(gamma), C.c_int(order), C.byref(lp), C.byref(tc), arr, C.c_int(nr),
                                      tc.stickers, _d(fl), _d(tfl), _d(ws), _d(lev), C.byref(err)), err)
    return (fl, tfl[:, :ts.n], ws, lev) if lagrangian else (fl, tfl[:, :ts.n])


def lagrangian_update_tr(mesh, ws, lag_ev, dt, ext, tr_ext):
    """LagrangianExtensiveUpdater's factor on the extensives and the extensive
    tracers (already updated by SimpleExtensiveUpdater)."""
    ext, tr_ext = _f64(ext).copy(), _f64(tr_ext).copy()
    _setup_tr().ro_lagrangian_update_tr(C.byref(mesh.view()), _d(_f64(ws)), _d(_f64(lag_ev)), C.c_double(dt), None,
                                        _d(ext), _d(tr_ext), C.c_int(tr_ext.shape[1]))
    return ext, tr_ext


def run_cas_tr(mesh, cells, ext, tr, tr_ext, ev, gamma, steps, order, lp, rules, ts, cfl_number=0.3,
               lagrangian_update=False):
    """hdsim::TimeAdvance steps with a condition/action flux calculator and
    tracers on a fixed mesh; returns (cells, ext, tracers, extensive tracers, dts)."""
    cells, ext = _f64(cells).copy(), _f64(ext).copy()
    tr, tr_ext = _f64(tr).copy(), _f64(tr_ext).copy()
    arr, nr = _rules(rules)
    L = _setup_tr()
    dts = []
    for _ in range(steps):
        dt, err, tc = C.c_double(), RoError(), ts.c()
        _check(L.ro_step_cas_tr(C.byref(mesh.view()), _d(cells), _d(ext), _d(tr), _d(tr_ext), _d(_f64(ev)),
                                C.c_double(gamma), C.c_double(cfl_number), C.c_int(order), C.byref(lp), arr,
                                C.c_int(nr), C.byref(tc), C.c_int(1 if lagrangian_update else 0), C.byref(dt),
                                C.byref(err)), err)
        dts.append(dt.value)
    return cells, ext, tr, tr_ext, np.array(dts)


# ---------------------------------------------------------------- 3D first-order path

def _setup3():
    L = lib()
    if getattr(L, "_ro3", False):
        return L
    from meshview import RgMesh3DView
    m3 = C.POINTER(RgMesh3DView)
    dp = C.POINTER(C.c_double)
    L.ro3_init_extensives.argtypes = [m3, dp, C.c_double, dp]
    L.ro3_init_extensives.restype = None
    L.ro3_cfl.argtypes = [m3, dp, C.c_double, C.c_double]
    L.ro3_cfl.restype = C.c_double
    L.ro3_flux.argtypes = [m3, dp, dp, C.c_double, dp, C.POINTER(RoError)]
    L.ro3_extensive_update.argtypes = [m3, dp, C.c_double, dp]
    L.ro3_extensive_update.restype = None
    L.ro3_cell_update.argtypes = [m3, dp, C.c_double, dp, C.POINTER(RoError)]
    L.ro3_step.argtypes = [m3, dp, dp, C.c_double, C.c_double, dp, C.POINTER(RoError)]
    L._ro3 = True
    return L


def init_extensives3(mesh, cells, gamma):
    out = np.zeros((mesh.n_cells, 5))
    cells = _f64(cells)
    _setup3().ro3_init_extensives(C.byref(mesh.view()), _d(cells), gamma, _d(out))
    return out


def cfl3(mesh, cells, gamma, cfl_number=0.3):
    cells = _f64(cells)
    return _setup3().ro3_cfl(C.byref(mesh.view()), _d(cells), gamma, cfl_number)


def flux3(mesh, cells, gamma, face_velocity=None):
    out = np.zeros((mesh.n_faces, 5))
    err = RoError()
    cells = _f64(cells)
    fv = None if face_velocity is None else _d(_f64(face_velocity))
    _check(_setup3().ro3_flux(C.byref(mesh.view()), _d(cells), fv, gamma, _d(out), C.byref(err)), err)
    return out


def extensive_update3(mesh, fluxes, dt, ext):
    ext = _f64(ext).copy()
    fluxes = _f64(fluxes)
    _setup3().ro3_extensive_update(C.byref(mesh.view()), _d(fluxes), dt, _d(ext))
    return ext


def cell_update3(mesh, ext, gamma):
    out = np.zeros((mesh.n_cells, 5))
    err = RoError()
    ext = _f64(ext)
    _check(_setup3().ro3_cell_update(C.byref(mesh.view()), _d(ext), gamma, _d(out), C.byref(err)), err)
    return out


def run3(mesh, cells, ext, gamma, steps, cfl_number=0.3):
    """HDSim3D::timeAdvance steps on a fixed mesh; returns (cells, ext, dts)."""
    cells = _f64(cells).copy()
    ext = _f64(ext).copy()
    L = _setup3()
    dts = []
    for _ in range(steps):
        dt = C.c_double()
        err = RoError()
        _check(L.ro3_step(C.byref(mesh.view()), _d(cells), _d(ext), gamma, cfl_number, C.byref(dt), C.byref(err)),
               err)
        dts.append(dt.value)
    return cells, ext, np.array(dts)
