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


def step(mesh, cells, ext, ev, gamma, cfl_number=0.3, order=2, lp=None, heun=False):
    """One fixed-mesh hot-path pass (hdsim::TimeAdvance, or TimeAdvance2Heun
    with heun=True); returns (cells, ext, dt)."""
    cells = _f64(cells).copy()
    ext = _f64(ext).copy()
    ev = _f64(ev)
    lp = lp or lgi_params()
    dt = C.c_double()
    err = RoError()
    fn = lib().ro_step_heun if heun else lib().ro_step
    _check(fn(C.byref(mesh.view()), _d(cells), _d(ext), _d(ev), C.c_double(gamma),
              C.c_double(cfl_number), C.c_int(order), C.byref(lp), C.byref(dt), C.byref(err)), err)
    return cells, ext, dt.value


def run(mesh, cells, ext, ev, gamma, steps, cfl_number=0.3, order=2, lp=None, heun=False):
    dts = []
    for _ in range(steps):
        cells, ext, dt = step(mesh, cells, ext, ev, gamma, cfl_number, order, lp, heun)
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
