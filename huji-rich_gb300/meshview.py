"""ctypes mirror of ``rg_mesh_view`` / ``rg_config`` (include/rich_gb300.h) and a
numpy-backed packed-mesh container shared by the library binding
(``richgpu.py``), the workload generator (``synthetic.py``) and the tests."""
import ctypes as C

import numpy as np

MESH_FIELDS = ("point_xy", "cm_xy", "volume", "cd_volume", "ghost_source", "ghost_face",
               "face_cells", "face_vertices", "cell_face_offset", "cell_faces")
_DTYPES = {"point_xy": np.float64, "cm_xy": np.float64, "volume": np.float64,
           "cd_volume": np.float64, "ghost_source": np.int32, "ghost_face": np.int32,
           "face_cells": np.int32, "face_vertices": np.float64,
           "cell_face_offset": np.int32, "cell_faces": np.int32}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class RgMeshView(C.Structure):
    _fields_ = [("n_cells", C.c_int32), ("n_ghosts", C.c_int32), ("n_faces", C.c_int32),
                ("reserved", C.c_int32),
                ("point_xy", _dp), ("cm_xy", _dp), ("volume", _dp), ("cd_volume", _dp),
                ("ghost_source", _ip), ("ghost_face", _ip), ("face_cells", _ip),
                ("face_vertices", _dp), ("cell_face_offset", _ip), ("cell_faces", _ip)]


class RgConfig(C.Structure):
    _fields_ = [("gamma", C.c_double), ("cfl", C.c_double), ("order", C.c_int32),
                ("ghost_kind", C.c_int32), ("slope_limiter", C.c_int32), ("precision", C.c_int32),
                ("delta_v", C.c_double), ("theta", C.c_double), ("delta_p", C.c_double),
                ("device", C.c_int32), ("time_integrator", C.c_int32)]


class RgError(C.Structure):
    _fields_ = [("status", C.c_int32), ("phase", C.c_int32), ("index", C.c_int64),
                ("value", C.c_double)]


GHOST_RIGID_WALL = 0
GHOST_PERIODIC = 1
FP64 = 0
FP32_MIXED = 1

STATUS_NAMES = {0: "RG_OK", 1: "RG_ERR_INVALID_ARGUMENT", 2: "RG_ERR_CUDA", 3: "RG_ERR_NOT_READY",
                4: "RG_ERR_OUT_OF_MEMORY", 10: "RG_ERR_NEGATIVE_DENSITY",
                11: "RG_ERR_NEGATIVE_ENERGY", 12: "RG_ERR_HLLC_NAN",
                13: "RG_ERR_HLLC_WAVE_SPEEDS", 14: "RG_ERR_SINGULAR_MATRIX",
                15: "RG_ERR_TOO_MANY_NEIGHBORS", 16: "RG_ERR_TIMEOUT"}

# Messages of the reference's UniversalError for each physical failure.
REFERENCE_MESSAGES = {10: "Negative density", 11: "Negative thermal energy",
                      12: "Hllc::Solved entered with nan",
                      13: "Invalid wave speeds in hllc solver", 14: "Singular matrix",
                      15: "Cell has too many neighbors"}


TIME_ADVANCE = 0
TIME_ADVANCE_HEUN = 1


def make_config(gamma=5.0 / 3.0, cfl=0.3, order=2, ghost_kind=GHOST_RIGID_WALL, slope_limiter=1,
                precision=FP64, delta_v=0.2, theta=0.5, delta_p=0.7, device=0, time_integrator=TIME_ADVANCE):
    return RgConfig(gamma, cfl, order, ghost_kind, slope_limiter, precision, delta_v, theta,
                    delta_p, device, time_integrator)


class PackedMesh:
    """Packed tessellation: numpy arrays laid out as rg_mesh_view describes."""

    def __init__(self, **arrays):
        for k in MESH_FIELDS:
            a = np.ascontiguousarray(arrays[k], dtype=_DTYPES[k])
            setattr(self, k, a)
        self.n_cells = int(self.volume.shape[0])
        self.n_ghosts = int(self.ghost_source.shape[0])
        self.n_faces = int(self.face_cells.shape[0])
        self._view = None

    @classmethod
    def from_npz(cls, z, prefix="mesh_"):
        return cls(**{k: z[prefix + k] for k in MESH_FIELDS})

    def view(self):
        if self._view is None:
            def p(a, t):
                return a.ctypes.data_as(t)
            self._view = RgMeshView(self.n_cells, self.n_ghosts, self.n_faces, 0,
                                    p(self.point_xy, _dp), p(self.cm_xy, _dp),
                                    p(self.volume, _dp), p(self.cd_volume, _dp),
                                    p(self.ghost_source, _ip), p(self.ghost_face, _ip),
                                    p(self.face_cells, _ip), p(self.face_vertices, _dp),
                                    p(self.cell_face_offset, _ip), p(self.cell_faces, _ip))
        return self._view

    def nbytes(self):
        return sum(getattr(self, k).nbytes for k in MESH_FIELDS)

    def topology_view(self):
        """The view without cm_xy, volume and cd_volume (NULL): for uploads with
        RG_MESH_DEVICE_GEOMETRY, which computes them on the device."""
        v = self.view()
        return RgMeshView(v.n_cells, v.n_ghosts, v.n_faces, 0, v.point_xy, None, None, None, v.ghost_source,
                          v.ghost_face, v.face_cells, v.face_vertices, v.cell_face_offset, v.cell_faces)

    def topology_nbytes(self):
        return sum(getattr(self, k).nbytes for k in MESH_FIELDS if k not in ("cm_xy", "volume", "cd_volume"))


def dptr(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


# ---------------------------------------------------------------- 3D

MESH3_FIELDS = ("face_cells", "face_normal", "face_area", "volume", "width", "cell_face_offset", "cell_faces")
_DTYPES3 = {"face_cells": np.int32, "face_normal": np.float64, "face_area": np.float64,
            "volume": np.float64, "width": np.float64, "cell_face_offset": np.int32,
            "cell_faces": np.int32}


class RgMesh3DView(C.Structure):
    _fields_ = [("n_cells", C.c_int32), ("n_faces", C.c_int32), ("face_cells", _ip), ("face_normal", _dp),
                ("face_area", _dp), ("volume", _dp), ("width", _dp), ("cell_face_offset", _ip),
                ("cell_faces", _ip)]


class PackedMesh3D:
    """Packed 3D tessellation: numpy arrays laid out as rg_mesh3d_view describes."""

    def __init__(self, **arrays):
        for k in MESH3_FIELDS:
            setattr(self, k, np.ascontiguousarray(arrays[k], dtype=_DTYPES3[k]))
        self.n_cells = int(self.volume.shape[0])
        self.n_faces = int(self.face_cells.shape[0])
        self._view = None

    @classmethod
    def from_npz(cls, z, prefix="mesh3_"):
        names = {"face_normal": "normal", "face_area": "area"}
        return cls(**{k: z[prefix + names.get(k, k)] for k in MESH3_FIELDS})

    def view(self):
        if self._view is None:
            def p(a, t):
                return a.ctypes.data_as(t)
            self._view = RgMesh3DView(self.n_cells, self.n_faces, p(self.face_cells, _ip), p(self.face_normal, _dp),
                                      p(self.face_area, _dp), p(self.volume, _dp), p(self.width, _dp),
                                      p(self.cell_face_offset, _ip), p(self.cell_faces, _ip))
        return self._view

    def nbytes(self):
        return sum(getattr(self, k).nbytes for k in MESH3_FIELDS)
