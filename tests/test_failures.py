"""Failure detection without a GPU fault.

Bad states are made on the host (negative mass, energy below the kinetic
energy, NaN velocity, a cell with more than 20 faces, a singular gradient
matrix).  The oracle must raise the reference's error for them (CPU tests);
the CUDA path must report the same status, phase, index and value through
the C ABI, and the handle must stay usable afterwards (GPU tests).  Nothing
here traps or hangs a GPU: kernels record the error and return.
"""
import numpy as np
import pytest

import oracle
import synthetic
from meshview import PackedMesh

GAMMA = 5.0 / 3.0


def base(nx=16, bnd="periodic"):
    box = (0.0, 1.0, 0.0, 1.0) if bnd == "periodic" else (-1.0, 1.0, -1.0, 1.0)
    mesh = synthetic.lattice_mesh(nx, nx, box, bnd, seed=7)
    cells = synthetic.bumps_cells(mesh) if bnd == "periodic" else synthetic.sedov_cells(mesh, GAMMA)
    return mesh, cells, oracle.init_extensives(mesh, cells, GAMMA)


def split_faces(mesh, cell, pieces=5):
    """The same tessellation with every face of `cell` cut into `pieces`
    collinear faces: a valid polygon mesh in which `cell` has > 20 faces."""
    fc = mesh.face_cells.tolist()
    fv = mesh.face_vertices.tolist()
    new_fc, new_fv = [], []
    own = set(mesh.cell_faces[mesh.cell_face_offset[cell]:mesh.cell_face_offset[cell + 1]].tolist())
    for e in range(mesh.n_faces):
        if e in own:
            x0, y0, x1, y1 = fv[e]
            for k in range(pieces):
                a, b = k / pieces, (k + 1) / pieces
                new_fc.append(fc[e])
                new_fv.append([x0 + a * (x1 - x0), y0 + a * (y1 - y0), x0 + b * (x1 - x0), y0 + b * (y1 - y0)])
        else:
            new_fc.append(fc[e])
            new_fv.append(fv[e])
    face_cells = np.array(new_fc, dtype=np.int32)
    n = mesh.n_cells
    lists = [[] for _ in range(n)]
    ghost_face = {}
    for e, (a, b) in enumerate(new_fc):
        for p in (a, b):
            if p < n:
                lists[p].append(e)
            elif p not in ghost_face:
                ghost_face[p] = e
    off = np.cumsum([0] + [len(x) for x in lists]).astype(np.int32)
    gf = np.array([ghost_face.get(n + g, -1) for g in range(mesh.n_ghosts)], dtype=np.int32)
    return PackedMesh(point_xy=mesh.point_xy, cm_xy=mesh.cm_xy, volume=mesh.volume,
                      cd_volume=mesh.cd_volume, ghost_source=mesh.ghost_source, ghost_face=gf,
                      face_cells=face_cells, face_vertices=np.array(new_fv),
                      cell_face_offset=off, cell_faces=np.concatenate(lists).astype(np.int32))


def singular_volume(mesh, cell):
    """A volume for `cell` that makes LinearGaussImproved's 2x2 matrix
    V*I - S singular (an eigenvalue of S, LinearGaussImproved.cpp:80-111)."""
    b, e = mesh.cell_face_offset[cell], mesh.cell_face_offset[cell + 1]
    S = np.zeros((2, 2))
    xi, ci = mesh.point_xy[cell], mesh.cm_xy[cell]
    for f in mesh.cell_faces[b:e]:
        a0, a1 = mesh.face_cells[f]
        o = a1 if a0 == cell else a0
        v = mesh.face_vertices[f]
        mid = 0.5 * (v[:2] + v[2:])
        c = mid - 0.5 * (mesh.cm_xy[o] + ci)
        d = mesh.point_xy[o] - xi
        r = d / np.linalg.norm(d) * np.linalg.norm(v[2:] - v[:2])
        S += np.array([[c[0] * r[0], c[1] * r[0]], [c[0] * r[1], c[1] * r[1]]])
    ev = np.linalg.eigvals(S)
    real = [x.real for x in ev if abs(x.imag) < 1e-14]
    return max(real) if real else None


def injections():
    mesh, cells, ext = base()
    out = {}
    e = ext.copy()
    e[37, 0] = -abs(e[37, 0])                       # negative mass -> negative density
    out["negative_density"] = (mesh, cells, e, 10)
    e = ext.copy()
    e[41, 1] = 0.1 * e[41, 1]
    e[41, 2] = 3.0 * e[41, 0]                       # kinetic energy above the total
    out["negative_energy"] = (mesh, cells, e, 11)
    c = cells.copy()
    c[50, 2] = np.nan                               # NaN velocity -> HLLC failure
    out["hllc_nan"] = (mesh, c, ext, None)
    cell = 21
    m2 = split_faces(mesh, cell)
    out["too_many_neighbours"] = (m2, cells, ext, 15)
    m3 = synthetic.lattice_mesh(16, 16, (0.0, 1.0, 0.0, 1.0), "periodic", seed=7)
    for cand in range(30, m3.n_cells):
        v = singular_volume(m3, cand)
        if v is not None and v > 0:
            vol = m3.volume.copy()
            vol[cand] = v
            m3 = PackedMesh(**{k: (vol if k == "volume" else getattr(m3, k)) for k in
                               ("point_xy", "cm_xy", "volume", "cd_volume", "ghost_source", "ghost_face",
                                "face_cells", "face_vertices", "cell_face_offset", "cell_faces")})
            out["singular_matrix"] = (m3, cells, ext, 14)
            break
    return out


CASES = injections()


def oracle_failure(mesh, cells, ext):
    ev = np.zeros((mesh.n_faces, 2))
    with pytest.raises(oracle.OracleError) as ei:
        oracle.step(mesh, cells, ext, ev, GAMMA, 0.3, 2, oracle.lgi_params(1))
    return ei.value


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reports_reference_error(name):
    mesh, cells, ext, status = CASES[name]
    err = oracle_failure(mesh, cells, ext)
    if status is None:
        assert err.status in (12, 13)
    else:
        assert err.status == status


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_reports_same_error_as_oracle(name):
    import richgpu
    mesh, cells, ext, _ = CASES[name]
    want = oracle_failure(mesh, cells, ext)
    with richgpu.Handle(gamma=GAMMA, order=2, ghost_kind=1, device=0) as h:
        try:
            h.upload_mesh(mesh)
        except richgpu.RichError as e:            # geometry errors surface at upload too
            assert (e.status, e.phase, e.index) == (want.status, want.phase, want.index)
            assert e.value == want.value
            return
        h.set_cells(cells)
        h.set_extensives(ext)
        h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
        with pytest.raises(richgpu.RichError) as ei:
            h.step()
        e = ei.value
        assert (e.status, e.phase, e.index) == (want.status, want.phase, want.index)
        if not np.isnan(want.value):
            assert e.value == want.value
        # the handle is still usable after a reported failure
        good_mesh, good_cells, good_ext = base()
        h.upload_mesh(good_mesh)
        h.set_cells(good_cells)
        h.set_extensives(good_ext)
        h.set_edge_velocities(np.zeros((good_mesh.n_faces, 2)))
        assert h.step() > 0


@pytest.mark.gpu
def test_gpu_run_reports_first_failing_step():
    """A failure in the first step of an rg_run is the one reported."""
    import richgpu
    mesh, cells, ext, status = CASES["negative_density"]
    with richgpu.Handle(gamma=GAMMA, order=2, ghost_kind=1, device=0) as h:
        h.upload_mesh(mesh)
        h.set_cells(cells)
        h.set_extensives(ext)
        h.set_edge_velocities(np.zeros((mesh.n_faces, 2)))
        with pytest.raises(richgpu.RichError) as ei:
            h.run(5)
        assert ei.value.status == status and ei.value.index == 37


def corrupted_meshes():
    mesh, _, _ = base(8)
    out = {}
    fc = mesh.face_cells.copy()
    fc[5, 1] = mesh.n_cells + mesh.n_ghosts + 3          # neighbour id out of range
    out["face_out_of_range"] = (fc, None, None)
    cf = mesh.cell_faces.copy()
    cf[7] = mesh.n_faces + 10                            # face id out of range
    out["csr_face_out_of_range"] = (None, cf, None)
    cf = mesh.cell_faces.copy()
    cf[3], cf[4] = cf[4], cf[3]                          # not ascending
    out["csr_not_ascending"] = (None, cf, None)
    off = mesh.cell_face_offset.copy()
    off[10] = off[11] + 1                                # offsets not monotone
    out["offsets_not_monotone"] = (None, None, off)
    return mesh, out


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(corrupted_meshes()[1]))
def test_gpu_rejects_invalid_mesh_without_fault(name):
    """Every index is checked on the device (bounds-checked reads) before any
    kernel uses it: a corrupted mesh is refused with RG_ERR_INVALID_ARGUMENT
    and the handle keeps working on its previous mesh."""
    import richgpu
    mesh, bad = corrupted_meshes()
    fc, cf, off = bad[name]
    fields = {k: getattr(mesh, k) for k in ("point_xy", "cm_xy", "volume", "cd_volume", "ghost_source",
                                            "ghost_face", "face_cells", "face_vertices",
                                            "cell_face_offset", "cell_faces")}
    if fc is not None:
        fields["face_cells"] = fc
    if cf is not None:
        fields["cell_faces"] = cf
    if off is not None:
        fields["cell_face_offset"] = off
    broken = PackedMesh(**fields)
    good, cells, ext = base(8)
    with richgpu.Handle(gamma=GAMMA, order=2, ghost_kind=1, device=0) as h:
        h.upload_mesh(good)
        h.set_cells(cells)
        h.set_extensives(ext)
        h.set_edge_velocities(np.zeros((good.n_faces, 2)))
        with pytest.raises(richgpu.RichError) as ei:
            h.upload_mesh(broken)
        assert ei.value.status == 1
        h.mesh = good
        assert h.step() > 0
