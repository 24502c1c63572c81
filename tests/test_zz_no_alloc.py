"""The allocation-free time step (rg_cfl_dt_noalloc) against rg_cfl_dt.

rg_cfl_dt_noalloc serves callers whose own allocator owns all GPU memory and
who therefore cannot let the library call cudaMalloc / cudaFree (an rg_handle
allocates its mesh and state).  It takes caller-owned device arrays and keeps
its reduction scratch in a fixed array inside the library.  This test calls
it through the C ABI twice in a row, on two different states, and requires
each result to equal what the existing entry point rg_cfl_dt gives for the
same state: exactly, as every FP64 parity test here does.  It runs last
(file name) and works alone or after the other tests.  A second case fills
the scratch array exactly (1,048,576 cells, 4,096 blocks on the completion
counter), and the argument checks are exercised with a misaligned device
pointer and a host pointer, which must be refused before any launch.
"""
import ctypes as C

import numpy as np
import pytest

import richgpu
import synthetic

pytestmark = pytest.mark.gpu


def test_noalloc_cfl_matches_handle_cfl_on_two_calls():
    torch = pytest.importorskip("torch")
    mesh = synthetic.lattice_mesh(256, 256, (-1.0, 1.0, -1.0, 1.0), "rigid", seed=2)
    gamma = 5.0 / 3.0
    rng = np.random.default_rng(11)
    states = []
    for k in range(2):
        cells = synthetic.sedov_cells(mesh, gamma)
        cells[:, 2:] = rng.normal(0, 0.1 * (k + 1), (mesh.n_cells, 2))
        pv = rng.normal(0, 0.05, (mesh.n_cells, 2))
        states.append((cells, synthetic.face_velocities(mesh, pv)))

    # the existing entry point
    expected = []
    with richgpu.Handle(gamma=gamma, order=2, ghost_kind=0, device=0) as h:
        h.upload_mesh(mesh)
        for cells, ev in states:
            h.set_cells(cells)
            h.set_edge_velocities(ev)
            expected.append(h.cfl_dt())

    lib = richgpu.load()
    dev = torch.device("cuda", 0)
    volume = torch.from_numpy(mesh.volume).to(dev)
    off = torch.from_numpy(mesh.cell_face_offset).to(dev)
    faces = torch.from_numpy(mesh.cell_faces).to(dev)
    stream = torch.cuda.current_stream(dev)
    for (cells, ev), want in zip(states, expected):
        d_cells = torch.from_numpy(np.ascontiguousarray(cells)).to(dev)
        d_ev = torch.from_numpy(np.ascontiguousarray(ev)).to(dev)
        d_dt = torch.full((1,), -1.0, dtype=torch.float64, device=dev)
        st = lib.rg_cfl_dt_noalloc(mesh.n_cells, C.c_void_p(d_cells.data_ptr()),
                                   C.c_void_p(volume.data_ptr()), C.c_void_p(off.data_ptr()),
                                   C.c_void_p(faces.data_ptr()), C.c_void_p(d_ev.data_ptr()),
                                   C.c_double(gamma), C.c_double(0.3),
                                   C.c_void_p(d_dt.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert st == 0
        stream.synchronize()
        assert d_dt.item() == want


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib = richgpu.load()
    one = C.c_void_p(1)
    assert lib.rg_cfl_dt_noalloc(1_048_577, one, one, one, one, one, C.c_double(1.4), C.c_double(0.3),
                                 one, None) == 1  # RG_ERR_INVALID_ARGUMENT
    assert lib.rg_cfl_dt_noalloc(0, one, one, one, one, one, C.c_double(1.4), C.c_double(0.3),
                                 one, None) == 1


def _noalloc(lib, n, cells, volume, off, faces, ev, gamma, dt, stream):
    return lib.rg_cfl_dt_noalloc(n, C.c_void_p(cells), C.c_void_p(volume), C.c_void_p(off),
                                 C.c_void_p(faces), C.c_void_p(ev), C.c_double(gamma),
                                 C.c_double(0.3), C.c_void_p(dt), C.c_void_p(stream))


def test_noalloc_cfl_at_its_cell_limit():
    """1024 x 1024 cells: every one of the 4096 scratch slots is written."""
    torch = pytest.importorskip("torch")
    mesh = synthetic.lattice_mesh(1024, 1024, (-1.0, 1.0, -1.0, 1.0), "rigid", seed=3)
    assert mesh.n_cells == 1_048_576
    gamma = 1.4
    rng = np.random.default_rng(5)
    cells = synthetic.sedov_cells(mesh, gamma)
    cells[:, 2:] = rng.normal(0, 0.2, (mesh.n_cells, 2))
    ev = synthetic.face_velocities(mesh, rng.normal(0, 0.05, (mesh.n_cells, 2)))
    with richgpu.Handle(gamma=gamma, order=2, ghost_kind=0, device=0) as h:
        h.upload_mesh(mesh)
        h.set_cells(cells)
        h.set_edge_velocities(ev)
        want = h.cfl_dt()
    lib = richgpu.load()
    dev = torch.device("cuda", 0)
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev)
         for k, v in (("cells", cells), ("volume", mesh.volume), ("off", mesh.cell_face_offset),
                      ("faces", mesh.cell_faces), ("ev", ev))}
    stream = torch.cuda.current_stream(dev)
    for _ in range(2):
        d_dt = torch.full((1,), -1.0, dtype=torch.float64, device=dev)
        st = _noalloc(lib, mesh.n_cells, t["cells"].data_ptr(), t["volume"].data_ptr(),
                      t["off"].data_ptr(), t["faces"].data_ptr(), t["ev"].data_ptr(), gamma,
                      d_dt.data_ptr(), stream.cuda_stream)
        assert st == 0
        stream.synchronize()
        assert d_dt.item() == want


def test_noalloc_refuses_misaligned_and_host_pointers():
    torch = pytest.importorskip("torch")
    mesh = synthetic.lattice_mesh(16, 16, (0.0, 1.0, 0.0, 1.0), "rigid", seed=1)
    cells = synthetic.sedov_cells(mesh, 1.4)
    ev = np.zeros((mesh.n_faces, 2))
    lib = richgpu.load()
    dev = torch.device("cuda", 0)
    # one spare double in front, so that the view from element 1 is 8- but not 16-byte aligned
    big_cells = torch.zeros(4 * mesh.n_cells + 1, dtype=torch.float64, device=dev)
    big_cells[1:] = torch.from_numpy(cells.reshape(-1)).to(dev)
    big_ev = torch.zeros(2 * mesh.n_faces + 1, dtype=torch.float64, device=dev)
    d_cells = torch.from_numpy(np.ascontiguousarray(cells)).to(dev)
    d_ev = torch.from_numpy(ev).to(dev)
    volume = torch.from_numpy(mesh.volume).to(dev)
    off = torch.from_numpy(mesh.cell_face_offset).to(dev)
    faces = torch.from_numpy(mesh.cell_faces).to(dev)
    d_dt = torch.full((1,), -1.0, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    n = mesh.n_cells
    assert big_cells[1:].data_ptr() % 16 == 8
    # misaligned cells, then misaligned edge velocities
    assert _noalloc(lib, n, big_cells[1:].data_ptr(), volume.data_ptr(), off.data_ptr(),
                    faces.data_ptr(), d_ev.data_ptr(), 1.4, d_dt.data_ptr(), stream) == 1
    assert _noalloc(lib, n, d_cells.data_ptr(), volume.data_ptr(), off.data_ptr(),
                    faces.data_ptr(), big_ev[1:].data_ptr(), 1.4, d_dt.data_ptr(), stream) == 1
    # host arrays where device arrays belong: pageable numpy, then a host dt_out
    h_cells = np.ascontiguousarray(cells)
    assert _noalloc(lib, n, h_cells.ctypes.data, volume.data_ptr(), off.data_ptr(),
                    faces.data_ptr(), d_ev.data_ptr(), 1.4, d_dt.data_ptr(), stream) == 1
    h_dt = np.full(1, -1.0)
    assert _noalloc(lib, n, d_cells.data_ptr(), volume.data_ptr(), off.data_ptr(),
                    faces.data_ptr(), d_ev.data_ptr(), 1.4, h_dt.ctypes.data, stream) == 1
    torch.cuda.synchronize(dev)
    # nothing ran: the outputs are untouched
    assert d_dt.item() == -1.0 and h_dt[0] == -1.0
    # and the well-formed call still works afterwards
    assert _noalloc(lib, n, d_cells.data_ptr(), volume.data_ptr(), off.data_ptr(),
                    faces.data_ptr(), d_ev.data_ptr(), 1.4, d_dt.data_ptr(), stream) == 0
    torch.cuda.synchronize(dev)
    assert d_dt.item() > 0
