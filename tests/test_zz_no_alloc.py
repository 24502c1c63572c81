"""The allocation-free time step (rg_cfl_dt_noalloc) against rg_cfl_dt.

rg_cfl_dt_noalloc serves callers whose own allocator owns all GPU memory and
who therefore cannot let the library call cudaMalloc / cudaFree (an rg_handle
allocates its mesh and state).  It takes caller-owned device arrays and keeps
its reduction scratch in a fixed array inside the library.  This test calls
it through the C ABI twice in a row, on two different states, and requires
each result to equal what the existing entry point rg_cfl_dt gives for the
same state: exactly, as every FP64 parity test here does.  It runs last
(file name) and works alone or after the other tests.
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
