"""The tessellator of the test and benchmark meshes (synthetic.lattice_mesh)
against the reference's own VoronoiMesh of the same points.

tests/golden/mesh/*.npz hold rich_pack(VoronoiMesh(points)) (the reference's
tessellation, packed by huji-rich_gb300/host/rich_pack.hpp; written by
oracle/ref/ref_dump.cpp's mesh_rigid / mesh_periodic cases through
tests/golden/make_golden.py) for the points synthetic.jittered_points gives,
in input order.  The two packings are the same mesh under an exact
renumbering:

* real cells: the same numbering and the same mesh points, bit for bit;
* ghost points: a bijection that keeps each ghost's source cell, its
  position equal to within a few ulp (the reference reflects about a wall as
  2 par (par . (x - v0)) - (x - v0) + v0, Delaunay.cpp:853, which rounds the
  coordinate along the wall; synthetic.py keeps it);
* faces: a bijection between faces with the same two (renumbered) points;
* every cell's faces (the CSR lists) map onto each other, ascending in
  their own numbering;
* face vertices, volumes, CacheData volumes and CMs equal to within
  rounding: the Voronoi vertices are circumcentres of the same Delaunay
  triangles, which the reference evaluates relative to one corner chosen by
  its own triangle orientation (Delaunay.cpp:1100-1140).  On a lattice
  jittered by 1e-3 of a cell, neighbouring quadruples of points are nearly
  cocircular, which amplifies rounding by about the inverse jitter: measured
  differences are at most 174 ulp of the box scale in the vertices and
  58 in the CMs, and 2.5e-12 relative in the cell volumes (tolerances
  below: 512 ulp, 512 ulp, 1e-11);
* each rigid-wall ghost's first face (ghost_face, whose real side the ghost
  reflects) is the same face; a periodic ghost copies its source cell and
  its first face, which depends on the face numbering, is not read.

The GPU kernels are exact functions of the packed mesh, so a benchmark or
test on synthetic meshes runs the reference's Voronoi mesh up to these
roundings and numberings.
"""
import os

import numpy as np
import pytest

import synthetic

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = {
    "lattice64_rigid": (64, 64, (-1.0, 1.0, -1.0, 1.0), "rigid", 2),
    "lattice64_periodic": (64, 64, (0.0, 1.0, 0.0, 1.0), "periodic", 3),
    "lattice48x16_rigid": (48, 16, (0.0, 1.0, 0.0, 0.2), "rigid", 1),
}
EPS = np.finfo(float).eps
GHOST_ULP = 8 * EPS      # ghost points: the wall reflection's rounding
GEOM_ULP = 512 * EPS     # vertices and CMs, relative to the box scale
VOLUME_REL = 1e-11       # cell volumes, relative per cell


def load(name):
    f = np.load(os.path.join(HERE, "golden", "mesh", name + ".npz"))
    return {k[5:]: f[k] for k in f.files if k.startswith("mesh_")}, f


def renumbering(ref, syn):
    """Point map (reference point id -> synthetic point id) and face map."""
    n = syn.n_cells
    rp, sp = ref["point_xy"], syn.point_xy
    rsrc, ssrc = ref["ghost_source"], syn.ghost_source
    pmap = np.arange(len(rp))
    by_source = {}
    for g, s in enumerate(ssrc):
        by_source.setdefault(int(s), []).append(n + g)
    used = set()
    for g in range(len(rsrc)):
        cand = by_source.get(int(rsrc[g]), [])
        d = [np.abs(sp[c] - rp[n + g]).max() for c in cand]
        assert cand, f"reference ghost {g} (source {rsrc[g]}) has no synthetic ghost"
        best = cand[int(np.argmin(d))]
        assert min(d) <= GHOST_ULP * np.abs(rp[n + g]).max(), (g, min(d))
        assert best not in used
        used.add(best)
        pmap[n + g] = best
    fc = pmap[ref["face_cells"]]
    skey = {(min(a, b), max(a, b)): e for e, (a, b) in enumerate(syn.face_cells)}
    fmap = np.array([skey[(min(a, b), max(a, b))] for a, b in fc])
    return pmap, fmap


@pytest.mark.parametrize("name", sorted(CASES))
def test_synthetic_lattice_is_the_reference_voronoi_mesh(name):
    nx, ny, box, boundary, seed = CASES[name]
    ref, raw = load(name)
    syn = synthetic.lattice_mesh(nx, ny, box, boundary, seed=seed)
    n = syn.n_cells
    assert ref["volume"].shape[0] == n
    # counts
    assert len(ref["face_cells"]) == syn.n_faces
    assert len(ref["ghost_source"]) == syn.n_ghosts
    # real cells: same numbering, same points bit for bit
    assert np.array_equal(ref["point_xy"][:n], syn.point_xy[:n])
    pmap, fmap = renumbering(ref, syn)
    # faces: a bijection between faces with the same two points
    assert len(np.unique(fmap)) == syn.n_faces
    # orientation: (first, second) either kept or swapped, with the vertices
    # in the matching order
    fc = pmap[ref["face_cells"]]
    sfc = syn.face_cells[fmap]
    kept = (fc == sfc).all(1)
    swapped = (fc[:, ::-1] == sfc).all(1)
    assert (kept | swapped).all()
    scale = np.abs(syn.point_xy).max()
    rv, sv = ref["face_vertices"], syn.face_vertices[fmap]
    d_same = np.abs(rv - sv).max(1)
    d_flip = np.abs(rv - sv[:, [2, 3, 0, 1]]).max(1)
    assert np.minimum(d_same, d_flip).max() <= GEOM_ULP * scale
    # every cell's faces are the same faces
    ro, rf = ref["cell_face_offset"], ref["cell_faces"]
    so, sf = syn.cell_face_offset, syn.cell_faces
    assert np.array_equal(np.diff(ro), np.diff(so))
    for i in range(n):
        assert sorted(fmap[rf[ro[i]:ro[i + 1]]]) == list(sf[so[i]:so[i + 1]])
        assert np.all(np.diff(rf[ro[i]:ro[i + 1]]) > 0)
    # ghost sources and first faces
    g = syn.n_ghosts
    inv = np.empty(g, dtype=np.int64)
    inv[pmap[n:] - n] = np.arange(g)
    assert np.array_equal(syn.ghost_source, ref["ghost_source"][inv])
    if boundary == "rigid":
        # the face whose real side a rigid-wall ghost reflects
        assert np.array_equal(syn.ghost_face, fmap[ref["ghost_face"]][inv])
    else:
        # periodic ghosts copy their source cell; the first face is not read,
        # and with another face numbering another of the ghost's faces is first
        for gi in range(g):
            assert n + gi in syn.face_cells[syn.ghost_face[gi]]
    # volumes (both formulas) and centres of mass
    for key in ("volume", "cd_volume"):
        a, b = ref[key], getattr(syn, key)
        assert (np.abs(a - b) / np.abs(a)).max() <= VOLUME_REL, key
    rcm = np.empty_like(ref["cm_xy"])
    rcm[pmap] = ref["cm_xy"]
    assert np.abs(rcm - syn.cm_xy).max() <= GEOM_ULP * scale


def test_mesh_pin_fixtures_are_the_generated_points():
    """The fixtures' real points are the synthetic generator's, in order."""
    for name, (nx, ny, box, boundary, seed) in CASES.items():
        ref, raw = load(name)
        px, py = synthetic.jittered_points(nx, ny, *box, seed)
        assert np.array_equal(ref["point_xy"][:nx * ny], np.stack([px.ravel(), py.ravel()], 1))
        assert tuple(raw["case_params"]) == (nx, ny, seed)
