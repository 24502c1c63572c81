"""Seeded synthetic workloads in the packed-mesh format (numpy only).

The reference builds its tessellation with its own Delaunay code on the host
(out of scope here; the hot path takes the packed arrays).  For benchmarks
and large-size tests, this module builds the Voronoi tessellation of a
jittered square lattice directly: with jitter far below the cell size the
Delaunay triangulation splits every lattice quad along one diagonal, chosen
by the in-circle test, so the Voronoi vertices are the circumcentres of
those triangles.  Boundaries follow VoronoiMesh's conventions:

* rigid walls (SquareBox): one layer of mirror points, reflected as
  VoronoiMesh.cpp:310-329 GetReflection does, no corner copies; edges of zero
  length (the degenerate wall quads) are dropped as VoronoiMesh::build_v does
  (VoronoiMesh.cpp:283-285);
* periodic (PeriodicBox): one layer of shifted copies including corners,
  ghost centres of mass shifted with their points (VoronoiMesh.cpp:363-375).

Cell volumes and centres of mass use the reference formulas
(VoronoiMesh.cpp:420-451, physical_geometry.cpp:13-21).  Initial conditions
follow the benchmark configurations (Sod, Sedov-Taylor, smooth periodic
bumps).
"""
import numpy as np

from meshview import PackedMesh


def jittered_points(nx, ny, x0, x1, y0, y1, seed, jitter=1e-3):
    rng = np.random.default_rng(seed)
    u = rng.uniform(-jitter, jitter, size=(nx, ny, 2))
    dx, dy = (x1 - x0) / nx, (y1 - y0) / ny
    i = np.arange(nx)[:, None]
    j = np.arange(ny)[None, :]
    return x0 + (i + 0.5 + u[..., 0]) * dx, y0 + (j + 0.5 + u[..., 1]) * dy


def _circumcentres(ax, ay, bx, by, cx, cy):
    d = 2.0 * (ax * (by - cy) + bx * (cy - ay) + cx * (ay - by))
    a2 = ax * ax + ay * ay
    b2 = bx * bx + by * by
    c2 = cx * cx + cy * cy
    ux = (a2 * (by - cy) + b2 * (cy - ay) + c2 * (ay - by)) / d
    uy = (a2 * (cx - bx) + b2 * (ax - cx) + c2 * (bx - ax)) / d
    return ux, uy


def lattice_mesh(nx, ny, box=(0.0, 1.0, 0.0, 1.0), boundary="rigid", seed=0, jitter=1e-3):
    """Packed Voronoi mesh of an nx x ny jittered lattice in box (x0, x1, y0, y1)."""
    x0, x1, y0, y1 = box
    lx, ly = x1 - x0, y1 - y0
    px, py = jittered_points(nx, ny, x0, x1, y0, y1, seed, jitter)
    n = nx * ny
    cid = (np.arange(nx)[:, None] * ny + np.arange(ny)[None, :]).astype(np.int64)
    NX, NY = nx + 2, ny + 2
    X = np.full((NX, NY), np.nan)
    Y = np.full((NX, NY), np.nan)
    SRC = np.full((NX, NY), -1, dtype=np.int64)
    REAL = np.zeros((NX, NY), dtype=bool)
    X[1:-1, 1:-1], Y[1:-1, 1:-1], SRC[1:-1, 1:-1] = px, py, cid
    REAL[1:-1, 1:-1] = True
    if boundary == "rigid":
        # VoronoiMesh.cpp GetReflection: point + (2*(boundary - x), 0) etc.
        X[0, 1:-1], Y[0, 1:-1], SRC[0, 1:-1] = px[0] + 2 * (x0 - px[0]), py[0], cid[0]
        X[-1, 1:-1], Y[-1, 1:-1], SRC[-1, 1:-1] = px[-1] + 2 * (x1 - px[-1]), py[-1], cid[-1]
        X[1:-1, 0], Y[1:-1, 0], SRC[1:-1, 0] = px[:, 0], py[:, 0] + 2 * (y0 - py[:, 0]), cid[:, 0]
        X[1:-1, -1], Y[1:-1, -1], SRC[1:-1, -1] = px[:, -1], py[:, -1] + 2 * (y1 - py[:, -1]), cid[:, -1]
    elif boundary == "periodic":
        X[0, 1:-1], Y[0, 1:-1], SRC[0, 1:-1] = px[-1] - lx, py[-1], cid[-1]
        X[-1, 1:-1], Y[-1, 1:-1], SRC[-1, 1:-1] = px[0] + lx, py[0], cid[0]
        X[1:-1, 0], Y[1:-1, 0], SRC[1:-1, 0] = px[:, -1], py[:, -1] - ly, cid[:, -1]
        X[1:-1, -1], Y[1:-1, -1], SRC[1:-1, -1] = px[:, 0], py[:, 0] + ly, cid[:, 0]
        for (gi, gj, si, sj, sx, sy) in ((0, 0, -1, -1, -lx, -ly), (-1, 0, 0, -1, lx, -ly),
                                         (0, -1, -1, 0, -lx, ly), (-1, -1, 0, 0, lx, ly)):
            X[gi, gj], Y[gi, gj], SRC[gi, gj] = px[si, sj] + sx, py[si, sj] + sy, cid[si, sj]
    else:
        raise ValueError(boundary)
    present = SRC >= 0

    # quads Q(I,J) with corners a=(I,J) b=(I+1,J) c=(I+1,J+1) d=(I,J+1)
    def corner(A, di, dj):
        return A[di:NX - 1 + di, dj:NY - 1 + dj]
    ax, ay, bx, by = corner(X, 0, 0), corner(Y, 0, 0), corner(X, 1, 0), corner(Y, 1, 0)
    cx, cy, dx_, dy_ = corner(X, 1, 1), corner(Y, 1, 1), corner(X, 0, 1), corner(Y, 0, 1)
    pa, pb, pc, pd = (corner(present, 0, 0), corner(present, 1, 0), corner(present, 1, 1),
                      corner(present, 0, 1))
    full = pa & pb & pc & pd
    with np.errstate(invalid="ignore"):
        adx, ady, bdx, bdy, cdx, cdy = ax - dx_, ay - dy_, bx - dx_, by - dy_, cx - dx_, cy - dy_
        incircle = (adx * (bdy * (cdx * cdx + cdy * cdy) - cdy * (bdx * bdx + bdy * bdy))
                    - ady * (bdx * (cdx * cdx + cdy * cdy) - cdx * (bdx * bdx + bdy * bdy))
                    + (adx * adx + ady * ady) * (bdx * cdy - bdy * cdx))
        diag_bd = full & (incircle > 0)  # d inside circle(a,b,c): split along b-d
        # T0 holds side ab, T1 holds side cd (see module docstring of the layout)
        t0x, t0y = _circumcentres(ax, ay, bx, by, np.where(diag_bd, dx_, cx), np.where(diag_bd, dy_, cy))
        t1x, t1y = _circumcentres(np.where(diag_bd, bx, ax), np.where(diag_bd, by, ay), cx, cy, dx_, dy_)
        # three-corner quads (rigid-wall corners): the one triangle of the present corners
        tri = ~full & (pa.astype(int) + pb + pc + pd == 3)
        if tri.any():
            qx = [np.where(pa, ax, np.nan), np.where(pb, bx, np.nan), np.where(pc, cx, np.nan), np.where(pd, dx_, np.nan)]
            qy = [np.where(pa, ay, np.nan), np.where(pb, by, np.nan), np.where(pc, cy, np.nan), np.where(pd, dy_, np.nan)]
            sx = np.stack(qx, -1)[tri]
            sy = np.stack(qy, -1)[tri]
            keep = ~np.isnan(sx)
            tx = sx[keep].reshape(-1, 3)
            ty = sy[keep].reshape(-1, 3)
            ux, uy = _circumcentres(tx[:, 0], ty[:, 0], tx[:, 1], ty[:, 1], tx[:, 2], ty[:, 2])
            t0x[tri], t0y[tri], t1x[tri], t1y[tri] = ux, uy, ux, uy
    # which triangle holds the right side bc and the left side da
    rcx, rcy = np.where(diag_bd, t1x, t0x), np.where(diag_bd, t1y, t0y)
    lcx, lcy = np.where(diag_bd, t0x, t1x), np.where(diag_bd, t0y, t1y)

    P = np.arange(NX * NY).reshape(NX, NY)  # extended-grid point index
    e_a, e_b, v0x, v0y, v1x, v1y = [], [], [], [], [], []

    def add(pa_, pb_, ux0, uy0, ux1, uy1, mask):
        e_a.append(pa_[mask]); e_b.append(pb_[mask])
        v0x.append(ux0[mask]); v0y.append(uy0[mask]); v1x.append(ux1[mask]); v1y.append(uy1[mask])

    # horizontal lattice edges (I,J)-(I+1,J), J = 1..NY-2: quads Q(I,J-1) (T1) and Q(I,J) (T0)
    A, B = P[:-1, 1:-1], P[1:, 1:-1]
    m = (present[:-1, 1:-1] & present[1:, 1:-1]) & (REAL[:-1, 1:-1] | REAL[1:, 1:-1])
    add(A, B, t1x[:, :-1], t1y[:, :-1], t0x[:, 1:], t0y[:, 1:], m)
    # vertical lattice edges (I,J)-(I,J+1), I = 1..NX-2: quads Q(I-1,J) (right side) and Q(I,J) (left side)
    A, B = P[1:-1, :-1], P[1:-1, 1:]
    m = (present[1:-1, :-1] & present[1:-1, 1:]) & (REAL[1:-1, :-1] | REAL[1:-1, 1:])
    add(A, B, rcx[:-1, :], rcy[:-1, :], lcx[1:, :], lcy[1:, :], m)
    # quad diagonals
    Pa, Pb, Pc, Pd = P[:-1, :-1], P[1:, :-1], P[1:, 1:], P[:-1, 1:]
    RA, RB, RC, RD = REAL[:-1, :-1], REAL[1:, :-1], REAL[1:, 1:], REAL[:-1, 1:]
    d1 = np.where(diag_bd, Pb, Pa)
    d2 = np.where(diag_bd, Pd, Pc)
    rr = np.where(diag_bd, RB | RD, RA | RC)
    add(d1, d2, t0x, t0y, t1x, t1y, full & rr)
    ea, eb = np.concatenate(e_a), np.concatenate(e_b)
    V = np.stack([np.concatenate(v0x), np.concatenate(v0y), np.concatenate(v1x), np.concatenate(v1y)], 1)
    length = np.hypot(V[:, 2] - V[:, 0], V[:, 3] - V[:, 1])
    keep = length > 1e-8 * min(lx / nx, ly / ny)  # VoronoiMesh::build_v drops zero-length edges
    ea, eb, V = ea[keep], eb[keep], V[keep]

    # point ids: real cells by lattice id, ghosts numbered in order of first face
    real_flat = REAL.ravel()
    src_flat = SRC.ravel()
    ida = np.where(real_flat[ea], src_flat[ea], -1)
    idb = np.where(real_flat[eb], src_flat[eb], -1)
    # face order: by the smallest real neighbour, then the other point
    key1 = np.where(ida >= 0, ida, n) * 1.0
    key1 = np.minimum(key1, np.where(idb >= 0, idb, n))
    key2 = np.maximum(np.where(ida >= 0, ida, -1), np.where(idb >= 0, idb, -1))
    order = np.lexsort((ea + eb, key2, key1))
    ea, eb, V, ida, idb = ea[order], eb[order], V[order], ida[order], idb[order]
    ne = len(ea)
    gflat = np.stack([np.where(ida < 0, ea, -1), np.where(idb < 0, eb, -1)], 1).ravel()
    pos = np.nonzero(gflat >= 0)[0]
    uniq, first = np.unique(gflat[pos], return_index=True)
    order_first = np.argsort(first, kind="stable")       # ghosts in order of first face
    ghost_pts = uniq[order_first]
    ghost_face = (pos[first[order_first]] // 2).astype(np.int32)
    g = len(ghost_pts)
    gmap = np.full(NX * NY, -1, dtype=np.int64)
    gmap[ghost_pts.astype(np.int64)] = n + np.arange(g)
    fa = np.where(ida >= 0, ida, gmap[ea])
    fb = np.where(idb >= 0, idb, gmap[eb])
    face_cells = np.stack([fa, fb], 1).astype(np.int32)
    ghost_pts = ghost_pts.astype(np.int64)
    point_xy = np.zeros((n + g, 2))
    point_xy[:n, 0] = px.ravel()
    point_xy[:n, 1] = py.ravel()
    point_xy[n:, 0] = X.ravel()[ghost_pts]
    point_xy[n:, 1] = Y.ravel()[ghost_pts]
    ghost_source = src_flat[ghost_pts].astype(np.int32)

    # CSR of real cells, ascending faces
    side_cell = np.concatenate([fa, fb])
    side_face = np.concatenate([np.arange(ne), np.arange(ne)])
    real_side = side_cell < n
    sc, sf = side_cell[real_side], side_face[real_side]
    o = np.lexsort((sf, sc))
    sc, sf = sc[o], sf[o]
    offset = np.zeros(n + 1, dtype=np.int64)
    offset[1:] = np.cumsum(np.bincount(sc, minlength=n))
    offset = offset.astype(np.int32)
    cell_faces = sf.astype(np.int32)

    # volumes and centres of mass with the reference formulas
    v0 = V[cell_faces, 0:2]
    v1 = V[cell_faces, 2:4]
    xc = point_xy[sc]
    p1, p2 = v0 - xc, v1 - xc
    tri_area = 0.5 * np.abs(p1[:, 0] * p2[:, 1] + p1[:, 1] * (-p2[:, 0]))
    volume = np.bincount(sc, weights=tri_area, minlength=n)
    anchor = V[cell_faces[offset[:-1]], 0:2][sc]
    q1, q2 = v0 - anchor, v1 - anchor
    first = np.zeros(len(sc), dtype=bool)
    first[offset[:-1]] = True
    a2 = np.where(first, 0.0, 0.5 * np.abs(q1[:, 0] * q2[:, 1] + q1[:, 1] * (-q2[:, 0])))
    cd_volume = np.bincount(sc, weights=a2, minlength=n)
    pcx = np.bincount(sc, weights=(a2 / 3.0) * (anchor[:, 0] + v0[:, 0] + v1[:, 0]), minlength=n)
    pcy = np.bincount(sc, weights=(a2 / 3.0) * (anchor[:, 1] + v0[:, 1] + v1[:, 1]), minlength=n)
    cm = np.zeros((n + g, 2))
    cm[:n, 0] = pcx / cd_volume
    cm[:n, 1] = pcy / cd_volume
    gs = ghost_source.astype(np.int64)
    if boundary == "rigid":
        gx, gy = X.ravel()[ghost_pts], Y.ravel()[ghost_pts]
        sxp, syp = point_xy[gs, 0], point_xy[gs, 1]
        cmx, cmy = cm[gs, 0].copy(), cm[gs, 1].copy()
        left, right = np.isclose(gx + sxp, 2 * x0), np.isclose(gx + sxp, 2 * x1)
        down, up = np.isclose(gy + syp, 2 * y0), np.isclose(gy + syp, 2 * y1)
        cmx = np.where(left, cmx + 2 * (x0 - cmx), np.where(right, cmx + 2 * (x1 - cmx), cmx))
        cmy = np.where(down, cmy + 2 * (y0 - cmy), np.where(up, cmy + 2 * (y1 - cmy), cmy))
        cm[n:, 0], cm[n:, 1] = cmx, cmy
    else:
        cm[n:] = cm[gs] + (point_xy[n:] - point_xy[gs])
    return PackedMesh(point_xy=point_xy, cm_xy=cm, volume=volume, cd_volume=cd_volume,
                      ghost_source=ghost_source, ghost_face=np.array(ghost_face, dtype=np.int32),
                      face_cells=face_cells, face_vertices=V, cell_face_offset=offset,
                      cell_faces=cell_faces)


# ------------------------------------------------------------------ states

def sod_cells(mesh, x_split=0.5):
    """2D Sod tube: rho=1, p=1 for x<x_split; rho=0.125, p=0.1 beyond."""
    x = mesh.point_xy[:mesh.n_cells, 0]
    c = np.zeros((mesh.n_cells, 4))
    left = x < x_split
    c[:, 0] = np.where(left, 1.0, 0.125)
    c[:, 1] = np.where(left, 1.0, 0.1)
    return c


def sedov_cells(mesh, gamma=5.0 / 3.0, energy=1.0, radius=0.02, p_ambient=1e-6):
    """Sedov-Taylor: rho=1, p=p_ambient, energy deposited as pressure in r<radius
    (at least the few cells nearest the centre on coarse meshes)."""
    x = mesh.point_xy[:mesh.n_cells]
    r = np.hypot(x[:, 0], x[:, 1])
    hot = r < radius
    if hot.sum() < 4:
        hot = r <= np.sort(r)[3]
    c = np.zeros((mesh.n_cells, 4))
    c[:, 0] = 1.0
    c[:, 1] = p_ambient
    c[hot, 1] = (gamma - 1) * energy / mesh.cd_volume[hot].sum()
    return c


def bumps_cells(mesh, seed=5, n_bumps=8, n_modes=16, amp=0.1):
    """Periodic smooth field: rho = 1 + sum of Gaussian bumps, p = 1, velocity
    from random Fourier modes of amplitude amp (the adjoint configuration)."""
    rng = np.random.default_rng(seed)
    x = mesh.point_xy[:mesh.n_cells]
    c = np.zeros((mesh.n_cells, 4))
    rho = np.ones(mesh.n_cells)
    for _ in range(n_bumps):
        cx, cy = rng.uniform(0, 1, 2)
        w = rng.uniform(0.02, 0.1)
        ddx = (x[:, 0] - cx + 0.5) % 1.0 - 0.5
        ddy = (x[:, 1] - cy + 0.5) % 1.0 - 0.5
        rho += amp * np.exp(-(ddx ** 2 + ddy ** 2) / w ** 2)
    vx = np.zeros(mesh.n_cells)
    vy = np.zeros(mesh.n_cells)
    for _ in range(n_modes):
        kx, ky = rng.integers(-3, 4, 2)
        ph = rng.uniform(0, 2 * np.pi, 2)
        a = rng.normal(0, amp / np.sqrt(n_modes), 2)
        arg = 2 * np.pi * (kx * x[:, 0] + ky * x[:, 1])
        vx += a[0] * np.sin(arg + ph[0])
        vy += a[1] * np.sin(arg + ph[1])
    c[:, 0], c[:, 1], c[:, 2], c[:, 3] = rho, 1.0, vx, vy
    return c


def face_velocities(mesh, point_velocities, stationary_box=True):
    """Edge velocities from point velocities with VoronoiMesh::CalcFaceVelocity
    (VoronoiMesh.cpp:146-151); StationaryBox (stationary_box.cpp:20-40) puts
    zero on faces whose two sides have the same original cell."""
    n = mesh.n_cells
    fa, fb = mesh.face_cells[:, 0].astype(np.int64), mesh.face_cells[:, 1].astype(np.int64)
    src = np.concatenate([np.arange(n), mesh.ghost_source.astype(np.int64)])
    oa, ob = src[fa], src[fb]
    wl, wr = point_velocities[oa], point_velocities[ob]
    rl, rr = mesh.point_xy[fa], mesh.point_xy[fb]
    f = 0.5 * (mesh.face_vertices[:, 0:2] + mesh.face_vertices[:, 2:4])
    d = rr - rl
    s = np.sum((wl - wr) * (f - (rr + rl) / 2), 1) / np.sum(d * d, 1)
    w = 0.5 * (wl + wr) + s[:, None] * d
    if stationary_box:
        w[oa == ob] = 0.0
    return np.ascontiguousarray(w)


# ------------------------------------------------------------------ batches

def concat_meshes(meshes):
    """Disjoint union of packed meshes: real cells of every problem first (in
    problem order), then every problem's ghosts; faces in problem order.
    Returns the mesh and the problem cell-offset table."""
    from meshview import PackedMesh
    ns = np.array([m.n_cells for m in meshes])
    gs = np.array([m.n_ghosts for m in meshes])
    es = np.array([m.n_faces for m in meshes])
    cell_base = np.concatenate([[0], np.cumsum(ns)])
    N = int(cell_base[-1])
    ghost_base = N + np.concatenate([[0], np.cumsum(gs)])
    face_base = np.concatenate([[0], np.cumsum(es)])
    fc, fv, pts_r, pts_g, cm_r, cm_g, gsrc, gface, offs, cf = ([] for _ in range(10))
    vol, cdv = [], []
    for k, m in enumerate(meshes):
        f = m.face_cells.astype(np.int64)
        f = np.where(f < m.n_cells, f + cell_base[k], f - m.n_cells + ghost_base[k])
        fc.append(f)
        fv.append(m.face_vertices)
        pts_r.append(m.point_xy[:m.n_cells])
        pts_g.append(m.point_xy[m.n_cells:])
        cm_r.append(m.cm_xy[:m.n_cells])
        cm_g.append(m.cm_xy[m.n_cells:])
        vol.append(m.volume)
        cdv.append(m.cd_volume)
        gsrc.append(m.ghost_source.astype(np.int64) + cell_base[k])
        gface.append(np.where(m.ghost_face >= 0, m.ghost_face.astype(np.int64) + face_base[k], -1))
        offs.append(m.cell_face_offset[1:].astype(np.int64) + (0 if k == 0 else offs_total))
        offs_total = int(offs[-1][-1])
        cf.append(m.cell_faces.astype(np.int64) + face_base[k])
    mesh = PackedMesh(point_xy=np.concatenate(pts_r + pts_g), cm_xy=np.concatenate(cm_r + cm_g),
                      volume=np.concatenate(vol), cd_volume=np.concatenate(cdv),
                      ghost_source=np.concatenate(gsrc), ghost_face=np.concatenate(gface),
                      face_cells=np.concatenate(fc), face_vertices=np.concatenate(fv),
                      cell_face_offset=np.concatenate([[0]] + offs), cell_faces=np.concatenate(cf))
    return mesh, cell_base.astype(np.int32)


def riemann_batch(n_problems=512, seed=11, min_cells=1024, max_cells=65536, jitter=1e-3):
    """Independent 2D Riemann problems on [0,1]^2 with rigid walls: cell
    counts log-uniform in [min_cells, max_cells] (square lattices), left and
    right states split by a random line through the centre, density and
    pressure log-uniform in [0.1, 10], velocities uniform in [-1, 1]^2,
    gamma 1.4 or 5/3.  Returns (mesh, problem offsets, gammas, cells)."""
    return riemann_batch_range(range(n_problems), seed, min_cells, max_cells, jitter)


def riemann_batch_range(problems, seed=11, min_cells=1024, max_cells=65536, jitter=1e-3):
    """The batch of the given problems of riemann_batch, in their order (one
    rank's shard)."""
    meshes, states, gammas = [], [], []
    for p in problems:
        m, c, g = riemann_problem(p, seed, min_cells, max_cells, jitter)
        meshes.append(m)
        states.append(c)
        gammas.append(g)
    mesh, offsets = concat_meshes(meshes)
    return mesh, offsets, np.array(gammas), np.concatenate(states), meshes


def _riemann_side(rng, min_cells, max_cells):
    count = np.exp(rng.uniform(np.log(min_cells), np.log(max_cells)))
    return max(4, int(round(np.sqrt(count))))


def riemann_problem_cells(p, seed=11, min_cells=1024, max_cells=65536):
    """Cell count of problem p of riemann_batch, without building its mesh."""
    return _riemann_side(np.random.default_rng([seed, p]), min_cells, max_cells) ** 2


def riemann_problem(p, seed=11, min_cells=1024, max_cells=65536, jitter=1e-3):
    """Problem p of riemann_batch on its own: (mesh, cells, gamma)."""
    rng = np.random.default_rng([seed, p])
    side = _riemann_side(rng, min_cells, max_cells)
    m = lattice_mesh(side, side, (0.0, 1.0, 0.0, 1.0), "rigid", seed=seed * 100003 + p, jitter=jitter)
    ang = rng.uniform(0, 2 * np.pi)
    nrm = np.array([np.cos(ang), np.sin(ang)])
    x = m.point_xy[:m.n_cells] - 0.5
    left = x @ nrm < 0
    rho = np.exp(rng.uniform(np.log(0.1), np.log(10.0), 2))
    prs = np.exp(rng.uniform(np.log(0.1), np.log(10.0), 2))
    vel = rng.uniform(-1.0, 1.0, (2, 2))
    c = np.zeros((m.n_cells, 4))
    c[:, 0] = np.where(left, rho[0], rho[1])
    c[:, 1] = np.where(left, prs[0], prs[1])
    c[:, 2] = np.where(left, vel[0, 0], vel[1, 0])
    c[:, 3] = np.where(left, vel[0, 1], vel[1, 1])
    gamma = 1.4 if rng.uniform() < 0.5 else 5.0 / 3.0
    return m, c, gamma


# ---------------------------------------------------------------- 3D

def cube_grid(nx, ny, nz, lo=(0.0, 0.0, 0.0), hi=(1.0, 0.8, 0.6)):
    """Packed CubeGrid (CubeGrid.cpp:23-160): faces normal to z, then y, then
    x, in the reference's index order; boundary faces have -1 outside; cell
    faces in ascending face order; Normal (CubeGrid.cpp:280-287) = (0,0,dz),
    (0,dy,0), (dx,0,0); Face::GetArea (Face.cpp:24-30) of the four vertices
    (two triangles, each 0.5*|(v1-v0) x (v2-v0)|), the vertices formed as
    CubeGrid forms them.  Cell index = i*ny*nz + j*nz + k for the cell at
    (x index i, y index j, z index k)."""
    from meshview import PackedMesh3D
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    dx, dy, dz = (hi[0] - lo[0]) / nx, (hi[1] - lo[1]) / ny, (hi[2] - lo[2]) / nz

    def cell(i, j, k):
        return i * ny * nz + j * nz + k

    def area(vs):
        # vs: (..., 4, 3) vertices; 0.5*abs(Cross(v[i+1]-v0, v[i+2]-v0)) summed over i = 0, 1
        res = np.zeros(vs.shape[:-2])
        for t in range(2):
            a = vs[..., t + 1, :] - vs[..., 0, :]
            b = vs[..., t + 2, :] - vs[..., 0, :]
            cx = a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1]
            cy = a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2]
            cz = a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]
            res = res + 0.5 * np.sqrt(cx * cx + cy * cy + cz * cz)
        return res

    faces, areas, normals = [], [], []
    # z faces: index i*nx + j + k*ny*nx for k in 0..nz, i (y) in 0..ny-1, j (x) in 0..nx-1
    side = [lo, lo + [dx, 0, 0], lo + [dx, dy, 0], lo + [0, dy, 0]]
    k, i, j = np.meshgrid(np.arange(nz + 1), np.arange(ny), np.arange(nx), indexing="ij")
    k, i, j = k.ravel(), i.ravel(), j.ravel()
    # side + Vector3D(dx*j, 0, dz*k) + Vector3D(0, dy*i, 0)
    vz = np.asarray(side, dtype=np.float64)[None] + np.stack([dx * j, 0 * j, dz * k], -1)[:, None, :].astype(np.float64)
    vz = vz + np.stack([0 * i, dy * i, 0 * i], -1)[:, None, :].astype(np.float64)
    fz = np.stack([np.where(k == 0, -1, cell(j, i, k - 1)), np.where(k == nz, -1, cell(j, i, k))], -1)
    faces.append(fz)
    areas.append(area(vz))
    normals.append(np.tile([0.0, 0.0, dz], (len(fz), 1)))
    # y faces: index i*nx*nz + k + j*nz + nx*(nz+1)*ny for k in 0..nz-1, i (y) in 0..ny, j (x) in 0..nx-1
    side = [lo, lo + [dx, 0, 0], lo + [dx, 0, dz], lo + [0, 0, dz]]
    k, i, j = np.meshgrid(np.arange(nz), np.arange(ny + 1), np.arange(nx), indexing="ij")
    idx = (i * nx * nz + k + j * nz).ravel()
    k, i, j = k.ravel(), i.ravel(), j.ravel()
    # side + Vector3D(dx*j, dy*i, 0) + Vector3D(0, 0, dz*k)
    vy = np.asarray(side, dtype=np.float64)[None] + np.stack([dx * j, dy * i, 0 * j], -1)[:, None, :].astype(np.float64)
    vy = vy + np.stack([0 * k, 0 * k, dz * k], -1)[:, None, :].astype(np.float64)
    fy = np.stack([np.where(i == 0, -1, cell(j, i - 1, k)), np.where(i == ny, -1, cell(j, i, k))], -1)
    order = np.argsort(idx, kind="stable")
    faces.append(fy[order])
    areas.append(area(vy)[order])
    normals.append(np.tile([0.0, dy, 0.0], (len(fy), 1)))
    # x faces: index i*nz + j*ny*nz + k + offsets for k in 0..nz-1, i (y) in 0..ny-1, j (x) in 0..nx
    side = [lo, lo + [0, dy, 0], lo + [0, dy, dz], lo + [0, 0, dz]]
    k, i, j = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx + 1), indexing="ij")
    idx = (i * nz + j * ny * nz + k).ravel()
    k, i, j = k.ravel(), i.ravel(), j.ravel()
    # side + Vector3D(0, dy*i, 0) + Vector3D(dx*j, 0, dz*k)
    vx = np.asarray(side, dtype=np.float64)[None] + np.stack([0 * i, dy * i, 0 * i], -1)[:, None, :].astype(np.float64)
    vx = vx + np.stack([dx * j, 0 * j, dz * k], -1)[:, None, :].astype(np.float64)
    fx = np.stack([np.where(j == 0, -1, cell(j - 1, i, k)), np.where(j == nx, -1, cell(j, i, k))], -1)
    order = np.argsort(idx, kind="stable")
    faces.append(fx[order])
    areas.append(area(vx)[order])
    normals.append(np.tile([dx, 0.0, 0.0], (len(fx), 1)))
    face_cells = np.concatenate(faces).astype(np.int32)
    n = nx * ny * nz
    # cell -> faces in ascending face order
    owner = np.concatenate([face_cells[:, 0], face_cells[:, 1]])
    fid = np.concatenate([np.arange(len(face_cells))] * 2)
    keep = owner >= 0
    owner, fid = owner[keep], fid[keep]
    order = np.lexsort((fid, owner))
    counts = np.bincount(owner, minlength=n)
    off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    return PackedMesh3D(face_cells=face_cells, face_normal=np.concatenate(normals), face_area=np.concatenate(areas),
                        volume=np.full(n, dx * dy * dz), width=np.full(n, min(min(dx, dy), dz)),
                        cell_face_offset=off, cell_faces=fid[order].astype(np.int32))


def cube_centres(nx, ny, nz, lo=(0.0, 0.0, 0.0), hi=(1.0, 0.8, 0.6)):
    """CubeGrid mesh points (CubeGrid.cpp:138-151), in cell order."""
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    dx, dy, dz = (hi[0] - lo[0]) / nx, (hi[1] - lo[1]) / ny, (hi[2] - lo[2]) / nz
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    p = np.stack([i * dx + 0.5 * dx, j * dy + 0.5 * dy, k * dz + 0.5 * dz], -1).reshape(-1, 3)
    return lo + p


def cube_blast_cells(nx, ny, nz, lo=(0.0, 0.0, 0.0), hi=(1.0, 0.8, 0.6), seed=3, gamma=5 / 3):
    """A 3D workload state: ambient gas (rho 1, p 1e-2) with a hot sphere
    (p 10) at the box centre and a seeded small random velocity field."""
    x = cube_centres(nx, ny, nz, lo, hi)
    c = np.asarray(lo) + 0.5 * (np.asarray(hi) - np.asarray(lo))
    r = np.sqrt(((x - c) ** 2).sum(1))
    rng = np.random.default_rng(seed)
    cells = np.zeros((len(x), 5))
    cells[:, 0] = 1.0
    cells[:, 1] = np.where(r < 0.1, 10.0, 1e-2)
    cells[:, 2:] = rng.uniform(-0.05, 0.05, (len(x), 3))
    return cells


def cube_sedov_cells(n, gamma=5 / 3, r0=0.04, energy=1.0, lo=(-0.5, -0.5, -0.5), hi=(0.5, 0.5, 0.5)):
    """3D Sedov-Taylor on an n^3 CubeGrid over [-0.5, 0.5]^3: rho 1, p 1e-6,
    total energy `energy` deposited as pressure in the cells with r < r0."""
    x = cube_centres(n, n, n, lo, hi)
    r = np.sqrt((x ** 2).sum(1))
    hot = r < r0
    vol = np.prod((np.asarray(hi) - np.asarray(lo)) / n)
    cells = np.zeros((len(x), 5))
    cells[:, 0] = 1.0
    cells[:, 1] = 1e-6
    cells[hot, 1] = (gamma - 1) * energy / (hot.sum() * vol)
    return cells
