// rg_motion.cu -- device-side geometry and point motion of the 2D path,
// compiled with --fmad=false so every operation rounds as the reference's.
//
// Geometry (per mesh upload, when the caller sends only points, topology and
// face vertices):
//   k_dev_geometry  per cell: Tessellation::GetVolume (VoronoiMesh.cpp:420-434),
//                   CalcCellCM (:436-451) and SlabSymmetry::calcVolume
//                   (physical_geometry.cpp:13-21, the same triangles)
//   k_ghost_cms     per ghost: the periodic shift or the reflection about the
//                   box side (VoronoiMesh.cpp:316-330, 355-398)
// Point motion (hdsim::TimeAdvance, hdsim2d.cpp:149-175):
//   k_point_velocities  Eulerian / Lagrangian / RoundCells::operator()
//                       (round_cells.cpp:69-81, 105-119)
//   k_apply_fix         RoundCells::ApplyFix (:83-103, 121-134) with
//                       CorrectPointsOverShoot (:15-63)
//   k_edge_velocities   StationaryBox (stationary_box.cpp:20-40) or
//                       PeriodicEdgeVelocities (periodic_edge_velocities.cpp:5-21)
//                       through VoronoiMesh::CalcFaceVelocity (:146-151)
#include <math.h>

#include "rg_convert.cuh"
#include "rg_div.cuh"
#include "rg_motion.cuh"

namespace rg {
namespace {

constexpr int kMoBlock = 256;

// 0.5*|p1 . zcross(p2)| (geometry.cpp:100-104, 138-141)
__device__ __forceinline__ double half_cross(double2 p1, double2 p2) {
  return 0.5 * fabs(p1.x * p2.y + p1.y * (-p2.x));
}

// Cells taken in `order` (per tile by neighbour count; null: thread i, cell i).
__global__ void __launch_bounds__(kMoBlock) k_dev_geometry(MeshDev m, const int* order, double2* cms,
                                                            double* volume, double* cd_volume) {
  const int th = blockIdx.x * blockDim.x + threadIdx.x;
  if (th >= m.n || mesh_rejected(m)) return;
  const int i = order ? order[th] : th;
  const int b = m.cell_off[i], e1 = m.cell_off[i + 1];
  const double2 c = m.points[i];
  // one pass over the faces: the volume's fan from the mesh point and the
  // CM's fan from the first face's first vertex, each summed in face order
  // (the first face starts the volume's sum and fixes the CM's anchor)
  double area = 0;
  double2 pc = make_double2(0, 0);
  double a2 = 0;
  double2 an = make_double2(0, 0);
  if (b < e1) {
    const dbl4 v = m.face_vertices[m.cell_faces[b]];
    area += half_cross(make_double2(v.x - c.x, v.y - c.y), make_double2(v.z - c.x, v.w - c.y));
    an = make_double2(v.x, v.y);
  }
  for (int k = b + 1; k < e1; ++k) {
    const dbl4 v = m.face_vertices[m.cell_faces[k]];
    area += half_cross(make_double2(v.x - c.x, v.y - c.y), make_double2(v.z - c.x, v.w - c.y));
    const double t = half_cross(make_double2(v.x - an.x, v.y - an.y), make_double2(v.z - an.x, v.w - an.y));
    a2 += t;
    const double s = quot(t, 3.0);
    pc.x += ((an.x + v.x) + v.z) * s;
    pc.y += ((an.y + v.y) + v.w) * s;
  }
  volume[i] = area;
  cms[i] = make_double2(quot(pc.x, a2), quot(pc.y, a2));
  cd_volume[i] = a2;
}

__global__ void __launch_bounds__(kMoBlock) k_ghost_cms(MeshDev m, double2* cms, int ghost_kind, dbl4 box) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= m.g || mesh_rejected(m)) return;
  const int p = m.n + g, src = m.ghost_source[g];
  const double2 cs = cms[src];
  const double2 q = m.points[p];
  double2 r = cs;
  if (ghost_kind == RG_GHOST_PERIODIC) {
    const double2 o = m.points[src];
    r = make_double2(cs.x + (q.x - o.x), cs.y + (q.y - o.y));
  } else if (q.x > box.y) {
    r = make_double2(cs.x + 2 * (box.y - cs.x), cs.y + 0.0);
  } else if (q.y > box.w) {
    r = make_double2(cs.x + 0.0, cs.y + 2 * (box.w - cs.y));
  } else if (q.x < box.x) {
    r = make_double2(cs.x + 2 * (box.x - cs.x), cs.y + 0.0);
  } else if (q.y < box.z) {
    r = make_double2(cs.x + 0.0, cs.y + 2 * (box.z - cs.y));
  }
  cms[p] = r;
}

__device__ __forceinline__ double vabs2(double x, double y) { return root(x * x + y * y); }

// CylindricalSymmetry (physical_geometry.cpp:44-110): Axis normalises its
// direction (:40-42); change_coordinate gives (along, |across|).
struct CylAxis {
  double ox, oy, dx, dy;
};
__device__ __forceinline__ CylAxis cyl_axis(dbl4 od, bool unit) {
  if (unit) return CylAxis{od.x, od.y, od.z, od.w};
  const double ab = vabs2(od.z, od.w);
  return CylAxis{od.x, od.y, quot(od.z, ab), quot(od.w, ab)};
}
__device__ __forceinline__ double2 change_coordinate(double vx, double vy, const CylAxis& a) {
  const double px = vx - a.ox, py = vy - a.oy;
  return make_double2(px * a.dx + py * a.dy, fabs(px * a.dy + py * (-a.dx)));
}
// :75-82 calc_cone_segment_volume (pow(x,2.) is x*x)
__device__ __forceinline__ double cone_segment(double2 p1, double2 p2, const CylAxis& a) {
  const double2 q1 = change_coordinate(p1.x, p1.y, a), q2 = change_coordinate(p2.x, p2.y, a);
  return (kPi / 3.) * (q2.x - q1.x) * (q1.y * q1.y + q2.y * q2.y + q1.y * q2.y);
}

__global__ void __launch_bounds__(kMoBlock) k_cyl_geometry(MeshDev m, double* xarea, double* cd_volume, dbl4 od,
                                                            int unit) {
  if (mesh_rejected(m)) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const CylAxis a = cyl_axis(od, unit != 0);
  if (t < m.e) {
    // :66-71 calcArea
    const dbl4 v = m.face_vertices[t];
    const double2 p1 = change_coordinate(v.x, v.y, a), p2 = change_coordinate(v.z, v.w, a);
    const double dy = p2.y - p1.y, dx = p2.x - p1.x;
    xarea[t] = kPi * (p1.y + p2.y) * root(dy * dy + dx * dx);
  }
  if (cd_volume && t < m.n) {
    // :94-104 calcVolume over the cell's edges, :84-92 calc_triangular_ring_volume
    const int b = m.cell_off[t], e1 = m.cell_off[t + 1];
    if (e1 > b) {
      const dbl4 v0 = m.face_vertices[m.cell_faces[b]];
      const double2 an = make_double2(v0.x, v0.y);
      double res = 0;
      for (int k = b + 1; k < e1; ++k) {
        const dbl4 v = m.face_vertices[m.cell_faces[k]];
        const double2 f = make_double2(v.x, v.y), s = make_double2(v.z, v.w);
        res += fabs(cone_segment(an, f, a) + cone_segment(f, s, a) + cone_segment(s, an, a));
      }
      cd_volume[t] = res;
    }
  }
}

__device__ __forceinline__ double sound(double g, const double* c) { return root(quot(g * c[1], c[0])); }

__global__ void __launch_bounds__(kMoBlock) k_point_velocities(StepArgs a, MotionArgs mo) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const MeshDev& m = a.mesh;
  if (i >= m.n) return;
  const double* c = a.cells + 4 * static_cast<size_t>(i);
  double2 w = make_double2(0, 0);
  if (mo.kind >= RG_MOTION_LAGRANGIAN) w = make_double2(c[2], c[3]);  // lagrangian.cpp:3-13
  if (mo.kind == RG_MOTION_ROUND_CELLS && !mo.cold) {
    const double2 r = m.points[i], s = m.cms[i];
    const double d = vabs2(s.x - r.x, s.y - r.y);
    const double R = a.geom.width[i];
    if (!(d < 0.9 * mo.eta * R)) {
      const double cs = smax(sound(a.gamma, c), vabs2(c[2], c[3]));
      const double f = mo.chi * cs;
      w.x += quot((s.x - r.x) * f, R);
      w.y += quot((s.y - r.y) * f, R);
    }
  }
  mo.pv[i] = w;
}

__global__ void __launch_bounds__(kMoBlock) k_apply_fix(StepArgs a, MotionArgs mo) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const MeshDev& m = a.mesh;
  if (i >= m.n) return;
  const double dt = a.dt_from_device ? a.status->dt : a.dt_host;
  double2 v = mo.pv[i];
  const double2 r = m.points[i];
  const double R = a.geom.width[i];
  if (mo.cold) {
    const double2 s = m.cms[i];
    const double d = vabs2(s.x - r.x, s.y - r.y);
    if (!(d < 0.9 * mo.eta * R)) {
      const double* c = a.cells + 4 * static_cast<size_t>(i);
      double cs = smax(vabs2(c[2], c[3]), sound(a.gamma, c));
      const int b = m.cell_off[i], nn = m.cell_off[i + 1] - b;
      for (int k = 0; k < nn; ++k) {
        const int2 fc = m.face_cells[m.cell_faces[b + k]];
        const int nb = fc.x != i ? fc.x : fc.y;
        // the reference compares the neighbour's id with the neighbour count
        // (round_cells.cpp:93-94); ids beyond the real cells it would read
        // out of range are left out
        if ((nb < m.n ? nb : m.ghost_source[nb - m.n]) == i || nb > nn || nb >= m.n) continue;
        const double* cn = a.cells + 4 * static_cast<size_t>(nb);
        cs = smax(cs, sound(a.gamma, cn));
        cs = smax(cs, vabs2(cn[2], cn[3]));
      }
      const double f = mo.chi * smin(quot(d, dt), cs);
      v.x += quot((s.x - r.x) * f, R);
      v.y += quot((s.y - r.y) * f, R);
    }
  }
  if (mo.fix) {
    const double inv_dt = quot(1.0, dt);
    const dbl4 bx = mo.box;  // left, right, down, up
    if ((v.x * dt * 2 + r.x) > bx.y) {
      double f = quot(0.25 * (bx.y - r.x) * inv_dt, vabs2(v.x, v.y));
      if (R * 0.1 > (bx.y - r.x)) f *= -0.1;
      v = make_double2(v.x * f, v.y * f);
    }
    if ((v.x * dt * 2 + r.x) < bx.x) {
      double f = quot(0.25 * (r.x - bx.x) * inv_dt, vabs2(v.x, v.y));
      if (R * 0.1 > (r.x - bx.x)) f *= -0.1;
      v = make_double2(v.x * f, v.y * f);
    }
    if ((v.y * dt * 2 + r.y) > bx.w) {
      double f = quot(0.25 * (bx.w - r.y) * inv_dt, vabs2(v.x, v.y));
      if (R * 0.1 > (bx.w - r.y)) f *= -0.1;
      v = make_double2(v.x * f, v.y * f);
    }
    if ((v.y * dt * 2 + r.y) < bx.z) {
      double f = quot(0.25 * (r.y - bx.z) * inv_dt, vabs2(v.x, v.y));
      if (R * 0.1 > (r.y - bx.z)) f *= -0.1;
      v = make_double2(v.x * f, v.y * f);
    }
  }
  mo.pv[i] = v;
}

__global__ void __launch_bounds__(kMoBlock) k_edge_velocities(StepArgs a, MotionArgs mo) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const MeshDev& m = a.mesh;
  if (e >= m.e) return;
  const int2 fc = m.face_cells[e];
  const int oa = fc.x < m.n ? fc.x : m.ghost_source[fc.x - m.n];
  const int ob = fc.y < m.n ? fc.y : m.ghost_source[fc.y - m.n];
  double2 w = make_double2(0, 0);
  if (mo.edges == RG_EDGES_PERIODIC || oa != ob) {
    const double2 wl = mo.pv[oa], wr = mo.pv[ob];
    const double2 rl = m.points[fc.x], rr = m.points[fc.y];
    const dbl4 v = m.face_vertices[e];
    const double fx = 0.5 * (v.x + v.z), fy = 0.5 * (v.y + v.w);  // Edge.cpp:88-91 calc_centroid
    const double mx = (rr.x + rl.x) / 2, my = (rr.y + rl.y) / 2;
    const double dx = rr.x - rl.x, dy = rr.y - rl.y;
    const double ab = a.geom.dab[e];  // sqrt(dx*dx + dy*dy), per mesh upload
    const double sp = (wl.x - wr.x) * (fx - mx) + (wl.y - wr.y) * (fy - my);
    const double den = ab * ab;
    w = make_double2((wl.x + wr.x) * 0.5 + quot(dx * sp, den), (wl.y + wr.y) * 0.5 + quot(dy * sp, den));
  }
  mo.ev[e] = w;
}

// The same face velocities for an FP32-mixed handle, straight into its FP32
// copy: the coordinate differences in FP64, each rounded once (x_R - x_L, and
// the face centroid's offset from the points' midpoint as
// ((v0 - x_L) + (v1 - x_R)) / 2), the rest in FP32 (|x_R - x_L| from the
// FP64 geometry).  The FP64 face velocities are formed when they are read
// back (rg_get_edge_velocities).
__global__ void __launch_bounds__(kMoBlock) k_edge_velocities32(StepArgs a, MotionArgs mo, float2* ev32) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const MeshDev& m = a.mesh;
  if (e >= m.e) return;
  const int2 fc = m.face_cells[e];
  const int oa = fc.x < m.n ? fc.x : m.ghost_source[fc.x - m.n];
  const int ob = fc.y < m.n ? fc.y : m.ghost_source[fc.y - m.n];
  float2 w = make_float2(0.0f, 0.0f);
  if (mo.edges == RG_EDGES_PERIODIC || oa != ob) {
    const double2 wl = mo.pv[oa], wr = mo.pv[ob];
    const double2 rl = m.points[fc.x], rr = m.points[fc.y];
    const dbl4 v = m.face_vertices[e];
    const float dx = narrow(rr.x - rl.x), dy = narrow(rr.y - rl.y);
    const float ox = 0.5f * (narrow(v.x - rl.x) + narrow(v.z - rr.x));
    const float oy = 0.5f * (narrow(v.y - rl.y) + narrow(v.w - rr.y));
    const float lx = narrow(wl.x), ly = narrow(wl.y), rx = narrow(wr.x), ry = narrow(wr.y);
    const float sp = (lx - rx) * ox + (ly - ry) * oy;
    const float ab = narrow(a.geom.dab[e]);
    const float q = sp / (ab * ab);
    w = make_float2(0.5f * (lx + rx) + dx * q, 0.5f * (ly + ry) + dy * q);
  }
  ev32[e] = w;
}

inline int mo_blocks(int n) { return (n + kMoBlock - 1) / kMoBlock; }

}  // namespace

cudaError_t launch_device_geometry(const MeshDev& m, const int* order, double2* cms, double* volume,
                                   double* cd_volume, int ghost_kind, const double* box, cudaStream_t s) {
  if (m.n > 0) k_dev_geometry<<<mo_blocks(m.n), kMoBlock, 0, s>>>(m, order, cms, volume, cd_volume);
  if (m.g > 0) k_ghost_cms<<<mo_blocks(m.g), kMoBlock, 0, s>>>(m, cms, ghost_kind, make_dbl4(box[0], box[1], box[2], box[3]));
  return cudaGetLastError();
}

cudaError_t launch_cyl_geometry(const MeshDev& m, double* xarea, double* cd_volume, const double* origin,
                                const double* direction, bool unit, cudaStream_t s) {
  const int work = m.e > m.n ? m.e : m.n;
  if (work > 0)
    k_cyl_geometry<<<mo_blocks(work), kMoBlock, 0, s>>>(
        m, xarea, cd_volume, make_dbl4(origin[0], origin[1], direction[0], direction[1]), unit ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_point_velocities(const StepArgs& a, const MotionArgs& mo, cudaStream_t s) {
  if (a.mesh.n > 0) k_point_velocities<<<mo_blocks(a.mesh.n), kMoBlock, 0, s>>>(a, mo);
  return cudaGetLastError();
}

cudaError_t launch_apply_fix(const StepArgs& a, const MotionArgs& mo, cudaStream_t s) {
  if (a.mesh.n > 0 && mo.kind == RG_MOTION_ROUND_CELLS && (mo.cold || mo.fix))
    k_apply_fix<<<mo_blocks(a.mesh.n), kMoBlock, 0, s>>>(a, mo);
  return cudaGetLastError();
}

cudaError_t launch_edge_velocities(const StepArgs& a, const MotionArgs& mo, cudaStream_t s) {
  if (a.mesh.e > 0) k_edge_velocities<<<mo_blocks(a.mesh.e), kMoBlock, 0, s>>>(a, mo);
  return cudaGetLastError();
}

cudaError_t launch_edge_velocities32(const StepArgs& a, const MotionArgs& mo, float2* ev32, cudaStream_t s) {
  if (a.mesh.e > 0) k_edge_velocities32<<<mo_blocks(a.mesh.e), kMoBlock, 0, s>>>(a, mo, ev32);
  return cudaGetLastError();
}

}  // namespace rg
