// rg_fp64.cu -- plain-FP64 kernels of the hydro hot path for sm_103a.
//
// Compiled with --fmad=false: every multiply and add rounds separately, in
// the reference's order, so results are bit-identical to the reference's
// FP64 path (IEEE division and square root are exact-rounded on the device
// as on the host).  Each device function cites the reference code it
// restates (paths relative to the RICH source root).
//
// Passes of one step (hdsim::TimeAdvance, hdsim2d.cpp:149-241, fixed mesh):
//   k_cfl        per cell: SimpleCFL bound, block min, last block writes dt;
//                extra threads fill the ghost states
//   k_slopes     per cell: LinearGaussImproved slope + limiter (order 2)
//   k_faces_*    per face: reconstruction to the face, HLLC in the face frame,
//                rotation back, optional dt*area scaling
//   k_update     per cell: ascending-face CSR gather of the face fluxes
//                (SimpleExtensiveUpdater order, no atomics) + SimpleCellUpdater
// Geometry-only terms are computed once per mesh upload (k_geom_*).
#include <math.h>

#include "rg_fp64.cuh"
#include "rg_hllc.cuh"

namespace rg {
namespace {

constexpr int kBlock = 256;

// ---------------------------------------------------------------- geometry

// Per face: physical_geometry.cpp:8-11 calcArea, Edge.cpp:83-86 Parallel,
// spatial_reconstruction.cpp:3-6 CalcCentroid, the flux-frame normal of
// simple_flux_calculator.cpp:91-93 (order 1) or modular_flux_calculator.cpp:12-22
// with simple_flux_calculator.cpp:27-31 (order 2).
__global__ void __launch_bounds__(kBlock) k_geom_faces(GeomArgs a) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.mesh.e || mesh_rejected(a.mesh)) return;
  const int2 fc = a.mesh.face_cells[e];
  const dbl4 v = a.mesh.face_vertices[e];
  const double ax = v.x - v.z, ay = v.y - v.w;
  const double area = root(ax * ax + ay * ay);
  a.area[e] = area;
  const double2 p = make_double2(v.z - v.x, v.w - v.y);
  a.par[e] = p;
  const double2 mid = make_double2((v.x + v.z) * 0.5, (v.y + v.w) * 0.5);
  double2 n;
  if (a.order == 1) {
    const double2 x0 = a.mesh.points[fc.x], x1 = a.mesh.points[fc.y];
    n = make_double2(x1.x - x0.x, x1.y - x0.y);
  } else {
    double2 w;
    if (fc.x >= 0 && fc.x < a.mesh.n) {
      const double2 x0 = a.mesh.points[fc.x];
      w = make_double2(v.x - x0.x, v.y - x0.y);
    } else {
      const double2 x1 = a.mesh.points[fc.y];
      w = make_double2(x1.x - v.x, x1.y - v.y);
    }
    const double sp = w.x * p.x + w.y * p.y;
    const double pp = p.x * p.x + p.y * p.y;
    n = make_double2(w.x - quot(p.x * sp, pp), w.y - quot(p.y * sp, pp));
  }
  a.nrm[e] = n;
  a.nabs[e] = root(n.x * n.x + n.y * n.y);
  const double2 c0 = a.mesh.cms[fc.x], c1 = a.mesh.cms[fc.y];
  a.dm0[e] = make_double2(mid.x - c0.x, mid.y - c0.y);
  a.dm1[e] = make_double2(mid.x - c1.x, mid.y - c1.y);
  // |x1 - x0| (VoronoiMesh::CalcFaceVelocity's |rR - rL|) and the per-face
  // halves of calc_naive_slope (LinearGaussImproved.cpp:85-88): r_ij =
  // normalize(x_other - x_cell)*length and c_ij = centroid - 0.5*(cm_other +
  // cm_cell).  The second cell's r_ij is exactly -r_ij (x_a - x_b = -(x_b -
  // x_a), and rounding is sign-symmetric) and its c_ij the same (the sum
  // commutes), so each face computes them once.
  const double2 x0 = a.mesh.points[fc.x], x1 = a.mesh.points[fc.y];
  const double ddx = x1.x - x0.x, ddy = x1.y - x0.y;
  const double dab = root(ddx * ddx + ddy * ddy);
  a.dab[e] = dab;
  // Edge::GetLength = |second - first| = |first - second| = area
  a.rij[e] = make_double2(quot(ddx, dab) * area, quot(ddy, dab) * area);
  a.cij[e] = make_double2(mid.x - (c1.x + c0.x) * 0.5, mid.y - (c1.y + c0.y) * 0.5);
}

// Per cell: VoronoiMesh.cpp:410-413 GetWidth; the CSR neighbour words; the
// state-independent half of calc_naive_slope (LinearGaussImproved.cpp:67-126:
// matrix, determinant check, inverse, 0.5*r_ij) or of GetBoundarySlope (:401-417).
__global__ void __launch_bounds__(kBlock) k_geom_cells(GeomArgs a) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const MeshDev& m = a.mesh;
  if (t >= m.n || mesh_rejected(m)) return;
  const int i = a.cell_order ? a.cell_order[t] : t;
  a.width[i] = root(quot(m.volume[i], kPi));
  const int b = m.cell_off[i], nn = m.cell_off[i + 1] - b;
  // k_cell_order has set the boundary-slope flag (a face between a point and
  // its own mirror image); one pass over the faces writes the neighbour words
  // and the flag's half of the slope
  if (a.cflags[i] & kCellBoundarySlope) {
    const double2 cci = m.cms[i];
    double sxsy = 0, sy2 = 0, sx2 = 0;
    for (int k = 0; k < nn; ++k) {
      const int2 fc = m.face_cells[m.cell_faces[b + k]];
      const bool first = fc.x == i;
      const int other = first ? fc.y : fc.x;
      const bool mirror = orig_of(m, fc.x) == orig_of(m, fc.y);
      a.nbr[b + k] = static_cast<uint32_t>(other) | (mirror ? kNbrMirror : 0u) | (first ? kNbrFirst : 0u);
      const double2 co = m.cms[other];
      const double dx = co.x - cci.x, dy = co.y - cci.y;
      a.hr[b + k] = make_double2(dx, dy);
      sxsy += dy * dx;
      sx2 += dx * dx;
      sy2 += dy * dy;
    }
    a.minv[i] = make_dbl4(sxsy, sx2, sy2, sxsy * sxsy - sx2 * sy2);
    return;
  }
  if (nn > kMaxNaiveNeighbours) {
    record_error(a.status, 0, RG_ERR_TOO_MANY_NEIGHBORS, 2, i, nn);
    a.minv[i] = make_dbl4(0, 0, 0, 0);
    for (int k = 0; k < nn; ++k) {
      const int2 fc = m.face_cells[m.cell_faces[b + k]];
      const bool first = fc.x == i;
      a.nbr[b + k] = static_cast<uint32_t>(first ? fc.y : fc.x) | (first ? kNbrFirst : 0u);
    }
    return;
  }
  // no neighbour of this cell is a mirror image of it
  double m0 = 0, m1 = 0, m2 = 0, m3 = 0;
  for (int k = 0; k < nn; ++k) {
    const int e = m.cell_faces[b + k];
    const int2 fc = m.face_cells[e];
    const bool first = fc.x == i;
    a.nbr[b + k] = static_cast<uint32_t>(first ? fc.y : fc.x) | (first ? kNbrFirst : 0u);
    const double2 r = a.rij[e], c = a.cij[e];
    // -r_ij for the second cell: a sign flip of the bit pattern
    const uint64_t flip = first ? 0u : 0x8000000000000000ull;
    const double rx = conv_double_bits(conv_dbits(r.x) ^ flip), ry = conv_double_bits(conv_dbits(r.y) ^ flip);
    m0 -= c.x * rx;
    m1 -= c.y * rx;
    m2 -= c.x * ry;
    m3 -= c.y * ry;
    a.hr[b + k] = make_double2(rx * 0.5, ry * 0.5);
  }
  const double vol = m.volume[i];
  m0 += vol;
  m3 += vol;
  const double det = m0 * m3 - m1 * m2;
  if (fabs(det) < 1e-10 * vol * vol) record_error(a.status, 0, RG_ERR_SINGULAR_MATRIX, 2, i, det);
  const double di = quot(1.0, det);
  a.minv[i] = make_dbl4(m3 * di, -m1 * di, -m2 * di, m0 * di);
}

// Per ghost: which cell it copies and, for rigid walls, the unit normal of
// RigidWallGenerator.cpp:5-15 (ghost minus real point, divided by its length).
__global__ void __launch_bounds__(kBlock) k_geom_ghosts(GeomArgs a) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const MeshDev& m = a.mesh;
  if (g >= m.g || mesh_rejected(m)) return;
  const int e = m.ghost_face[g];
  if (a.ghost_kind == RG_GHOST_PERIODIC || e < 0) {
    a.ghost_real[g] = m.ghost_source[g];
    a.ghost_unit[g] = make_double2(0, 0);
    return;
  }
  const int2 fc = m.face_cells[e];
  const bool ghost_first = fc.x >= m.n;
  a.ghost_real[g] = ghost_first ? fc.y : fc.x;
  const double2 x0 = m.points[fc.x], x1 = m.points[fc.y];
  const double2 nr = ghost_first ? make_double2(x0.x - x1.x, x0.y - x1.y)
                                 : make_double2(x1.x - x0.x, x1.y - x0.y);
  const double ab = root(nr.x * nr.x + nr.y * nr.y);
  a.ghost_unit[g] = make_double2(quot(nr.x, ab), quot(nr.y, ab));
}

// Per tile of kOrderTile cells: the order in which the per-cell FP64 kernels
// (device geometry, the per-cell geometry pass, slopes, update) take them, by
// (boundary-slope flag, neighbour count) and then by index.  Their per-cell
// loops run over a cell's neighbours, so a warp whose cells have equal counts
// runs no lane idle; every cell is still computed by one thread from the same
// inputs, so the results do not depend on the order.  The flag is
// LinearGaussImproved's (a face between a point and its own mirror image),
// taken from the topology and stored as the cell's flag for the per-cell
// geometry pass; runs after the index validation.
__global__ void __launch_bounds__(kOrderTile) k_cell_order(MeshDev m, int* order, int* cflags) {
  constexpr int kKeys = 128, kWarps = kOrderTile / 32;
  // count[w][k]: cells of warp w with key k, then their offset within key k
  __shared__ int count[kWarps][kKeys];
  __shared__ int start[kKeys];
  if (mesh_rejected(m)) return;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int base = blockIdx.x * kOrderTile, i = base + t, n = m.n;
  for (int j = t; j < kWarps * kKeys; j += kOrderTile) count[j / kKeys][j % kKeys] = 0;
  const bool live = i < n;
  int k = 0;
  if (live) {
    const int b = m.cell_off[i], nn = m.cell_off[i + 1] - b;
    bool mirror = false;
    for (int j = 0; j < nn; ++j) {
      const int2 fc = m.face_cells[m.cell_faces[b + j]];
      mirror |= orig_of(m, fc.x) == orig_of(m, fc.y);
    }
    k = (nn < 0 ? 0 : (nn > 63 ? 63 : nn)) | (mirror ? 64 : 0);
    cflags[i] = mirror ? kCellBoundarySlope : 0;
  }
  __syncthreads();
  // rank within the warp among equal keys (lanes in ascending order)
  const unsigned act = __ballot_sync(0xffffffffu, live);
  int before = 0;
  if (live) {
    const unsigned peers = __match_any_sync(act, k);
    before = __popc(peers & ((1u << lane) - 1u));
    if (lane == __ffs(peers) - 1) count[w][k] = __popc(peers);
  }
  __syncthreads();
  // per key: offsets of the warps (ascending), then the key's total
  if (t < kKeys) {
    int sum = 0;
    for (int ww = 0; ww < kWarps; ++ww) {
      const int c = count[ww][t];
      count[ww][t] = sum;
      sum += c;
    }
    start[t] = sum;
  }
  __syncthreads();
  if (t == 0) {
    int sum = 0;
    for (int kk = 0; kk < kKeys; ++kk) {
      const int c = start[kk];
      start[kk] = sum;
      sum += c;
    }
  }
  __syncthreads();
  if (live) order[base + start[k] + count[w][k] + before] = i;
}

// Index validation of an uploaded mesh, before any kernel indexes with it.
// Every read is bounds-checked against the array sizes; the first bad entry
// (smallest key: faces, then ghosts, then cells) is recorded.  Phase 0 keys:
// index = array position, value = the offending entry.
__global__ void __launch_bounds__(kBlock) k_validate(MeshDev m, DevStatus* st) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int np = m.n + m.g;
  if (t < m.e) {
    const int2 fc = m.face_cells[t];
    if (fc.x < 0 || fc.x >= np || fc.y < 0 || fc.y >= np || fc.x == fc.y || (fc.x >= m.n && fc.y >= m.n))
      record_error(st, 0, RG_ERR_INVALID_ARGUMENT, 0, t, fc.x);
  }
  if (t < m.g) {
    const int src = m.ghost_source[t], gf = m.ghost_face[t];
    bool bad = src < 0 || src >= m.n || gf < -1 || gf >= m.e;
    if (!bad && gf >= 0) {
      const int2 fc = m.face_cells[gf];
      bad = fc.x != m.n + t && fc.y != m.n + t;
    }
    if (bad) record_error(st, 0, RG_ERR_INVALID_ARGUMENT, 0, (1ll << 40) + t, gf);
  }
  if (t < m.n) {
    const int b = m.cell_off[t], e1 = m.cell_off[t + 1];
    bool bad = (t == 0 && b != 0) || b < 0 || e1 < b || e1 > m.m || e1 - b > (1 << 20);
    const int lo = b < 0 ? 0 : b, hi = e1 > m.m ? m.m : e1;
    int prev = -1;
    for (int k = lo; k < hi && !bad; ++k) {
      const int f = m.cell_faces[k];
      if (f < 0 || f >= m.e || f <= prev) {
        bad = true;
      } else {
        const int2 fc = m.face_cells[f];
        bad = fc.x != t && fc.y != t;
      }
      prev = f;
    }
    if (bad) record_error(st, 0, RG_ERR_INVALID_ARGUMENT, 0, (2ll << 40) + t, b);
  }
}

// ---------------------------------------------------------------- per step

// simple_cfl.cpp:28-47 (per cell) and :58-71 + lazy_list.hpp:185-191 (min, times cfl).
template <bool kBatch>
__global__ void __launch_bounds__(kMaxBlock) k_cfl(StepArgs a, int fill_ghosts) {
  const MeshDev& m = a.mesh;
  const int total = fill_ghosts ? m.n + m.g : m.n;
  // this thread's minimum of 1/bound as a bit pattern (positive doubles and
  // +inf order as integers)
  unsigned long long bits = kInfBits;
  // the trip count is uniform across a warp (base is per block), as the
  // warp-aggregated per-problem minimum of the batch form needs
  for (int base = blockIdx.x * blockDim.x; base < total; base += gridDim.x * blockDim.x) {
    const int t = base + threadIdx.x;
    double x = __longlong_as_double(static_cast<long long>(kInfBits));
    if (t < m.n) {
      const Cell c = load_cell(a.cells, t);
      const double radius = a.geom.width[t];
      const double cs = root(quot(gamma_at<kBatch>(a, t) * c.p, c.d));
      // fmax over faces of (cs + sqrt(q_e)) / radius equals (cs + sqrt(max q_e)) /
      // radius exactly: sqrt, + and / are correctly rounded, hence monotone, so
      // the maximum commutes with them.  NaN terms are skipped as fmax skips them.
      double q = 0;
      bool any = false;
      const int b = m.cell_off[t], e1 = m.cell_off[t + 1];
      if (a.ev_zero) {
        // every face at rest: each term is vx^2 + vy^2 (v - 0 == v)
        const double qq = c.vx * c.vx + c.vy * c.vy;
        if (e1 > b && !isnan(qq)) {
          q = fmax(q, qq);
          any = true;
        }
      } else {
        for (int k = b; k < e1; ++k) {
          const double2 w = reinterpret_cast<const double2*>(a.ev)[m.cell_faces[k]];
          const double dx = c.vx - w.x, dy = c.vy - w.y;
          const double qq = dx * dx + dy * dy;
          if (!isnan(qq)) {
            q = fmax(q, qq);
            any = true;
          }
        }
      }
      const double res = any ? fmax(0.0, quot(cs + root(q), radius)) : 0.0;
      x = quot(1.0, res);
    } else if (t < total) {
      fill_ghost(a, t - m.n);
    }
    const unsigned long long xb = static_cast<unsigned long long>(__double_as_longlong(x));
    if (kBatch)
      // per-problem minimum; the update kernel turns it into the problem's dt
      problem_min(a.dtmin_p, t < m.n ? a.cell_problem[t] : -1, xb);
    else
      bits = xb < bits ? xb : bits;
  }
  if (kBatch) return;
  grid_min_times(a.status, bits, a.cfl, &a.status->dt);
}

__global__ void __launch_bounds__(kBlock) k_ghost_fill(StepArgs a) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < a.mesh.g) fill_ghost(a, g);
}

// LinearGaussImproved.cpp:425-494 calc_slope for one cell (serial build).
template <bool kBatch>
__device__ __forceinline__ void k_slopes_item(const StepArgs& a, int i) {
  const MeshDev& m = a.mesh;
  const Cell cell = load_cell(a.cells, i);
  const int b = m.cell_off[i], nn = m.cell_off[i + 1] - b;
  const dbl4 mi = a.geom.minv[i];
  Cell sx, sy;
  if (a.geom.cflags[i] & kCellBoundarySlope) {
    // :401-422 GetBoundarySlope
    Cell phisy{0, 0, 0, 0}, phisx{0, 0, 0, 0};
    for (int k = 0; k < nn; ++k) {
      const Cell nb = point_state(a, static_cast<int>(a.geom.nbr[b + k] & kNbrIdMask));
      const double2 h = a.geom.hr[b + k];
      const Cell df{nb.d - cell.d, nb.p - cell.p, nb.vx - cell.vx, nb.vy - cell.vy};
      phisy.d = phisy.d + df.d * h.y;
      phisy.p = phisy.p + df.p * h.y;
      phisy.vx = phisy.vx + df.vx * h.y;
      phisy.vy = phisy.vy + df.vy * h.y;
      phisx.d = phisx.d + df.d * h.x;
      phisx.p = phisx.p + df.p * h.x;
      phisx.vx = phisx.vx + df.vx * h.x;
      phisx.vy = phisx.vy + df.vy * h.x;
    }
    const double sxsy = mi.x, sx2 = mi.y, sy2 = mi.z, den = mi.w;
    sx = Cell{quot(phisy.d * sxsy - phisx.d * sy2, den), quot(phisy.p * sxsy - phisx.p * sy2, den),
              quot(phisy.vx * sxsy - phisx.vx * sy2, den), quot(phisy.vy * sxsy - phisx.vy * sy2, den)};
    sy = Cell{quot(phisx.d * sxsy - phisy.d * sx2, den), quot(phisx.p * sxsy - phisy.p * sx2, den),
              quot(phisx.vx * sxsy - phisy.vx * sx2, den), quot(phisx.vy * sxsy - phisy.vy * sx2, den)};
  } else {
    // :80-133 calc_naive_slope, right-hand side and solve
    // the first neighbour starts the sums (cell*h, then + nb*h); the loop
    // takes the rest, so no iteration joins two computed values
    Cell vx{0, 0, 0, 0}, vy{0, 0, 0, 0};
    if (nn > 0) {
      const Cell nb = point_state(a, static_cast<int>(a.geom.nbr[b] & kNbrIdMask));
      const double2 h = a.geom.hr[b];
      vx = Cell{cell.d * h.x, cell.p * h.x, cell.vx * h.x, cell.vy * h.x};
      vy = Cell{cell.d * h.y, cell.p * h.y, cell.vx * h.y, cell.vy * h.y};
      addmult(vy, nb, h.y);
      addmult(vx, nb, h.x);
    }
    for (int k = 1; k < nn; ++k) {
      const Cell nb = point_state(a, static_cast<int>(a.geom.nbr[b + k] & kNbrIdMask));
      const double2 h = a.geom.hr[b + k];
      addmult(vx, cell, h.x);
      addmult(vy, cell, h.y);
      addmult(vy, nb, h.y);
      addmult(vx, nb, h.x);
    }
    sx = Cell{vx.d * mi.x, vx.p * mi.x, vx.vx * mi.x, vx.vy * mi.x};
    sy = Cell{vy.d * mi.w, vy.p * mi.w, vy.vx * mi.w, vy.vy * mi.w};
    addmult(sx, vy, mi.y);
    addmult(sy, vx, mi.z);
  }
  if (a.slf) {
    // :136-157 is_shock / PressureRatio.  cond1 is
    // (div v)*width < -delta_v*cs: false whenever the left side is >= 0,
    // otherwise screened in FP32 against |left| vs delta_v*cs.
    const double lhs = (sx.vx + sy.vy) * a.geom.width[i];
    bool shock = false;
    if (lt(lhs, 0.0)) {
      const double gp = gamma_at<kBatch>(a, i) * cell.p;
      bool decided = false;
      if (fp32_safe(lhs) && fp32_safe(gp) && fp32_safe(cell.d)) {
        const float rhs_f = narrow(a.delta_v) * sqrtf(narrow(gp) / narrow(cell.d));
        const float l_f = -narrow(lhs);
        if (l_f > rhs_f * 1.000002f) {
          shock = true;
          decided = true;
        } else if (l_f < rhs_f * 0.999998f) {
          decided = true;
        }
      }
      if (!decided) shock = lhs < (-a.delta_v) * root(quot(gp, cell.d));
    }
    if (!shock && nn == 0) shock = 1.0 < a.delta_p;  // PressureRatio of no neighbours is 1
    if (!shock) {
      // PressureRatio < delta_p  <=>  some neighbour's ratio < delta_p
      const float dp_f = narrow(a.delta_p);
      for (int k = 0; k < nn && !shock; ++k) {
        const double np_ = point_state(a, static_cast<int>(a.geom.nbr[b + k] & kNbrIdMask)).p;
        const bool lower = lt(np_, cell.p);
        const double num = lower ? np_ : cell.p;
        const double den = lower ? cell.p : np_;
        if (fp32_safe(num) && fp32_safe(den)) {
          const float rf = narrow(num) / narrow(den);
          if (rf < dp_f * 0.999999f) {
            shock = true;
            break;
          }
          if (rf > dp_f * 1.000001f) continue;
        }
        shock = lt(quot(num, den), a.delta_p);
      }
    }
    if (a.shock) a.shock[i] = shock ? 1 : 0;
    // neighbour extrema as bit patterns (std::max / std::min on the integer pipe)
    uint64_t mx[4] = {conv_dbits(cell.d), conv_dbits(cell.p), conv_dbits(cell.vx), conv_dbits(cell.vy)};
    uint64_t mn[4] = {mx[0], mx[1], mx[2], mx[3]};
    for (int k = 0; k < nn; ++k) {
      const uint32_t w = a.geom.nbr[b + k];
      if (!shock && (w & kNbrMirror)) continue;  // :194-195 skips self-mirror neighbours
      if (skipped(a, static_cast<int>(w & kNbrIdMask))) continue;  // :192-193, :314-315 skip_key
      const Cell nb = point_state(a, static_cast<int>(w & kNbrIdMask));
      const uint64_t nbb[4] = {conv_dbits(nb.d), conv_dbits(nb.p), conv_dbits(nb.vx), conv_dbits(nb.vy)};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        mx[q] = max_first_u(mx[q], nbb[q]);
        mn[q] = min_first_u(mn[q], nbb[q]);
      }
    }
    const Cell maxd{conv_double_bits(mx[0]) - cell.d, conv_double_bits(mx[1]) - cell.p,
                    conv_double_bits(mx[2]) - cell.vx, conv_double_bits(mx[3]) - cell.vy};
    const Cell mind{conv_double_bits(mn[0]) - cell.d, conv_double_bits(mn[1]) - cell.p,
                    conv_double_bits(mn[2]) - cell.vx, conv_double_bits(mn[3]) - cell.vy};
    const double f = shock ? 0.1 : 0.05;
    const Cell thr{f * conv_double_bits(max_first_u(abs_u(maxd.d), abs_u(mind.d))),
                   f * conv_double_bits(max_first_u(abs_u(maxd.p), abs_u(mind.p))),
                   f * conv_double_bits(max_first_u(abs_u(maxd.vx), abs_u(mind.vx))),
                   f * conv_double_bits(max_first_u(abs_u(maxd.vy), abs_u(mind.vy)))};
    uint64_t psi0 = kOneBits, psi1 = kOneBits, psi2 = kOneBits, psi3 = kOneBits;
    float pf0 = 1, pf1 = 1, pf2 = 1, pf3 = 1;
    for (int k = 0; k < nn; ++k) {
      const uint32_t w = a.geom.nbr[b + k];
      if (shock && skipped(a, static_cast<int>(w & kNbrIdMask))) continue;  // :339-340
      const int e = m.cell_faces[b + k];
      const double2 dm = centroid_offset(a.geom, w, e);
      Cell cv = cell;
      addmult(cv, sx, dm.x);
      addmult(cv, sy, dm.y);
      const Cell dphi{cv.d - cell.d, cv.p - cell.p, cv.vx - cell.vx, cv.vy - cell.vy};
      if (!shock) {
        // :174-300 slope_limit
        limit_comp(dphi.d, cv.d, cell.d, thr.d, maxd.d, mind.d, false, psi0, pf0);
        limit_comp(dphi.p, cv.p, cell.p, thr.p, maxd.p, mind.p, false, psi1, pf1);
        limit_comp(dphi.vx, cv.vx, cell.vx, thr.vx, maxd.vx, mind.vx, true, psi2, pf2);
        limit_comp(dphi.vy, cv.vy, cell.vy, thr.vy, maxd.vy, mind.vy, true, psi3, pf3);
      } else {
        // :302-399 shocked_slope_limit
        const Cell nb = point_state(a, static_cast<int>(w & kNbrIdMask));
        shocked_comp(dphi.d, cv.d, cell.d, thr.d, nb.d, a.theta, psi0, pf0);
        shocked_comp(dphi.p, cv.p, cell.p, thr.p, nb.p, a.theta, psi1, pf1);
        shocked_comp(dphi.vx, cv.vx, cell.vx, thr.vx, nb.vx, a.theta, psi2, pf2);
        shocked_comp(dphi.vy, cv.vy, cell.vy, thr.vy, nb.vy, a.theta, psi3, pf3);
      }
    }
    const double p0 = conv_double_bits(psi0), p1 = conv_double_bits(psi1), p2 = conv_double_bits(psi2),
                 p3 = conv_double_bits(psi3);
    sx.d *= p0; sy.d *= p0;
    sx.p *= p1; sy.p *= p1;
    sx.vx *= p2; sy.vx *= p2;
    sx.vy *= p3; sy.vy *= p3;
  }
  double2* o = reinterpret_cast<double2*>(a.slopes) + 4 * i;
  o[0] = make_double2(sx.d, sx.p);
  o[1] = make_double2(sx.vx, sx.vy);
  o[2] = make_double2(sy.d, sy.p);
  o[3] = make_double2(sy.vx, sy.vy);
}

// kMinBlocks > 0: register-capped builds for blocks of up to kCappedBlock
// threads with kMinBlocks resident per SM (launch-shape variants 2 and 3)
template <bool kBatch, int kMinBlocks = 0>
__global__ void __launch_bounds__(kMinBlocks ? kCappedBlock : kMaxBlock, kMinBlocks ? kMinBlocks : 1)
    k_slopes(StepArgs a) {
  // the dt of this step, computed by the previous step's update (the face
  // kernel, launched after this one, reads status->dt)
  if (a.take_next_dt && blockIdx.x == 0 && threadIdx.x == 0) a.status->dt = a.status->dt_next;
  const int* order = a.geom.cell_order;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < a.mesh.n; t += gridDim.x * blockDim.x)
    k_slopes_item<kBatch>(a, order ? order[t] : t);
}

// ---------------------------------------------------------------- faces

// simple_flux_calculator.cpp:9-15 convert_to_primitive (ideal_gas.cpp:13-16, 40-44)
__device__ __forceinline__ Prim to_prim(double g, const Cell& c) {
  return Prim{c.d, c.p, c.vx, c.vy, quot(quot(c.p, c.d), g - 1), root(quot(g * c.p, c.d))};
}

// simple_flux_calculator.cpp:130-165 rotate / Hllc / rotate_back
__device__ __forceinline__ bool solve_face(Prim l, Prim r, double velocity, double2 n, double na, double2 p,
                                           double pa, Cons& out, const StepArgs& a, int face) {
  const double lx = quot(l.vx * n.x + l.vy * n.y, na), ly = quot(l.vx * p.x + l.vy * p.y, pa);
  const double rx = quot(r.vx * n.x + r.vy * n.y, na), ry = quot(r.vx * p.x + r.vy * p.y, pa);
  l.vx = lx;
  l.vy = ly;
  r.vx = rx;
  r.vy = ry;
  Cons c;
  if (!hllc(l, r, velocity, c, a.status, a.step, face)) return false;
  out.m = c.m;
  out.mx = quot(n.x * c.mx, na) + quot(p.x * c.my, pa);
  out.my = quot(n.y * c.mx, na) + quot(p.y * c.my, pa);
  out.en = c.en;
  return true;
}

// rotate / LagrangianHLLC / rotate_back (LagrangianFlux, condition_action_sequence_2.cpp:284-290)
__device__ __forceinline__ bool solve_face_lagrangian(Prim l, Prim r, double velocity, bool massflux, double2 n,
                                                      double na, double2 p, double pa, Cons& out, double& energy,
                                                      const StepArgs& a, int face) {
  const double lx = quot(l.vx * n.x + l.vy * n.y, na), ly = quot(l.vx * p.x + l.vy * p.y, pa);
  const double rx = quot(r.vx * n.x + r.vy * n.y, na), ry = quot(r.vx * p.x + r.vy * p.y, pa);
  l.vx = lx;
  l.vy = ly;
  r.vx = rx;
  r.vy = ry;
  Cons c;
  if (!lagrangian_hllc(l, r, velocity, massflux, c, energy, a.status, a.step, face)) return false;
  out.m = c.m;
  out.mx = quot(n.x * c.mx, na) + quot(p.x * c.my, pa);
  out.my = quot(n.y * c.mx, na) + quot(p.y * c.my, pa);
  out.en = c.en;
  return true;
}

template <bool kBatch>
__device__ __forceinline__ void write_flux(const StepArgs& a, int e, int real_side, const Cons& c, bool scaled,
                                           double area) {
  if (scaled) {
    const double s = scaled_dt<kBatch>(a, real_side) * area;  // simple_extensive_updater.cpp:26-27
    store4(a.fluxes, e, c.m * s, c.en * s, c.mx * s, c.my * s);
  } else {
    store4(a.fluxes, e, c.m, c.en, c.mx, c.my);
  }
}

// ModularFluxCalculator (modular_flux_calculator.cpp:39-71) with the face
// states of LinearGaussImproved (:570-590 real sides, :596-634 ghost sides).
template <bool kScaled, bool kBatch>
__device__ __forceinline__ void k_faces_lgi_item(const StepArgs& a, int e) {
  const MeshDev& m = a.mesh;
  const int2 fc = m.face_cells[e];
  Cell side[2];
  const int ids[2] = {fc.x, fc.y};
  const double2 dms[2] = {a.geom.dm0[e], a.geom.dm1[e]};
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const int pid = ids[s];
    Cell c = point_state(a, pid);
    int sid = pid;
    bool zero = false;
    if (pid >= m.n) {
      if (a.ghost_kind == RG_GHOST_PERIODIC)
        sid = m.ghost_source[pid - m.n];  // PeriodicGhostGenerator.cpp:19-24
      else
        zero = true;  // RigidWallGenerator.cpp:39-54: zero gradient
    }
    Cell gx{0, 0, 0, 0}, gy{0, 0, 0, 0};
    if (!zero) {
      const double2* sp = reinterpret_cast<const double2*>(a.slopes) + 4 * sid;
      const double2 s0 = sp[0], s1 = sp[1], s2 = sp[2], s3 = sp[3];
      gx = Cell{s0.x, s0.y, s1.x, s1.y};
      gy = Cell{s2.x, s2.y, s3.x, s3.y};
    }
    addmult(c, gx, dms[s].x);
    addmult(c, gy, dms[s].y);
    side[s] = c;
  }
  const double2 w = a.ev_zero ? make_double2(0.0, 0.0) : reinterpret_cast<const double2*>(a.ev)[e];
  const double2 n = a.geom.nrm[e], p = a.geom.par[e];
  const double na = a.geom.nabs[e], pa = a.geom.area[e];
  // a face at rest has speed +-0 (the sign only reaches signs of zeros)
  const double speed = (w.x == 0.0 && w.y == 0.0) ? 0.0 : quot(n.x * w.x + n.y * w.y, na);
  const int real_side = fc.x < m.n ? fc.x : fc.y;
  const double g = gamma_at<kBatch>(a, real_side);
  Cons c;
  if (!solve_face(to_prim(g, side[0]), to_prim(g, side[1]), speed, n, na, p, pa, c, a, e)) return;
  if (a.mflux) a.mflux[e] = c.m;
  write_flux<kBatch>(a, e, real_side, c, kScaled, a.geom.xarea[e]);
}

template <bool kScaled, bool kBatch>
__global__ void __launch_bounds__(kMaxBlock) k_faces_lgi(StepArgs a) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < a.mesh.e; e += gridDim.x * blockDim.x)
    k_faces_lgi_item<kScaled, kBatch>(a, e);
}

// simple_flux_calculator.cpp:17-25 reflect (Reflect, geometry.cpp:117-120);
// keeps the source's energy and sound speed.
__device__ __forceinline__ Prim reflect(Prim q, double2 axis, double aa) {
  const double s = 2 * (q.vx * axis.x + q.vy * axis.y);
  const double pp = aa * aa;
  const double tx = quot(axis.x * s, pp), ty = quot(axis.y * s, pp);
  q.vx = tx - q.vx;
  q.vy = ty - q.vy;
  return q;
}

// SimpleFluxCalculator (simple_flux_calculator.cpp:80-126 riemann_reduce,
// :216-244).  A ghost that is not its neighbour's own mirror takes its source
// cell's state.
template <bool kScaled, bool kBatch>
__device__ __forceinline__ void k_faces_pcm_item(const StepArgs& a, int e) {
  const MeshDev& m = a.mesh;
  const int2 fc = m.face_cells[e];
  const double2 p = a.geom.par[e], n = a.geom.nrm[e];
  const double pa = a.geom.area[e], na = a.geom.nabs[e];
  const bool va = fc.x < m.n, vb = fc.y < m.n;
  const int oa = orig_of(m, fc.x), ob = orig_of(m, fc.y);
  const int real_side = va ? fc.x : fc.y;
  const double g = gamma_at<kBatch>(a, real_side);
  Prim l, r;
  if (!va) {
    r = to_prim(g, load_cell(a.cells, fc.y));
    l = oa == ob ? reflect(r, p, pa) : to_prim(g, load_cell(a.cells, oa));
  } else if (!vb) {
    l = to_prim(g, load_cell(a.cells, fc.x));
    r = oa == ob ? reflect(l, p, pa) : to_prim(g, load_cell(a.cells, ob));
  } else {
    l = to_prim(g, load_cell(a.cells, fc.x));
    r = to_prim(g, load_cell(a.cells, fc.y));
  }
  const double2 w = a.ev_zero ? make_double2(0.0, 0.0) : reinterpret_cast<const double2*>(a.ev)[e];
  const double velocity = (w.x == 0.0 && w.y == 0.0) ? 0.0 : quot(n.x * w.x + n.y * w.y, na);
  Cons c;
  if (!solve_face(l, r, velocity, n, na, p, pa, c, a, e)) return;
  if (a.mflux) a.mflux[e] = c.m;
  write_flux<kBatch>(a, e, real_side, c, kScaled, a.geom.xarea[e]);
}

template <bool kScaled, bool kBatch>
__global__ void __launch_bounds__(kMaxBlock) k_faces_pcm(StepArgs a) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < a.mesh.e; e += gridDim.x * blockDim.x)
    k_faces_pcm_item<kScaled, kBatch>(a, e);
}

// ---------------------------------------------------------------- condition/action fluxes

// geometry.cpp normalize: v/abs(v)
__device__ __forceinline__ double2 normalize2(double x, double y) {
  const double ab = root(x * x + y * y);
  return make_double2(quot(x, ab), quot(y, ab));
}
// simple_flux_calculator.cpp:27-31 remove_parallel_component, then normalize
__device__ __forceinline__ double2 wall_normal(double wx, double wy, double2 p) {
  const double s = wx * p.x + wy * p.y, pp = p.x * p.x + p.y * p.y;
  return normalize2(wx - quot(p.x * s, pp), wy - quot(p.y * s, pp));
}
__device__ __forceinline__ bool has_sticker(const StepArgs& a, int p, int bit) {
  return a.stickers != nullptr && ((a.stickers[orig_of(a.mesh, p)] >> bit) & 1u) != 0;
}

// One face of ConditionActionSequence (condition_action_sequence.cpp:17-61)
// or ConditionActionSequence2 (condition_action_sequence_2.cpp:40-127): the
// first rule of sequence 0, else of sequence 1, whose condition holds picks
// the action; cell states are the cells' own records (a periodic ghost reads
// its source cell), face states LinearGaussImproved's (order 2).
template <bool kScaled>
__device__ __forceinline__ void k_faces_cas_item(const StepArgs& a, int e) {
  const MeshDev& m = a.mesh;
  const int2 fc = m.face_cells[e];
  int chosen = -1;
  bool aux = false;
  for (int pass = 0; pass < 2 && chosen < 0; ++pass) {
    for (int k = 0; k < a.n_rules && chosen < 0; ++k) {
      if (a.rules[k][0] != pass) continue;
      const int cond = a.rules[k][1];
      bool applies = false, ax = false;
      if (cond == RG_COND_BOUNDARY_EDGE) {  // :228-253, serial build
        if (fc.x >= m.n) applies = true;
        else if (fc.y >= m.n) applies = ax = true;
      } else if (cond == RG_COND_BULK_EDGE) {  // :255-271
        applies = (fc.x < m.n && fc.y < m.n) || orig_of(m, fc.x) != orig_of(m, fc.y);
      } else {  // :273-289 RegularSpecialEdge: exactly one side carries the sticker
        const bool sa = has_sticker(a, fc.x, a.rules[k][2]), sb = has_sticker(a, fc.y, a.rules[k][2]);
        applies = sa ? !sb : sb;
        ax = !sa && sb;
      }
      if (applies) {
        chosen = k;
        aux = ax;
      }
    }
  }
  if (a.tr_side) a.tr_side[e] = 0;  // no tracer flux unless an action sets one
  if (chosen < 0) {  // "Error in ConditionActionSequence"
    record_error(a.status, a.step, RG_ERR_INVALID_ARGUMENT, 3, e, 0.0);
    return;
  }
  if (a.lag_ws) {
    // LagrangianFlux::Reset: faces of other actions carry no ws / speed
    a.lag_ws[e] = 0.0;
    a.lag_ev[e] = 0.0;
  }
  const dbl4 v = m.face_vertices[e];
  const double2 p = normalize2(v.z - v.x, v.w - v.y);
  const double pa = root(p.x * p.x + p.y * p.y);
  const double g = a.gamma;
  const Cell c0 = load_cell(a.cells, orig_of(m, fc.x)), c1 = load_cell(a.cells, orig_of(m, fc.y));
  int action = a.rules[chosen][3];
  if (action == RG_ACT_RATCHET) {
    // condition_action_sequence_2.cpp:232-249
    const double2 x0 = m.points[fc.x], x1 = m.points[fc.y];
    const double nx = aux ? x1.x - x0.x : x0.x - x1.x, ny = aux ? x1.y - x0.y : x0.y - x1.y;
    const Cell& sc = aux ? c0 : c1;
    const double sign = 2.0 * (a.rules[chosen][4] != 0 ? 1.0 : 0.0) - 1.0;
    action = (nx * sc.vx + ny * sc.vy) * sign < 0 ? RG_ACT_FREE_FLOW : RG_ACT_RIGID_WALL2;
  }
  // LinearGaussImproved face states (order 2), as k_faces_lgi_item forms them
  Cell s0 = c0, s1 = c1;
  if (action == RG_ACT_REGULAR2 || action == RG_ACT_RIGID_WALL2 || action == RG_ACT_LAGRANGIAN) {
    const int ids[2] = {fc.x, fc.y};
    const double2 dms[2] = {a.geom.dm0[e], a.geom.dm1[e]};
    Cell side[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int pid = ids[s];
      Cell c = point_state(a, pid);
      int sid = pid;
      bool zero = false;
      if (pid >= m.n) {
        if (a.ghost_kind == RG_GHOST_PERIODIC)
          sid = m.ghost_source[pid - m.n];
        else
          zero = true;
      }
      Cell gx{0, 0, 0, 0}, gy{0, 0, 0, 0};
      if (!zero) {
        const double2* sp = reinterpret_cast<const double2*>(a.slopes) + 4 * sid;
        const double2 q0 = sp[0], q1 = sp[1], q2 = sp[2], q3 = sp[3];
        gx = Cell{q0.x, q0.y, q1.x, q1.y};
        gy = Cell{q2.x, q2.y, q3.x, q3.y};
      }
      addmult(c, gx, dms[s].x);
      addmult(c, gy, dms[s].y);
      side[s] = c;
    }
    s0 = side[0];
    s1 = side[1];
  }
  if (action == RG_ACT_LAGRANGIAN) {
    // condition_action_sequence_2.cpp:270-294: ModularFluxCalculator's frame
    // and face speed, WallsMassFlux (:300-312) picking rs or rs2
    const double2 w = a.ev_zero ? make_double2(0.0, 0.0) : reinterpret_cast<const double2*>(a.ev)[e];
    const double2 nn = a.geom.nrm[e], pp = a.geom.par[e];
    const double na = a.geom.nabs[e], ppa = a.geom.area[e];
    const double speed = (w.x == 0.0 && w.y == 0.0) ? 0.0 : quot(nn.x * w.x + nn.y * w.y, na);
    const bool lag = orig_of(m, fc.x) != orig_of(m, fc.y);
    const bool mf = (((lag ? a.rules[chosen][5] : a.rules[chosen][5] >> 1)) & 1) != 0;
    Cons c;
    double energy = 0.0;
    if (!solve_face_lagrangian(to_prim(g, s0), to_prim(g, s1), speed, mf, nn, na, pp, ppa, c, energy, a, e)) return;
    if (a.lag_ws) {
      a.lag_ws[e] = lag ? energy : 0.0;
      a.lag_ev[e] = speed;
    }
    // convert_conserved_to_extensive (:29-40): Mass * the face value upwind
    if (a.tr_side) {
      a.mflux[e] = c.m;
      a.tr_side[e] = kTrSideFace | (c.m > 0 ? kTrSideFirst : kTrSideSecond);
    }
    write_flux<false>(a, e, fc.x < m.n ? fc.x : fc.y, c, kScaled, a.geom.xarea[e]);
    return;
  }
  Prim l, r;
  double2 n;
  double vel = 0;
  if (action == RG_ACT_REGULAR || action == RG_ACT_REGULAR2) {
    // condition_action_sequence.cpp:84-110, condition_action_sequence_2.cpp:129-157
    const double2 x0 = m.points[fc.x], x1 = m.points[fc.y];
    n = normalize2(x1.x - x0.x, x1.y - x0.y);
    const double2 w = a.ev_zero ? make_double2(0.0, 0.0) : reinterpret_cast<const double2*>(a.ev)[e];
    vel = n.x * w.x + n.y * w.y;
    l = to_prim(g, action == RG_ACT_REGULAR ? c0 : s0);
    r = to_prim(g, action == RG_ACT_REGULAR ? c1 : s1);
  } else {
    // RigidWallFlux / RigidWallFlux2 / FreeFlowFlux: the wall frame
    const double2 x0 = m.points[fc.x], x1 = m.points[fc.y];
    n = aux ? wall_normal(v.x - x0.x, v.y - x0.y, p) : wall_normal(x1.x - v.x, x1.y - v.y, p);
    if (action == RG_ACT_FREE_FLOW) {
      l = r = to_prim(g, aux ? c0 : c1);
    } else {
      const Prim q = to_prim(g, action == RG_ACT_RIGID_WALL ? (aux ? c0 : c1) : (aux ? s0 : s1));
      if (aux) {
        l = q;
        r = reflect(q, p, pa);
      } else {
        r = q;
        l = reflect(q, p, pa);
      }
    }
  }
  const double na = root(n.x * n.x + n.y * n.y);
  Cons c;
  if (!solve_face(l, r, vel, n, na, p, pa, c, a, e)) return;
  if (a.tr_side) {
    // the tracer flux is Mass times the tracers of: the upwind cell
    // (RegularFlux, condition_action_sequence.cpp:110-114) or face value
    // (RegularFlux2, condition_action_sequence_2.cpp:156), the cell on the
    // aux side (RigidWallFlux, FreeFlowFlux: :178, :221) or its face value
    // (RigidWallFlux2, condition_action_sequence_2.cpp:221)
    a.mflux[e] = c.m;
    const bool regular = action == RG_ACT_REGULAR || action == RG_ACT_REGULAR2;
    const bool face = action == RG_ACT_REGULAR2 || action == RG_ACT_RIGID_WALL2;
    const bool first = regular ? c.m > 0 : aux;
    a.tr_side[e] = (face ? kTrSideFace : 0) | (first ? kTrSideFirst : kTrSideSecond);
  }
  const int real_side = fc.x < m.n ? fc.x : fc.y;
  write_flux<false>(a, e, real_side, c, kScaled, a.geom.xarea[e]);
}

template <bool kScaled>
__global__ void __launch_bounds__(kMaxBlock) k_faces_cas(StepArgs a) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < a.mesh.e; e += gridDim.x * blockDim.x)
    k_faces_cas_item<kScaled>(a, e);
}

// ---------------------------------------------------------------- cells

// The next step's SimpleCFL bound of cell i with state (d, pres, vx, vy), as
// k_cfl computes it, as the bit pattern of 1/bound.
template <bool kBatch>
__device__ __forceinline__ unsigned long long cfl_bound_bits(const StepArgs& a, int i, double d, double pres,
                                                             double vx, double vy) {
  const MeshDev& m = a.mesh;
  const double cs = root(quot(gamma_at<kBatch>(a, i) * pres, d));
  double q = 0;
  bool any = false;
  if (a.ev_zero) {
    const double qq = vx * vx + vy * vy;
    if (m.cell_off[i + 1] > m.cell_off[i] && !isnan(qq)) {
      q = fmax(q, qq);
      any = true;
    }
  } else {
    for (int k = m.cell_off[i]; k < m.cell_off[i + 1]; ++k) {
      const double2 w = reinterpret_cast<const double2*>(a.ev)[m.cell_faces[k]];
      const double dx = vx - w.x, dy = vy - w.y;
      const double qq = dx * dx + dy * dy;
      if (!isnan(qq)) {
        q = fmax(q, qq);
        any = true;
      }
    }
  }
  const double res = any ? fmax(0.0, quot(cs + root(q), a.geom.width[i])) : 0.0;
  return static_cast<unsigned long long>(__double_as_longlong(quot(1.0, res)));
}

// SimpleExtensiveUpdater (simple_extensive_updater.cpp:11-35) as a gather:
// each cell applies its faces' contributions in ascending face order, which
// is the order the reference's edge loop applies them to that cell; then
// SimpleCellUpdater::regular_update (simple_cell_updater.cpp:22-59).
template <bool kBatch>
__device__ __forceinline__ unsigned long long k_update_item(const StepArgs& a, int i, int from_unscaled, int do_ext,
                                                         int do_cells) {
  const MeshDev& m = a.mesh;
  double2* ext2 = reinterpret_cast<double2*>(a.ext);
  double2 e01 = ext2[2 * i], e23 = ext2[2 * i + 1];
  double mass = e01.x, en = e01.y, px = e23.x, py = e23.y;
  if (do_ext) {
    const double dt = from_unscaled ? step_dt(a) : 0.0;
    const int b = m.cell_off[i], e1 = m.cell_off[i + 1];
    for (int k = b; k < e1; ++k) {
      const int e = m.cell_faces[k];
      const double2* f = reinterpret_cast<const double2*>(a.fluxes) + 2 * e;
      const double2 f01 = f[0], f23 = f[1];
      double dm = f01.x, de = f01.y, dx = f23.x, dy = f23.y;
      if (from_unscaled) {
        const double s = dt * a.geom.xarea[e];
        dm *= s;
        de *= s;
        dx *= s;
        dy *= s;
      }
      if (a.geom.nbr[k] & kNbrFirst) {
        mass -= dm;
        en -= de;
        px -= dx;
        py -= dy;
      } else {
        mass += dm;
        en += de;
        px += dx;
        py += dy;
      }
    }
    if (a.lag_update) {
      const double f = lag_factor(a, i);
      mass *= f;
      en *= f;
      px *= f;
      py *= f;
    }
    if (a.ext_avg) {
      // hdsim2d.cpp:311-320 average_extensive: 0.5*(mid + old)
      const double2* o = reinterpret_cast<const double2*>(a.ext_avg);
      const double2 o01 = o[2 * i], o23 = o[2 * i + 1];
      mass = 0.5 * (mass + o01.x);
      en = 0.5 * (en + o01.y);
      px = 0.5 * (px + o23.x);
      py = 0.5 * (py + o23.y);
    }
    double2* out2 = reinterpret_cast<double2*>(a.ext_out ? a.ext_out : a.ext);
    out2[2 * i] = make_double2(mass, en);
    out2[2 * i + 1] = make_double2(px, py);
  }
  if (do_cells) {
    if (a.frozen_mask && (a.stickers[i] & a.frozen_mask)) {
      // simple_cell_updater.cpp:61-83 with (HasSticker, SkipUpdate): the old
      // cell stays (its extensives above still took the fluxes)
      const Cell c = load_cell(a.cells, i);
      if (a.cells_out) store4(a.cells_out, i, c.d, c.p, c.vx, c.vy);
      if (!a.cfl_next) return kInfBits;
      return cfl_bound_bits<kBatch>(a, i, c.d, c.p, c.vx, c.vy);
    }
    const double d = quot(mass, m.cd_volume[i]);
    if (d < 0) {
      record_error(a.status, a.step, RG_ERR_NEGATIVE_DENSITY, 5, i, d);
      return kInfBits;
    }
    const double vx = quot(px, mass), vy = quot(py, mass);
    const double energy = quot(en, mass) - 0.5 * (vx * vx + vy * vy);
    if (energy < 0) {
      record_error(a.status, a.step, RG_ERR_NEGATIVE_ENERGY, 5, i, energy);
      return kInfBits;
    }
    const double pres = (gamma_at<kBatch>(a, i) - 1) * energy * d;
    store4(a.cells_out ? a.cells_out : a.cells, i, d, pres, vx, vy);
    // the next step's SimpleCFL bound of this cell, from the record just stored
    if (a.cfl_next) return cfl_bound_bits<kBatch>(a, i, d, pres, vx, vy);
  }
  return kInfBits;
}

template <bool kBatch>
__global__ void __launch_bounds__(kMaxBlock) k_update(StepArgs a, int from_unscaled, int do_ext, int do_cells) {
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  if (kBatch && do_ext && !from_unscaled && !a.batch_keep_dt) {
    for (int p = t0; p < a.n_problems; p += stride) {
      // every face of this step has read its problem's minimum: record the dt,
      // advance the problem's time and reset the minimum for the next step
      const double dt = a.cfl * __longlong_as_double(static_cast<long long>(a.dtmin_p[p]));
      a.dt_p[p] = dt;
      a.time_p[p] += dt;
      a.dtmin_p[p] = kInfBits;
    }
  }
  unsigned long long bits = kInfBits;
  const int* order = a.geom.cell_order;
  for (int t = t0; t < a.mesh.n; t += stride) {
    const unsigned long long b = k_update_item<kBatch>(a, order ? order[t] : t, from_unscaled, do_ext, do_cells);
    bits = b < bits ? b : bits;
  }
  if (!kBatch && a.cfl_next) grid_min_times(a.status, bits, a.cfl, &a.status->dt_next);
}

// hdsim2d.cpp:41-67 init_extensives
template <bool kBatch>
__global__ void __launch_bounds__(kBlock) k_init_ext(StepArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.mesh.n) return;
  const Cell c = load_cell(a.cells, i);
  const double mass = a.mesh.cd_volume[i] * c.d;
  store4(a.ext, i, mass, quot(quot(c.p, c.d), gamma_at<kBatch>(a, i) - 1) * mass + 0.5 * mass * (c.vx * c.vx + c.vy * c.vy),
         c.vx * mass, c.vy * mass);
}

// *flag = 1 if any of v[0..n) is not +-0 (NaN counts as nonzero)
__global__ void __launch_bounds__(kBlock) k_any_nonzero(const double* v, long long n, int* flag) {
  bool any = false;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    any = any || !(v[i] == 0.0);
  if (__any_sync(0xffffffffu, any) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

inline int blocks(int n) { return (n + kBlock - 1) / kBlock; }

}  // namespace

// Problem of every point of a batch (real cells by the offset table, ghosts by
// their source cell) and the check that no face joins two problems.
__global__ void __launch_bounds__(kBlock) k_problems(MeshDev m, const int* offsets, int P, int* cell_problem,
                                                     DevStatus* st) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < m.n) {
    int lo = 0, hi = P;  // largest p with offsets[p] <= t
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (offsets[mid] <= t) lo = mid; else hi = mid;
    }
    cell_problem[t] = lo;
  }
  __syncthreads();
  if (t < m.g) {
    const int src = m.ghost_source[t];
    int lo = 0, hi = P;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (offsets[mid] <= src) lo = mid; else hi = mid;
    }
    cell_problem[m.n + t] = lo;
  }
}

__global__ void __launch_bounds__(kBlock) k_check_problems(MeshDev m, const int* cell_problem, DevStatus* st) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < m.e) {
    const int2 fc = m.face_cells[t];
    if (cell_problem[fc.x] != cell_problem[fc.y]) record_error(st, 0, RG_ERR_INVALID_ARGUMENT, 0, t, fc.y);
  }
}

cudaError_t launch_problems(const MeshDev& m, const int* offsets, int P, int* cell_problem, DevStatus* st,
                            cudaStream_t s) {
  const int work = m.n > m.g ? m.n : m.g;
  k_problems<<<blocks(work > 0 ? work : 1), kBlock, 0, s>>>(m, offsets, P, cell_problem, st);
  if (m.e > 0) k_check_problems<<<blocks(m.e), kBlock, 0, s>>>(m, cell_problem, st);
  return cudaGetLastError();
}

cudaError_t launch_any_nonzero(const double* v, long long n, int* flag, cudaStream_t s) {
  if (n > 0) {
    const long long nb = (n + kBlock - 1) / kBlock;
    k_any_nonzero<<<static_cast<int>(nb < 4096 ? nb : 4096), kBlock, 0, s>>>(v, n, flag);
  }
  return cudaGetLastError();
}

cudaError_t launch_validate(const MeshDev& m, DevStatus* st, cudaStream_t s) {
  int work = m.e > m.n ? m.e : m.n;
  work = work > m.g ? work : m.g;
  k_validate<<<blocks(work > 0 ? work : 1), kBlock, 0, s>>>(m, st);
  return cudaGetLastError();
}

cudaError_t launch_cell_order(const MeshDev& m, int* order, int* cflags, cudaStream_t s) {
  if (m.n > 0) k_cell_order<<<(m.n + kOrderTile - 1) / kOrderTile, kOrderTile, 0, s>>>(m, order, cflags);
  return cudaGetLastError();
}

cudaError_t launch_geometry(const GeomArgs& a, cudaStream_t s) {
  if (a.mesh.e > 0) k_geom_faces<<<blocks(a.mesh.e), kBlock, 0, s>>>(a);
  if (a.mesh.n > 0) k_geom_cells<<<blocks(a.mesh.n), kBlock, 0, s>>>(a);
  if (a.mesh.g > 0) k_geom_ghosts<<<blocks(a.mesh.g), kBlock, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_geom_ghosts(const GeomArgs& a, cudaStream_t s) {
  if (a.mesh.g > 0) k_geom_ghosts<<<blocks(a.mesh.g), kBlock, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_cfl(const StepArgs& a, cudaStream_t s, bool fill_ghosts) {
  const int total = a.mesh.n + (fill_ghosts ? a.mesh.g : 0);
  if (a.cell_problem)
    k_cfl<true><<<grid_of(a.shapes.cfl, total), a.shapes.cfl.block, 0, s>>>(a, fill_ghosts ? 1 : 0);
  else
    k_cfl<false><<<grid_of(a.shapes.cfl, total), a.shapes.cfl.block, 0, s>>>(a, fill_ghosts ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_ghost_fill(const StepArgs& a, cudaStream_t s) {
  if (a.mesh.g > 0) k_ghost_fill<<<blocks(a.mesh.g), kBlock, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_slopes(const StepArgs& a, cudaStream_t s) {
  if (a.mesh.n > 0) {
    const LaunchShape& sh = a.shapes.slopes;
    const int nb = grid_of(sh, a.mesh.n), bs = sh.block;
    const bool b = a.cell_problem != nullptr;
    // builds: 0 plain, 2 and 3 register-capped for 3 and 4 resident blocks of
    // up to 256 threads
    switch (sh.variant) {
      case 2: b ? k_slopes<true, 3><<<nb, bs, 0, s>>>(a) : k_slopes<false, 3><<<nb, bs, 0, s>>>(a); break;
      case 3: b ? k_slopes<true, 4><<<nb, bs, 0, s>>>(a) : k_slopes<false, 4><<<nb, bs, 0, s>>>(a); break;
      default: b ? k_slopes<true><<<nb, bs, 0, s>>>(a) : k_slopes<false><<<nb, bs, 0, s>>>(a);
    }
  }
  return cudaGetLastError();
}

cudaError_t launch_faces(const StepArgs& a, cudaStream_t s, bool scaled) {
  if (a.mesh.e == 0) return cudaSuccess;
  const int nb = grid_of(a.shapes.faces, a.mesh.e), bs = a.shapes.faces.block;
  const bool b = a.cell_problem != nullptr;
  if (a.n_rules > 0) {
    scaled ? k_faces_cas<true><<<nb, bs, 0, s>>>(a) : k_faces_cas<false><<<nb, bs, 0, s>>>(a);
    return cudaGetLastError();
  }
  if (a.order == 1) {
    if (scaled)
      b ? k_faces_pcm<true, true><<<nb, bs, 0, s>>>(a) : k_faces_pcm<true, false><<<nb, bs, 0, s>>>(a);
    else
      b ? k_faces_pcm<false, true><<<nb, bs, 0, s>>>(a) : k_faces_pcm<false, false><<<nb, bs, 0, s>>>(a);
  } else {
    if (scaled)
      b ? k_faces_lgi<true, true><<<nb, bs, 0, s>>>(a) : k_faces_lgi<true, false><<<nb, bs, 0, s>>>(a);
    else
      b ? k_faces_lgi<false, true><<<nb, bs, 0, s>>>(a) : k_faces_lgi<false, false><<<nb, bs, 0, s>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t launch_update(const StepArgs& a, cudaStream_t s, bool from_unscaled, bool extensive, bool cells) {
  const int work = a.cell_problem && a.n_problems > a.mesh.n ? a.n_problems : a.mesh.n;
  if (work > 0) {
    if (a.cell_problem)
      k_update<true><<<grid_of(a.shapes.update, work), a.shapes.update.block, 0, s>>>(a, from_unscaled ? 1 : 0, extensive ? 1 : 0, cells ? 1 : 0);
    else
      k_update<false><<<grid_of(a.shapes.update, work), a.shapes.update.block, 0, s>>>(a, from_unscaled ? 1 : 0, extensive ? 1 : 0, cells ? 1 : 0);
  }
  return cudaGetLastError();
}

cudaError_t launch_init_extensives(const StepArgs& a, cudaStream_t s) {
  if (a.mesh.n > 0) {
    if (a.cell_problem)
      k_init_ext<true><<<blocks(a.mesh.n), kBlock, 0, s>>>(a);
    else
      k_init_ext<false><<<blocks(a.mesh.n), kBlock, 0, s>>>(a);
  }
  return cudaGetLastError();
}

}  // namespace rg
