// rg_mixed.cu -- FP32-mixed kernels of the hydro hot path for sm_103a.
//
// Reconstruction (LinearGaussImproved / piecewise constant), HLLC and the
// CFL bound run in FP32 (FMA allowed) on FP32 copies of the primitives and of
// the geometry.  The FP32 geometry is formed once per mesh upload from FP64
// coordinate differences (k_geom_faces32, k_geom_cells32), or rounded from
// the FP64 geometry pass (rg_fp64.cu) where FP64 passes run on the same mesh
// (tracers, differentiation).  FP64 stays where the
// precision is needed: cell volumes, the extensive accumulation (each face's
// dt*area-scaled flux is widened to FP64 and summed per cell in ascending
// face order, so every face adds exactly what its neighbour subtracts) and
// the internal energy e = E/m - v^2/2, whose cancellation at high Mach
// numbers FP32 cannot carry.
//
// On GB300 the FP32 pipe issues 128 FFMA/clk/SM against 2 DFMA/clk/SM, so
// this path is bound by memory traffic and by its remaining FP64 work (the
// gather and the energy conversion), not by the flux arithmetic.
#include <math.h>

#include "rg_adjoint.cuh"
#include "rg_convert.cuh"
#include "rg_div.cuh"
#include "rg_mixed.cuh"

namespace rg {
namespace {

constexpr int kBlock = 256;

struct C4 { float d, p, vx, vy; };
struct P6 { float d, p, vx, vy, e, c; };
struct F4 { float m, mx, my, en; };

__device__ __forceinline__ C4 ld4(const float4* a, int i) {
  const float4 v = a[i];
  return C4{v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ void addm(C4& r, const C4& o, float s) {
  r.d = fmaf(o.d, s, r.d);
  r.p = fmaf(o.p, s, r.p);
  r.vx = fmaf(o.vx, s, r.vx);
  r.vy = fmaf(o.vy, s, r.vy);
}

// a*b + c*d and a*b - c*d as one product and one fused multiply-add, written
// out so that every build of the slopes kernel (and its trace) rounds alike
// whatever the compiler would contract
__device__ __forceinline__ float dot2(float a, float b, float c, float d) {
  return __fmaf_rn(c, d, __fmul_rn(a, b));
}
__device__ __forceinline__ float dif2(float a, float b, float c, float d) {
  return __fmaf_rn(-c, d, __fmul_rn(a, b));
}
// the unlimited slope from the neighbour sums vx, vy: boundary cells' least
// squares (mi = SxSy, Sx2, Sy2, den) or the Green-Gauss inverse (mi = the
// 2x2 matrix, row major)
__device__ __forceinline__ void naive_slope(bool boundary, const C4& vx, const C4& vy, const float4& mi, C4& sx,
                                            C4& sy) {
  if (boundary) {
    const float inv = 1.0f / mi.w;
    sx = C4{__fmul_rn(dif2(vy.d, mi.x, vx.d, mi.z), inv), __fmul_rn(dif2(vy.p, mi.x, vx.p, mi.z), inv),
            __fmul_rn(dif2(vy.vx, mi.x, vx.vx, mi.z), inv), __fmul_rn(dif2(vy.vy, mi.x, vx.vy, mi.z), inv)};
    sy = C4{__fmul_rn(dif2(vx.d, mi.x, vy.d, mi.y), inv), __fmul_rn(dif2(vx.p, mi.x, vy.p, mi.y), inv),
            __fmul_rn(dif2(vx.vx, mi.x, vy.vx, mi.y), inv), __fmul_rn(dif2(vx.vy, mi.x, vy.vy, mi.y), inv)};
  } else {
    sx = C4{dot2(vx.d, mi.x, vy.d, mi.y), dot2(vx.p, mi.x, vy.p, mi.y), dot2(vx.vx, mi.x, vy.vx, mi.y),
            dot2(vx.vy, mi.x, vy.vy, mi.y)};
    sy = C4{dot2(vy.d, mi.w, vx.d, mi.z), dot2(vy.p, mi.w, vx.p, mi.z), dot2(vy.vx, mi.w, vx.vx, mi.z),
            dot2(vy.vy, mi.w, vx.vy, mi.z)};
  }
}

// ------------------------------------------------------------ geometry copies
// (the roundings on the integer pipe: rg_convert.cuh)

__global__ void __launch_bounds__(kBlock) k_geom32(MixedGeomArgs a) {
  if (a.invalid && *a.invalid != ~0ull) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int stride = gridDim.x * blockDim.x;
  const GeomDev& g = a.g64;
  for (int e = t; e < a.e; e += stride) {
    const double2 n = g.nrm[e], p = g.par[e], d0 = g.dm0[e], d1 = g.dm1[e];
    a.nrm[e] = make_float2(narrow(n.x), narrow(n.y));
    a.nabs[e] = narrow(g.nabs[e]);
    a.par[e] = make_float2(narrow(p.x), narrow(p.y));
    a.area[e] = narrow(g.area[e]);
    if (a.xarea != a.area) a.xarea[e] = narrow(g.xarea[e]);
    a.dm0[e] = make_float2(narrow(d0.x), narrow(d0.y));
    a.dm1[e] = make_float2(narrow(d1.x), narrow(d1.y));
  }
  for (int i = t; i < a.n; i += stride) {
    a.width[i] = narrow(g.width[i]);
    // the FP32 reciprocal of the rounded volume (an FP64 division would cost
    // more than the rest of the kernel)
    a.inv_cd_volume[i] = __frcp_rn(narrow(a.cd_volume[i]));
    const dbl4 m = g.minv[i];
    a.minv[i] = make_float4(narrow(m.x), narrow(m.y), narrow(m.z), narrow(m.w));
  }
  for (int k = t; k < a.m; k += stride) {
    const double2 h = g.hr[k];
    const int e = a.cell_faces[k];
    const bool first = g.nbr[k] & kNbrFirst;
    const double2 d = first ? g.dm0[e] : g.dm1[e];
    a.ent[k] = make_float4(narrow(h.x), narrow(h.y), narrow(d.x), narrow(d.y));
    a.fsign[k] = e | (first ? static_cast<int>(0x80000000u) : 0);
  }
  for (int q = t; q < a.g; q += stride) {
    const double2 u = g.ghost_unit[q];
    a.ghost_unit[q] = make_float2(narrow(u.x), narrow(u.y));
  }
}

// The FP32-mixed geometry without the FP64 geometry pass.  The face
// geometry is formed in FP64 and rounded once, as the FP64 pass forms it:
// vertex differences (Parallel), areas, centroid offsets (CalcCentroid - CM)
// and |x1 - x0|.  The normal is kept as +-(-p.y, p.x) with |n| = |p|, p the
// FP64 vertex difference: calc_parallel_normal's direction, exact in FP64 and
// bit-equal for the two periodic images of a face (so what one cell loses
// the other gains).  The reconstruction stencil (r_ij, c_ij, the naive
// slope's matrix and inverse, the boundary slope's sums) is formed in FP32,
// as the FP32 reconstruction uses it.  The FP64 pass costs GB300's FP64 pipe
// (2 operations per clock per SM) for quantities that were only rounded.
__global__ void __launch_bounds__(kBlock) k_geom_faces32(GeomArgs ga, MixedGeomArgs a) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const MeshDev& m = ga.mesh;
  if (e >= m.e || mesh_rejected(m)) return;
  const int2 fc = m.face_cells[e];
  const dbl4 v = m.face_vertices[e];
  // products and sums rounded separately below (this file allows contraction;
  // the FP64 pass does not)
  const double ax = v.x - v.z, ay = v.y - v.w;
  const float area = narrow(root(__dadd_rn(__dmul_rn(ax, ax), __dmul_rn(ay, ay))));
  // second - first = -(first - second) exactly
  const float px = -narrow(ax), py = -narrow(ay);
  a.par[e] = make_float2(px, py);
  a.area[e] = area;
  if (a.xarea != a.area) a.xarea[e] = narrow(a.g64.xarea[e]);
  const double2 x0 = m.points[fc.x], x1 = m.points[fc.y];
  const double ddx = x1.x - x0.x, ddy = x1.y - x0.y;
  const double dab = root(__dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy)));
  ga.dab[e] = dab;  // the face velocities read it in FP64
  const float dx = narrow(ddx), dy = narrow(ddy), dab32 = narrow(dab);
  if (ga.order == 1) {
    a.nrm[e] = make_float2(dx, dy);  // x1 - x0
    a.nabs[e] = dab32;
  } else {
    // pointing from the first neighbour to the second, as w - (w.p) p / p.p
    // of calc_parallel_normal does (w from a point to the face's line)
    const bool up = px * dy - py * dx >= 0.0f;
    a.nrm[e] = up ? make_float2(-py, px) : make_float2(py, -px);
    a.nabs[e] = area;
  }
  const double mx = __dmul_rn(__dadd_rn(v.x, v.z), 0.5), my = __dmul_rn(__dadd_rn(v.y, v.w), 0.5);
  const double2 c0 = m.cms[fc.x], c1 = m.cms[fc.y];
  const float4 dm = make_float4(narrow(mx - c0.x), narrow(my - c0.y), narrow(mx - c1.x), narrow(my - c1.y));
  a.dm0[e] = make_float2(dm.x, dm.y);
  a.dm1[e] = make_float2(dm.z, dm.w);
  // calc_naive_slope's r_ij as the first neighbour sees it (FP32)
  const float s = area / dab32;
  a.frec[2 * e] = make_float4(dx * s, dy * s, __int_as_float(fc.x), __int_as_float(fc.y));
  a.frec[2 * e + 1] = dm;
}

// Two passes over a warp's 32 consecutive cells.  The entry pass writes
// their CSR entries one entry per lane (coalesced stores: the neighbour
// word, the {stencil vector, centroid offset} record and the signed face
// index), the entry's cell found by a binary search over the lanes' offsets.
// The cell pass sums each cell's entries in order (the boundary slope's
// sums, or the naive slope's matrix and its inverse), re-reading the face
// records from cache.
__global__ void __launch_bounds__(kBlock) k_geom_cells32(GeomArgs ga, MixedGeomArgs a) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const MeshDev& m = ga.mesh;
  if (mesh_rejected(m)) return;
  if (t < m.g) {
    const double2 u = a.g64.ghost_unit[t];
    a.ghost_unit[t] = make_float2(narrow(u.x), narrow(u.y));
  }
  const int lane = threadIdx.x & 31;
  const int c0 = t - lane;  // the warp's first cell
  if (c0 < m.n) {
    const unsigned full = 0xffffffffu;
    const int my_off = m.cell_off[c0 + lane < m.n ? c0 + lane : m.n];
    const int last = m.cell_off[c0 + 32 < m.n ? c0 + 32 : m.n];
    const int base = __shfl_sync(full, my_off, 0);
    for (int k0 = base; k0 < last; k0 += 32) {
      const int k = k0 + lane;
      // the entry's cell: the last lane j with cell_off[c0 + j] <= k
      int j = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const int o = __shfl_sync(full, my_off, j + step);
        if (o <= k) j += step;
      }
      if (k < last) {
        const int i = c0 + j;
        const int e = __ldg(m.cell_faces + k);
        const float4 r0 = __ldg(a.frec + 2 * e), r1 = __ldg(a.frec + 2 * e + 1);
        const int f0 = __float_as_int(r0.z), f1 = __float_as_int(r0.w);
        const bool first = f0 == i;
        const int other = first ? f1 : f0;
        const float dmx = first ? r1.x : r1.z, dmy = first ? r1.y : r1.w;
        if (ga.cflags[i] & kCellBoundarySlope) {
          const bool mirror = orig_of(m, f0) == orig_of(m, f1);
          ga.nbr[k] = static_cast<uint32_t>(other) | (mirror ? kNbrMirror : 0u) | (first ? kNbrFirst : 0u);
          const double2 cci = m.cms[i], co = m.cms[other];
          a.ent[k] = make_float4(narrow(co.x - cci.x), narrow(co.y - cci.y), dmx, dmy);
        } else {
          ga.nbr[k] = static_cast<uint32_t>(other) | (first ? kNbrFirst : 0u);
          const float rx = first ? r0.x : -r0.x, ry = first ? r0.y : -r0.y;
          a.ent[k] = make_float4(rx * 0.5f, ry * 0.5f, dmx, dmy);
        }
        a.fsign[k] = e | (first ? static_cast<int>(0x80000000u) : 0);
      }
    }
  }
  if (t >= m.n) return;
  const int i = t;
  const double width = root(quot(m.volume[i], kPi));
  ga.width[i] = width;
  a.width[i] = narrow(width);
  a.inv_cd_volume[i] = __frcp_rn(narrow(m.cd_volume[i]));
  const int b = m.cell_off[i], nn = m.cell_off[i + 1] - b;
  if (ga.cflags[i] & kCellBoundarySlope) {
    // GetBoundarySlope's sums over the CM offsets
    const double2 cci = m.cms[i];
    float sxsy = 0, sy2 = 0, sx2 = 0;
    for (int k = 0; k < nn; ++k) {
      const int e = __ldg(m.cell_faces + b + k);
      const float4 r0 = __ldg(a.frec + 2 * e);
      const int f0 = __float_as_int(r0.z), f1 = __float_as_int(r0.w);
      const double2 co = m.cms[f0 == i ? f1 : f0];
      const float dx = narrow(co.x - cci.x), dy = narrow(co.y - cci.y);
      sxsy += dy * dx;
      sx2 += dx * dx;
      sy2 += dy * dy;
    }
    a.minv[i] = make_float4(sxsy, sx2, sy2, sxsy * sxsy - sx2 * sy2);
    return;
  }
  if (nn > kMaxNaiveNeighbours) {
    record_error(ga.status, 0, RG_ERR_TOO_MANY_NEIGHBORS, 2, i, nn);
    a.minv[i] = make_float4(0, 0, 0, 0);
    return;
  }
  float m0 = 0, m1 = 0, m2 = 0, m3 = 0;
  for (int k = 0; k < nn; ++k) {
    const int e = __ldg(m.cell_faces + b + k);
    const float4 r0 = __ldg(a.frec + 2 * e), r1 = __ldg(a.frec + 2 * e + 1);
    const bool first = __float_as_int(r0.z) == i;
    // -r_ij for the second neighbour; c_ij = centroid - (cm_a + cm_b) / 2
    const float rx = first ? r0.x : -r0.x, ry = first ? r0.y : -r0.y;
    const float cx = 0.5f * (r1.x + r1.z), cy = 0.5f * (r1.y + r1.w);
    m0 -= cx * rx;
    m1 -= cy * rx;
    m2 -= cx * ry;
    m3 -= cy * ry;
  }
  const float vol = narrow(m.volume[i]);
  m0 += vol;
  m3 += vol;
  const float det = m0 * m3 - m1 * m2;
  if (fabsf(det) < 1e-10f * vol * vol) record_error(ga.status, 0, RG_ERR_SINGULAR_MATRIX, 2, i, det);
  const float di = 1.0f / det;
  a.minv[i] = make_float4(m3 * di, -m1 * di, -m2 * di, m0 * di);
}

// ------------------------------------------------------------ conversions

__global__ void __launch_bounds__(kBlock) k_cells_to32(const double* c64, float4* c32, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 a = reinterpret_cast<const double2*>(c64)[2 * i];
  const double2 b = reinterpret_cast<const double2*>(c64)[2 * i + 1];
  c32[i] = make_float4(narrow(a.x), narrow(a.y), narrow(b.x), narrow(b.y));
}

__global__ void __launch_bounds__(kBlock) k_cells_to64(const float4* c32, double* c64, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 v = c32[i];
  reinterpret_cast<double2*>(c64)[2 * i] = make_double2(widen_exact(v.x), widen_exact(v.y));
  reinterpret_cast<double2*>(c64)[2 * i + 1] = make_double2(widen_exact(v.z), widen_exact(v.w));
}

__global__ void __launch_bounds__(kBlock) k_vec2_to32(const double* v64, float2* v32, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 v = reinterpret_cast<const double2*>(v64)[i];
  v32[i] = make_float2(narrow(v.x), narrow(v.y));
}

__global__ void __launch_bounds__(kBlock) k_flux_to64(const float4* f32, double* f64, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 v = f32[i];
  reinterpret_cast<double2*>(f64)[2 * i] = make_double2(widen_exact(v.x), widen_exact(v.y));
  reinterpret_cast<double2*>(f64)[2 * i + 1] = make_double2(widen_exact(v.z), widen_exact(v.w));
}

__global__ void __launch_bounds__(kBlock) k_flux_to32(const double* f64, float4* f32, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 a = reinterpret_cast<const double2*>(f64)[2 * i];
  const double2 b = reinterpret_cast<const double2*>(f64)[2 * i + 1];
  f32[i] = make_float4(narrow(a.x), narrow(a.y), narrow(b.x), narrow(b.y));
}

// ------------------------------------------------------------ per step

template <bool kBatch>
__device__ __forceinline__ float gamma32(const MixedArgs& a, int point) {
  return kBatch ? a.gamma_p[a.cell_problem[point]] : a.gamma;
}
template <bool kBatch>
__device__ __forceinline__ float inv_gm1_32(const MixedArgs& a, int point) {
  return kBatch ? a.inv_gm1_p[a.cell_problem[point]] : a.inv_gm1;
}

// Ghost state: RigidWallGenerator.cpp:5-15 reflection / PeriodicGhostGenerator copy.
__device__ __forceinline__ float4 ghost_state32(const MixedArgs& a, int q) {
  float4 c = a.cells32[a.geom.ghost_real[q]];
  if (a.ghost_kind != RG_GHOST_PERIODIC) {
    const float2 u = a.g32.ghost_unit[q];
    const float s = 2.0f * (c.z * u.x + c.w * u.y);
    c.z -= u.x * s;
    c.w -= u.y * s;
  }
  return c;
}
__device__ __forceinline__ void fill_ghost32(const MixedArgs& a, int q) { a.cells32[a.mesh.n + q] = ghost_state32(a, q); }
// State of point p: a real cell's record, or a ghost's state formed from the
// current state of its cell (the per-step kernels read no ghost records)
__device__ __forceinline__ C4 point32(const MixedArgs& a, int p) {
  const float4 v = p < a.mesh.n ? a.cells32[p] : ghost_state32(a, p - a.mesh.n);
  return C4{v.x, v.y, v.z, v.w};
}

// point p carries LinearGaussImproved's skip_key sticker (a ghost: its cell's)
__device__ __forceinline__ bool skipped32(const MixedArgs& a, int p) {
  return a.skip_mask != 0 && (a.stickers[p < a.mesh.n ? p : a.geom.ghost_real[p - a.mesh.n]] & a.skip_mask) != 0;
}

// SimpleCFL (simple_cfl.cpp:28-47, 58-71) in FP32.  max_e (c+|v-w_e|)/R is
// (c + sqrt(max_e |v-w_e|^2))/R: the bound is monotone in |v-w|.
// cell t's bound 1 / max_e((c + |v - w_e|) / R)
template <bool kBatch>
__device__ __forceinline__ float cfl32_cell(const MixedArgs& a, int t) {
  const MeshDev& m = a.mesh;
  const float4 c = a.cells32[t];
  const float cs = sqrtf(gamma32<kBatch>(a, t) * c.y / c.x);
  float q = 0.0f;
  const int b = m.cell_off[t], e1 = m.cell_off[t + 1];
  if (a.ev_zero) {
    if (e1 > b) q = fmaxf(q, fmaf(c.z, c.z, c.w * c.w));
  } else {
    for (int k = b; k < e1; ++k) {
      const float2 w = a.ev32[m.cell_faces[k]];
      const float dx = c.z - w.x, dy = c.w - w.y;
      q = fmaxf(q, fmaf(dx, dx, dy * dy));
    }
  }
  const float res = (cs + sqrtf(q)) / a.g32.width[t];
  return 1.0f / res;
}

template <bool kBatch>
__global__ void __launch_bounds__(kMaxBlock) k_cfl32(MixedArgs a, int fill_ghosts) {
  const MeshDev& m = a.mesh;
  const int total = fill_ghosts ? m.n + m.g : m.n;
  unsigned int bits = 0x7f800000u;  // this thread's minimum (+inf; non-negative floats order as integers)
  // warp-uniform trip count (see k_cfl)
  for (int base = blockIdx.x * blockDim.x; base < total; base += gridDim.x * blockDim.x) {
    const int t = base + threadIdx.x;
    float x = __int_as_float(0x7f800000);
    if (t < m.n) {
      x = cfl32_cell<kBatch>(a, t);
    } else if (t < total) {
      fill_ghost32(a, t - m.n);
    }
    if (kBatch)
      problem_min(a.dtmin_p, t < m.n ? a.cell_problem[t] : -1,
                  static_cast<unsigned long long>(__double_as_longlong(widen_exact(x))));
    else
      bits = min(bits, __float_as_uint(x));
  }
  if (kBatch) return;
  grid_min_times(a.status, static_cast<unsigned long long>(__double_as_longlong(widen_exact(__uint_as_float(bits)))),
                 a.cfl, &a.status->dt, &a.status->dt32);
}

__global__ void __launch_bounds__(kBlock) k_ghost_fill32(MixedArgs a) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < a.mesh.g) fill_ghost32(a, q);
}

// The limiters' candidate of one neighbour, without branches: the candidate
// quotient is always formed and taken only where the limiter takes it, so
// psi is the same bits as with the limiter's if / else-if, and a warp's
// lanes never diverge here.
__device__ __forceinline__ void limit32(float dphi, float cv, float cellv, float thr, float maxd, float mind,
                                        bool use_abs, float& psi) {
  const bool active = fabsf(dphi) > thr || cv * cellv < 0.0f;
  const float t = use_abs ? fabsf(1e-9f * cellv) : 1e-9f * cellv;
  const float nt = use_abs ? -fabsf(1e-9f * cellv) : -1e-9f * cellv;
  const bool up = dphi > t;
  const float cand = __fdividef(up ? maxd : mind, dphi);
  psi = active && (up || dphi < nt) ? fminf(psi, cand) : psi;
}

__device__ __forceinline__ void shocked32(float dphi, float cv, float cellv, float thr, float nbv, float theta,
                                          float& psi) {
  const bool active = (fabsf(dphi) > thr || cv * cellv < 0.0f) && fabsf(dphi) > 1e-9f * cellv;
  const float cand = fmaxf(__fdividef(theta * (nbv - cellv), dphi), 0.0f);
  psi = active ? fminf(psi, cand) : psi;
}

// The FP32 slopes of a periodic mesh (no self-mirror neighbour, no boundary
// slope), written widened and as the FP32 slopes the face kernel reads, with
// the limiter trace the adjoint's reverse slope kernel reads
// (SlopeTrace: the unlimited slope, each component's factor, the centroid
// difference and neighbour of its active candidate).  The arithmetic is
// k_slopes32_item's; the arg max / min follow the first strict improvement
// as std::max / std::min do, and each psi is the smallest candidate taken in
// edge order, which is what fminf over the candidates gives.
__global__ void __launch_bounds__(kBlock) k_slopes32_trace(MixedArgs a, double* slopes64, SlopeTrace* trace) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const MeshDev& m = a.mesh;
  if (i >= m.n) return;
  const C4 cell = ld4(a.cells32, i);
  const int b = m.cell_off[i], nn = m.cell_off[i + 1] - b;
  const float4 mi = a.g32.minv[i];
  C4 vx{0, 0, 0, 0}, vy{0, 0, 0, 0};
  float cmax[4] = {cell.d, cell.p, cell.vx, cell.vy}, cmin[4] = {cell.d, cell.p, cell.vx, cell.vy};
  int amax[4] = {-1, -1, -1, -1}, amin[4] = {-1, -1, -1, -1};
  bool ratio_shock = false;
  for (int k = 0; k < nn; ++k) {
    const C4 nb = point32(a, static_cast<int>(a.geom.nbr[b + k] & kNbrIdMask));
    const float4 en = a.g32.ent[b + k];
    const C4 s2{cell.d + nb.d, cell.p + nb.p, cell.vx + nb.vx, cell.vy + nb.vy};
    addm(vx, s2, en.x);
    addm(vy, s2, en.y);
    const float nv[4] = {nb.d, nb.p, nb.vx, nb.vy};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (cmax[q] < nv[q]) {
        cmax[q] = nv[q];
        amax[q] = k;
      }
      if (nv[q] < cmin[q]) {
        cmin[q] = nv[q];
        amin[q] = k;
      }
    }
    ratio_shock = ratio_shock || fminf(cell.p, nb.p) < a.delta_p * fmaxf(cell.p, nb.p);
  }
  C4 nx, ny;
  naive_slope(false, vx, vy, mi, nx, ny);
  float sx[4] = {nx.d, nx.p, nx.vx, nx.vy};
  float sy[4] = {ny.d, ny.p, ny.vx, ny.vy};
  SlopeTrace& tr = trace[i];
  const float cq[4] = {cell.d, cell.p, cell.vx, cell.vy};
  float psi[4] = {1, 1, 1, 1};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    tr.naive[q] = sx[q];
    tr.naive[4 + q] = sy[q];
    tr.dphi[q] = 0;
    tr.code[q] = kTraceNone;
  }
  if (a.slf) {
    const float cs = sqrtf(a.gamma * cell.p / cell.d);
    const bool shock = (sx[2] + sy[3]) * a.g32.width[i] < (-a.delta_v) * cs || ratio_shock;
    const float f = shock ? 0.1f : 0.05f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float maxd = cmax[q] - cq[q], mind = cmin[q] - cq[q];
      const float thr = f * fmaxf(fabsf(maxd), fabsf(mind));
      for (int k = 0; k < nn; ++k) {
        const float4 en = a.g32.ent[b + k];
        float cv = fmaf(sx[q], en.z, cq[q]);
        cv = fmaf(sy[q], en.w, cv);
        const float dphi = cv - cq[q];
        if (!(fabsf(dphi) > thr || cv * cq[q] < 0.0f)) continue;
        if (!shock) {
          const bool use_abs = q >= 2;
          const float t = use_abs ? fabsf(1e-9f * cq[q]) : 1e-9f * cq[q];
          const float nt = use_abs ? -fabsf(1e-9f * cq[q]) : -1e-9f * cq[q];
          const bool up = dphi > t;
          if (up || dphi < nt) {
            const float cand = __fdividef(up ? maxd : mind, dphi);
            if (cand < psi[q]) {
              psi[q] = cand;
              tr.code[q] = k | ((up ? 0 : 1) << 8) | (((up ? amax[q] : amin[q]) + 1) << 16);
              tr.dphi[q] = dphi;
            }
          }
        } else if (fabsf(dphi) > 1e-9f * cq[q]) {
          const C4 nb = point32(a, static_cast<int>(a.geom.nbr[b + k] & kNbrIdMask));
          const float nv[4] = {nb.d, nb.p, nb.vx, nb.vy};
          const float cand = __fdividef(a.theta * (nv[q] - cq[q]), dphi);
          const bool clamp = cand < 0.0f;
          const float x = clamp ? 0.0f : cand;
          if (x < psi[q]) {
            psi[q] = x;
            tr.code[q] = k | ((clamp ? 3 : 2) << 8) | ((k + 1) << 16);
            tr.dphi[q] = dphi;
          }
        }
      }
    }
  }
  double2* o = reinterpret_cast<double2*>(slopes64) + 4 * i;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    tr.psi[q] = psi[q];
    sx[q] *= psi[q];
    sy[q] *= psi[q];
  }
  o[0] = make_double2(sx[0], sx[1]);
  o[1] = make_double2(sx[2], sx[3]);
  o[2] = make_double2(sy[0], sy[1]);
  o[3] = make_double2(sy[2], sy[3]);
  // the same slopes for the face kernel of the recomputed step
  a.slopes32[2 * i] = make_float4(sx[0], sx[1], sx[2], sx[3]);
  a.slopes32[2 * i + 1] = make_float4(sy[0], sy[1], sy[2], sy[3]);
}

// LinearGaussImproved::calc_slope (LinearGaussImproved.cpp:425-494) in FP32.
template <bool kBatch, int kUnroll>
__device__ __forceinline__ void k_slopes32_item(const MixedArgs& a, int i) {
  const MeshDev& m = a.mesh;
  const C4 cell = ld4(a.cells32, i);
  const int b = m.cell_off[i], nn = m.cell_off[i + 1] - b;
  const float4 mi = a.g32.minv[i];
  const bool boundary = a.geom.cflags[i] & kCellBoundarySlope;
  // one pass over the neighbours: the gradient's sums, the neighbour
  // max / min over all neighbours and over those that are not self-mirror
  // ghosts (the unshocked limiter skips those, LinearGaussImproved.cpp:194-195)
  // and the pressure-ratio shock test
  C4 vx{0, 0, 0, 0}, vy{0, 0, 0, 0};
  C4 amax = cell, amin = cell, nmax = cell, nmin = cell;
  bool ratio_shock = false;
#pragma unroll(kUnroll)
  for (int k = 0; k < nn; ++k) {
    const uint32_t w = a.geom.nbr[b + k];
    const C4 nb = point32(a, static_cast<int>(w & kNbrIdMask));
    const float4 en = a.g32.ent[b + k];
    // boundary cells: least squares on differences (:401-422); others: the
    // Green-Gauss sum of 0.5 r_ij (cell + neighbour) (:80-133)
    const C4 s = boundary ? C4{nb.d - cell.d, nb.p - cell.p, nb.vx - cell.vx, nb.vy - cell.vy}
                          : C4{cell.d + nb.d, cell.p + nb.p, cell.vx + nb.vx, cell.vy + nb.vy};
    addm(vx, s, en.x);
    addm(vy, s, en.y);
    // neighbours with LinearGaussImproved's skip_key sticker stay out of
    // both extrema (:192-193, :314-315)
    if (!skipped32(a, static_cast<int>(w & kNbrIdMask))) {
      amax = C4{fmaxf(amax.d, nb.d), fmaxf(amax.p, nb.p), fmaxf(amax.vx, nb.vx), fmaxf(amax.vy, nb.vy)};
      amin = C4{fminf(amin.d, nb.d), fminf(amin.p, nb.p), fminf(amin.vx, nb.vx), fminf(amin.vy, nb.vy)};
      if (boundary && !(w & kNbrMirror)) {
        nmax = C4{fmaxf(nmax.d, nb.d), fmaxf(nmax.p, nb.p), fmaxf(nmax.vx, nb.vx), fmaxf(nmax.vy, nb.vy)};
        nmin = C4{fminf(nmin.d, nb.d), fminf(nmin.p, nb.p), fminf(nmin.vx, nb.vx), fminf(nmin.vy, nb.vy)};
      }
    }
    // min(p, p_k) / max(p, p_k) < delta_p without the division
    ratio_shock = ratio_shock || fminf(cell.p, nb.p) < a.delta_p * fmaxf(cell.p, nb.p);
  }
  if (!boundary) {
    // a cell with a self-mirror neighbour takes the boundary slope: every
    // other cell's neighbours count in both extrema
    nmax = amax;
    nmin = amin;
  }
  // boundary cells: vx, vy hold sum(df*dx), sum(df*dy)
  C4 sx, sy;
  naive_slope(boundary, vx, vy, mi, sx, sy);
  if (a.slf) {
    const float cs = sqrtf(gamma32<kBatch>(a, i) * cell.p / cell.d);
    const bool shock = (sx.vx + sy.vy) * a.g32.width[i] < (-a.delta_v) * cs || ratio_shock;
    if (a.shock) a.shock[i] = shock ? 1 : 0;  // read by the tracer slopes
    const C4 cmax = shock ? amax : nmax, cmin = shock ? amin : nmin;
    const C4 maxd{cmax.d - cell.d, cmax.p - cell.p, cmax.vx - cell.vx, cmax.vy - cell.vy};
    const C4 mind{cmin.d - cell.d, cmin.p - cell.p, cmin.vx - cell.vx, cmin.vy - cell.vy};
    const float f = shock ? 0.1f : 0.05f;
    const C4 thr{f * fmaxf(fabsf(maxd.d), fabsf(mind.d)), f * fmaxf(fabsf(maxd.p), fabsf(mind.p)),
                 f * fmaxf(fabsf(maxd.vx), fabsf(mind.vx)), f * fmaxf(fabsf(maxd.vy), fabsf(mind.vy))};
    float psi0 = 1, psi1 = 1, psi2 = 1, psi3 = 1;
#pragma unroll(kUnroll)
    for (int k = 0; k < nn; ++k) {
      const float4 en = a.g32.ent[b + k];
      C4 cv = cell;
      addm(cv, sx, en.z);
      addm(cv, sy, en.w);
      const C4 dphi{cv.d - cell.d, cv.p - cell.p, cv.vx - cell.vx, cv.vy - cell.vy};
      if (!shock) {
        limit32(dphi.d, cv.d, cell.d, thr.d, maxd.d, mind.d, false, psi0);
        limit32(dphi.p, cv.p, cell.p, thr.p, maxd.p, mind.p, false, psi1);
        limit32(dphi.vx, cv.vx, cell.vx, thr.vx, maxd.vx, mind.vx, true, psi2);
        limit32(dphi.vy, cv.vy, cell.vy, thr.vy, maxd.vy, mind.vy, true, psi3);
      } else {
        const int p = static_cast<int>(a.geom.nbr[b + k] & kNbrIdMask);
        if (skipped32(a, p)) continue;  // :339-340
        const C4 nb = point32(a, p);
        shocked32(dphi.d, cv.d, cell.d, thr.d, nb.d, a.theta, psi0);
        shocked32(dphi.p, cv.p, cell.p, thr.p, nb.p, a.theta, psi1);
        shocked32(dphi.vx, cv.vx, cell.vx, thr.vx, nb.vx, a.theta, psi2);
        shocked32(dphi.vy, cv.vy, cell.vy, thr.vy, nb.vy, a.theta, psi3);
      }
    }
    sx.d *= psi0; sy.d *= psi0;
    sx.p *= psi1; sy.p *= psi1;
    sx.vx *= psi2; sy.vx *= psi2;
    sx.vy *= psi3; sy.vy *= psi3;
  }
  a.slopes32[2 * i] = make_float4(sx.d, sx.p, sx.vx, sx.vy);
  a.slopes32[2 * i + 1] = make_float4(sy.d, sy.p, sy.vx, sy.vy);
}

// The same slope with the neighbour states and stencil records of cells
// with at most kPrefetch neighbours loaded up front, all independent, so
// their latencies overlap; the arithmetic runs over them in the order of
// k_slopes32_item and gives the same bits.  Cells with more neighbours take
// k_slopes32_item.
constexpr int kPrefetch = 8;
template <bool kBatch>
__device__ __forceinline__ void k_slopes32_pf_item(const MixedArgs& a, int i) {
  const MeshDev& m = a.mesh;
  const int b = m.cell_off[i], nn = m.cell_off[i + 1] - b;
  if (nn > kPrefetch) {
    k_slopes32_item<kBatch, 1>(a, i);
    return;
  }
  const C4 cell = ld4(a.cells32, i);
  const float4 mi = a.g32.minv[i];
  const bool boundary = a.geom.cflags[i] & kCellBoundarySlope;
  C4 nbk[kPrefetch];
  float4 enk[kPrefetch];
  uint32_t wk[kPrefetch];
#pragma unroll
  for (int k = 0; k < kPrefetch; ++k) {
    if (k < nn) {
      wk[k] = a.geom.nbr[b + k];
      enk[k] = a.g32.ent[b + k];
    }
  }
#pragma unroll
  for (int k = 0; k < kPrefetch; ++k)
    if (k < nn) nbk[k] = point32(a, static_cast<int>(wk[k] & kNbrIdMask));
  C4 vx{0, 0, 0, 0}, vy{0, 0, 0, 0};
  C4 amax = cell, amin = cell, nmax = cell, nmin = cell;
  bool ratio_shock = false;
#pragma unroll
  for (int k = 0; k < kPrefetch; ++k) {
    if (k >= nn) break;
    const C4& nb = nbk[k];
    const float4 en = enk[k];
    const C4 s = boundary ? C4{nb.d - cell.d, nb.p - cell.p, nb.vx - cell.vx, nb.vy - cell.vy}
                          : C4{cell.d + nb.d, cell.p + nb.p, cell.vx + nb.vx, cell.vy + nb.vy};
    addm(vx, s, en.x);
    addm(vy, s, en.y);
    if (!skipped32(a, static_cast<int>(wk[k] & kNbrIdMask))) {
      amax = C4{fmaxf(amax.d, nb.d), fmaxf(amax.p, nb.p), fmaxf(amax.vx, nb.vx), fmaxf(amax.vy, nb.vy)};
      amin = C4{fminf(amin.d, nb.d), fminf(amin.p, nb.p), fminf(amin.vx, nb.vx), fminf(amin.vy, nb.vy)};
      if (boundary && !(wk[k] & kNbrMirror)) {
        nmax = C4{fmaxf(nmax.d, nb.d), fmaxf(nmax.p, nb.p), fmaxf(nmax.vx, nb.vx), fmaxf(nmax.vy, nb.vy)};
        nmin = C4{fminf(nmin.d, nb.d), fminf(nmin.p, nb.p), fminf(nmin.vx, nb.vx), fminf(nmin.vy, nb.vy)};
      }
    }
    ratio_shock = ratio_shock || fminf(cell.p, nb.p) < a.delta_p * fmaxf(cell.p, nb.p);
  }
  if (!boundary) {
    // a cell with a self-mirror neighbour takes the boundary slope: every
    // other cell's neighbours count in both extrema
    nmax = amax;
    nmin = amin;
  }
  C4 sx, sy;
  naive_slope(boundary, vx, vy, mi, sx, sy);
  if (a.slf) {
    const float cs = sqrtf(gamma32<kBatch>(a, i) * cell.p / cell.d);
    const bool shock = (sx.vx + sy.vy) * a.g32.width[i] < (-a.delta_v) * cs || ratio_shock;
    if (a.shock) a.shock[i] = shock ? 1 : 0;  // read by the tracer slopes
    const C4 cmax = shock ? amax : nmax, cmin = shock ? amin : nmin;
    const C4 maxd{cmax.d - cell.d, cmax.p - cell.p, cmax.vx - cell.vx, cmax.vy - cell.vy};
    const C4 mind{cmin.d - cell.d, cmin.p - cell.p, cmin.vx - cell.vx, cmin.vy - cell.vy};
    const float f = shock ? 0.1f : 0.05f;
    const C4 thr{f * fmaxf(fabsf(maxd.d), fabsf(mind.d)), f * fmaxf(fabsf(maxd.p), fabsf(mind.p)),
                 f * fmaxf(fabsf(maxd.vx), fabsf(mind.vx)), f * fmaxf(fabsf(maxd.vy), fabsf(mind.vy))};
    float psi0 = 1, psi1 = 1, psi2 = 1, psi3 = 1;
#pragma unroll
    for (int k = 0; k < kPrefetch; ++k) {
      if (k >= nn) break;
      const float4 en = enk[k];
      C4 cv = cell;
      addm(cv, sx, en.z);
      addm(cv, sy, en.w);
      const C4 dphi{cv.d - cell.d, cv.p - cell.p, cv.vx - cell.vx, cv.vy - cell.vy};
      if (!shock) {
        limit32(dphi.d, cv.d, cell.d, thr.d, maxd.d, mind.d, false, psi0);
        limit32(dphi.p, cv.p, cell.p, thr.p, maxd.p, mind.p, false, psi1);
        limit32(dphi.vx, cv.vx, cell.vx, thr.vx, maxd.vx, mind.vx, true, psi2);
        limit32(dphi.vy, cv.vy, cell.vy, thr.vy, maxd.vy, mind.vy, true, psi3);
      } else {
        if (skipped32(a, static_cast<int>(wk[k] & kNbrIdMask))) continue;
        const C4& nb = nbk[k];
        shocked32(dphi.d, cv.d, cell.d, thr.d, nb.d, a.theta, psi0);
        shocked32(dphi.p, cv.p, cell.p, thr.p, nb.p, a.theta, psi1);
        shocked32(dphi.vx, cv.vx, cell.vx, thr.vx, nb.vx, a.theta, psi2);
        shocked32(dphi.vy, cv.vy, cell.vy, thr.vy, nb.vy, a.theta, psi3);
      }
    }
    sx.d *= psi0; sy.d *= psi0;
    sx.p *= psi1; sy.p *= psi1;
    sx.vx *= psi2; sy.vx *= psi2;
    sx.vy *= psi3; sy.vy *= psi3;
  }
  a.slopes32[2 * i] = make_float4(sx.d, sx.p, sx.vx, sx.vy);
  a.slopes32[2 * i + 1] = make_float4(sy.d, sy.p, sy.vx, sy.vy);
}

template <bool kBatch>
__global__ void __launch_bounds__(kMaxBlock) k_slopes32_pf(MixedArgs a) {
  if (a.take_next_dt && blockIdx.x == 0 && threadIdx.x == 0) {
    a.status->dt = a.status->dt_next;
    a.status->dt32 = a.status->dt_next32;
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.mesh.n; i += gridDim.x * blockDim.x)
    k_slopes32_pf_item<kBatch>(a, i);
}

template <bool kBatch, int kMinBlocks, int kUnroll>
__global__ void __launch_bounds__(kMinBlocks ? kCappedBlock : kMaxBlock, kMinBlocks ? kMinBlocks : 1)
    k_slopes32(MixedArgs a) {
  // the dt of this step, computed by the previous step's update
  if (a.take_next_dt && blockIdx.x == 0 && threadIdx.x == 0) {
    a.status->dt = a.status->dt_next;
    a.status->dt32 = a.status->dt_next32;
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.mesh.n; i += gridDim.x * blockDim.x)
    k_slopes32_item<kBatch, kUnroll>(a, i);
}

__device__ __forceinline__ P6 prim32(float g, float inv_gm1, const C4& c) {
  const float pd = __fdividef(c.p, c.d);
  return P6{c.d, c.p, c.vx, c.vy, pd * inv_gm1, sqrtf(g * pd)};
}

// Hllc (hllc.cpp:97-154, massflux) in FP32 in the face frame.
__device__ __forceinline__ bool hllc32(P6 l, P6 r, float vel, F4& f, const MixedArgs& a, int face) {
  if (isnan(r.vx)) {
    record_error(a.status, a.step, RG_ERR_HLLC_NAN, 3, face, r.vx);
    return false;
  }
  l.vx -= vel;
  r.vx -= vel;
  const float sl = fminf(l.vx - l.c, r.vx - r.c);
  const float sr = fmaxf(l.vx + l.c, r.vx + r.c);
  const float ss = __fdividef(r.p - l.p + l.d * l.vx * (sl - l.vx) - r.d * r.vx * (sr - r.vx),
                              l.d * (sl - l.vx) - r.d * (sr - r.vx));
  const bool use_left = sl > 0.0f || (sl <= 0.0f && ss >= 0.0f);
  const bool use_right = !use_left && ((ss < 0.0f && sr >= 0.0f) || sr < 0.0f);
  if (!use_left && !use_right) {
    record_error(a.status, a.step, RG_ERR_HLLC_WAVE_SPEEDS, 3, face, ss);
    return false;
  }
  const P6& q = use_left ? l : r;
  const float sk = use_left ? sl : sr;
  const float ek = q.d * (0.5f * (q.vx * q.vx + q.vy * q.vy) + q.e);
  const float dsp = q.d * q.vx;
  F4 fk{dsp, q.p + q.vx * dsp, q.vy * dsp, (ek + q.p) * q.vx};
  if (use_left ? !(sl > 0.0f) : !(sr < 0.0f)) {
    const float skv = sk - q.vx;
    const float ds = __fdividef(q.d * skv, sk - ss);
    const float id = __fdividef(1.0f, q.d);
    const float use = ds * (ek * id + (ss - q.vx) * (ss + __fdividef(q.p * id, skv)));
    fk.m += sk * (ds - q.d);
    fk.mx += (ds * ss - dsp) * sk;
    fk.my += (ds * q.vy - q.vy * q.d) * sk;
    fk.en += sk * (use - ek);
  }
  fk.en += fk.mx * vel + 0.5f * fk.m * vel * vel;
  fk.mx += vel * fk.m;
  f = fk;
  return true;
}

__device__ __forceinline__ bool solve32(P6 l, P6 r, float vel, float2 n, float na, float2 p, float pa, F4& out,
                                        const MixedArgs& a, int face) {
  const float in = __fdividef(1.0f, na), ip = __fdividef(1.0f, pa);
  const float lx = (l.vx * n.x + l.vy * n.y) * in, ly = (l.vx * p.x + l.vy * p.y) * ip;
  const float rx = (r.vx * n.x + r.vy * n.y) * in, ry = (r.vx * p.x + r.vy * p.y) * ip;
  l.vx = lx;
  l.vy = ly;
  r.vx = rx;
  r.vy = ry;
  F4 c;
  if (!hllc32(l, r, vel, c, a, face)) return false;
  out.m = c.m;
  out.mx = (n.x * c.mx) * in + (p.x * c.my) * ip;
  out.my = (n.y * c.mx) * in + (p.y * c.my) * ip;
  out.en = c.en;
  return true;
}

template <bool kBatch>
__device__ __forceinline__ void write32(const MixedArgs& a, int e, int real_side, const F4& c, bool scaled,
                                        float area) {
  float s = 1.0f;
  if (scaled) {
    if (kBatch)
      s = narrow(a.cfl * __longlong_as_double(static_cast<long long>(
                                          a.dtmin_p[a.cell_problem[real_side]]))) * area;
    else
      s = (a.dt32_from_device ? a.status->dt32 : a.dt32) * area;
  }
  a.flux32[e] = make_float4(c.m * s, c.en * s, c.mx * s, c.my * s);
  // the unscaled mass flux the tracer faces kernel upwinds with
  if (a.mflux) a.mflux[e] = static_cast<double>(c.m);
}

// LinearGaussImproved's face value of point pid at offset dm from its CM
__device__ __forceinline__ C4 side32(const MixedArgs& a, int pid, float2 dm) {
  const MeshDev& m = a.mesh;
  C4 c = point32(a, pid);
  int sid = pid;
  bool zero = false;
  if (pid >= m.n) {
    if (a.ghost_kind == RG_GHOST_PERIODIC)
      sid = m.ghost_source[pid - m.n];
    else
      zero = true;
  }
  if (!zero) {
    const C4 gx = ld4(a.slopes32, 2 * sid), gy = ld4(a.slopes32, 2 * sid + 1);
    addm(c, gx, dm.x);
    addm(c, gy, dm.y);
  }
  return c;
}

// Hllc on face e's two face values, scaled and written
template <bool kScaled, bool kBatch>
__device__ __forceinline__ void face32_solve(const MixedArgs& a, int e, int2 fc, const C4& s0, const C4& s1) {
  const MeshDev& m = a.mesh;
  const float2 w = a.ev_zero ? make_float2(0.0f, 0.0f) : a.ev32[e];
  const float2 n = a.g32.nrm[e], p = a.g32.par[e];
  const float na = a.g32.nabs[e], pa = a.g32.area[e];
  const float vel = (n.x * w.x + n.y * w.y) / na;
  const int real_side = fc.x < m.n ? fc.x : fc.y;
  const float g = gamma32<kBatch>(a, real_side), igm = inv_gm1_32<kBatch>(a, real_side);
  F4 c;
  if (!solve32(prim32(g, igm, s0), prim32(g, igm, s1), vel, n, na, p, pa, c, a, e)) return;
  write32<kBatch>(a, e, real_side, c, kScaled, a.g32.xarea[e]);
}

template <bool kScaled, bool kBatch>
__device__ __forceinline__ void k_faces32_lgi_item(const MixedArgs& a, int e) {
  const int2 fc = a.mesh.face_cells[e];
  const C4 s0 = side32(a, fc.x, a.g32.dm0[e]);
  const C4 s1 = side32(a, fc.y, a.g32.dm1[e]);
  face32_solve<kScaled, kBatch>(a, e, fc, s0, s1);
}

template <bool kScaled, bool kBatch>
__global__ void __launch_bounds__(kMaxBlock) k_faces32_lgi(MixedArgs a) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < a.mesh.e; e += gridDim.x * blockDim.x)
    k_faces32_lgi_item<kScaled, kBatch>(a, e);
}

// Two threads per face (launch-shape build 1): lane s of a pair forms face
// value s (half the gathers in each thread's dependent chain, twice the
// threads in flight); the pair swaps the two values with shuffles and the
// even lane solves and writes.  Each value comes from the same code as in
// k_faces32_lgi_item, so the fluxes are bit-identical to the one-thread build.
template <bool kScaled, bool kBatch>
__global__ void __launch_bounds__(kMaxBlock) k_faces32_lgi_pair(MixedArgs a) {
  const int s = threadIdx.x & 1;
  const unsigned pair = 3u << (threadIdx.x & 30);
  const int stride = (gridDim.x * blockDim.x) >> 1;
  for (int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 1; e < a.mesh.e; e += stride) {
    const int2 fc = a.mesh.face_cells[e];
    const C4 mine = side32(a, s ? fc.y : fc.x, s ? a.g32.dm1[e] : a.g32.dm0[e]);
    C4 other;
    other.d = __shfl_xor_sync(pair, mine.d, 1);
    other.p = __shfl_xor_sync(pair, mine.p, 1);
    other.vx = __shfl_xor_sync(pair, mine.vx, 1);
    other.vy = __shfl_xor_sync(pair, mine.vy, 1);
    if (s == 0) face32_solve<kScaled, kBatch>(a, e, fc, mine, other);
  }
}

template <bool kScaled, bool kBatch>
__device__ __forceinline__ void k_faces32_pcm_item(const MixedArgs& a, int e) {
  const MeshDev& m = a.mesh;
  const int2 fc = m.face_cells[e];
  const float2 p = a.g32.par[e], n = a.g32.nrm[e];
  const float pa = a.g32.area[e], na = a.g32.nabs[e];
  const bool va = fc.x < m.n, vb = fc.y < m.n;
  const int oa = va ? fc.x : m.ghost_source[fc.x - m.n];
  const int ob = vb ? fc.y : m.ghost_source[fc.y - m.n];
  auto reflect = [&](P6 q) {
    const float s = 2.0f * (q.vx * p.x + q.vy * p.y) / (pa * pa);
    q.vx = p.x * s - q.vx;
    q.vy = p.y * s - q.vy;
    return q;
  };
  const int real_side = va ? fc.x : fc.y;
  const float g = gamma32<kBatch>(a, real_side), igm = inv_gm1_32<kBatch>(a, real_side);
  P6 l, r;
  if (!va) {
    r = prim32(g, igm, ld4(a.cells32, fc.y));
    l = oa == ob ? reflect(r) : prim32(g, igm, ld4(a.cells32, oa));
  } else if (!vb) {
    l = prim32(g, igm, ld4(a.cells32, fc.x));
    r = oa == ob ? reflect(l) : prim32(g, igm, ld4(a.cells32, ob));
  } else {
    l = prim32(g, igm, ld4(a.cells32, fc.x));
    r = prim32(g, igm, ld4(a.cells32, fc.y));
  }
  const float2 w = a.ev_zero ? make_float2(0.0f, 0.0f) : a.ev32[e];
  const float vel = (n.x * w.x + n.y * w.y) / na;
  F4 c;
  if (!solve32(l, r, vel, n, na, p, pa, c, a, e)) return;
  if (oa == ob && vel == 0.0f) {
    // A static reflecting wall: the two states are mirror images, so the exact
    // HLLC contact speed is zero and so are the mass and energy fluxes.  FP32
    // rounding in the star-state algebra would leave ~1e-7 of the flux there
    // and leak mass through the wall; the FP64 path leaves ~1e-16.
    c.m = 0.0f;
    c.en = 0.0f;
  }
  write32<kBatch>(a, e, real_side, c, kScaled, a.g32.xarea[e]);
}

template <bool kScaled, bool kBatch>
__global__ void __launch_bounds__(kMaxBlock) k_faces32_pcm(MixedArgs a) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < a.mesh.e; e += gridDim.x * blockDim.x)
    k_faces32_pcm_item<kScaled, kBatch>(a, e);
}

// float -> double on the integer pipe.  GB300 issues FP64-pipe instructions,
// conversions included, at 2 per clock per SM against 64 for integer ones,
// and the update kernel is bound by that pipe.  Exact for zeros, normal
// floats, infinities and NaNs; a subnormal float (below 1.2e-38 in
// magnitude) becomes a zero of its sign.
__device__ __forceinline__ double widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned ex = (u >> 23) & 0xffu;
  const unsigned dex = ex == 0u ? 0u : (ex == 0xffu ? 0x7ffu : ex + 896u);  // rebias 127 -> 1023
  const unsigned mant = ex == 0u ? 0u : (u & 0x7fffffu);
  const unsigned hi = (u & 0x80000000u) | (dex << 20) | (mant >> 3);
  return __hiloint2double(static_cast<int>(hi), static_cast<int>(mant << 29));
}

// Error-free FP32 addition (Knuth's TwoSum): s + x == s' + err exactly.
__device__ __forceinline__ void two_sum(float& s, float& c, float x) {
  const float t = s + x;
  const float bb = t - s;
  const float err = (s - (t - bb)) + (x - bb);
  s = t;
  c += err;
}

// Gather and cell update (simple_extensive_updater.cpp:11-35,
// simple_cell_updater.cpp:22-59).  The FP32 face contributions of a cell are
// summed in float-float (TwoSum; ~48-bit, on the FP32 pipe, in ascending face
// order) and added to the FP64 extensives once per component, so a face's
// contribution enters its two cells with opposite signs and the extensives
// keep FP64 precision across steps.  e = E/m - v^2/2 is formed in FP64 with a
// Newton-refined reciprocal of m.
template <bool kBatch>
__device__ __forceinline__ unsigned long long k_update_mixed_item(const MixedArgs& a, int i, int from_unscaled,
                                                               int do_ext, int do_cells) {
  const MeshDev& m = a.mesh;
  double2* ext2 = reinterpret_cast<double2*>(a.ext);
  const double2 e01 = ext2[2 * i], e23 = ext2[2 * i + 1];
  double mass = e01.x, en = e01.y, px = e23.x, py = e23.y;
  if (do_ext) {
    float s0 = 0, s1 = 0, s2 = 0, s3 = 0, c0 = 0, c1 = 0, c2 = 0, c3 = 0;
    const int b = m.cell_off[i], e1 = m.cell_off[i + 1];
    for (int k = b; k < e1; ++k) {
      const int fs = a.g32.fsign[k];
      const int e = fs & 0x7fffffff;
      float4 f = a.flux32[e];
      if (from_unscaled) {
        const float sc = a.dt32 * a.g32.xarea[e];
        f = make_float4(f.x * sc, f.y * sc, f.z * sc, f.w * sc);
      }
      if (fs < 0) f = make_float4(-f.x, -f.y, -f.z, -f.w);
      two_sum(s0, c0, f.x);
      two_sum(s1, c1, f.y);
      two_sum(s2, c2, f.z);
      two_sum(s3, c3, f.w);
    }
    mass += widen(s0) + widen(c0);
    en += widen(s1) + widen(c1);
    px += widen(s2) + widen(c2);
    py += widen(s3) + widen(c3);
    if (a.ext_avg) {
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
      const float4 c = a.cells32[i];
      if (a.cells32_out) a.cells32_out[i] = c;
      if (!a.cfl_next) return kInfBits;
      const float cs = sqrtf(gamma32<kBatch>(a, i) * c.y / c.x);
      float q = 0.0f;
      if (a.ev_zero) {
        if (m.cell_off[i + 1] > m.cell_off[i]) q = fmaxf(q, fmaf(c.z, c.z, c.w * c.w));
      } else {
        for (int k = m.cell_off[i]; k < m.cell_off[i + 1]; ++k) {
          const float2 w = a.ev32[a.g32.fsign[k] & 0x7fffffff];
          const float dx = c.z - w.x, dy = c.w - w.y;
          q = fmaxf(q, fmaf(dx, dx, dy * dy));
        }
      }
      const float res = (cs + sqrtf(q)) / a.g32.width[i];
      return static_cast<unsigned long long>(__double_as_longlong(widen_exact(1.0f / res)));
    }
    const float mf = narrow(mass);
    const float d = mf * a.g32.inv_cd_volume[i];
    if (d < 0.0f) {
      record_error(a.status, a.step, RG_ERR_NEGATIVE_DENSITY, 5, i, d);
      return kInfBits;
    }
    // 1/m: the FP32 reciprocal (relative error < 2^-23) and one Newton step
    // (relative error < 2^-45, far below the FP32 rounding of the results)
    double r = widen(1.0f / mf);
    r = r * (2.0 - mass * r);
    // e = E/m - v^2/2 in FP64 (the cancellation at high Mach numbers)
    const double vx = px * r, vy = py * r;
    const double energy = en * r - 0.5 * (vx * vx + vy * vy);
    if (energy < 0) {
      record_error(a.status, a.step, RG_ERR_NEGATIVE_ENERGY, 5, i, energy);
      return kInfBits;
    }
    const float4 c = make_float4(d, (gamma32<kBatch>(a, i) - 1.0f) * narrow(energy) * d, narrow(vx), narrow(vy));
    (a.cells32_out ? a.cells32_out : a.cells32)[i] = c;
    if (a.cfl_next) {
      // the next step's SimpleCFL bound of this cell, as k_cfl32 computes it
      // from the record just stored
      const float cs = sqrtf(gamma32<kBatch>(a, i) * c.y / c.x);
      float q = 0.0f;
      if (a.ev_zero) {
        if (m.cell_off[i + 1] > m.cell_off[i]) q = fmaxf(q, fmaf(c.z, c.z, c.w * c.w));
      } else {
        for (int k = m.cell_off[i]; k < m.cell_off[i + 1]; ++k) {
          const float2 w = a.ev32[a.g32.fsign[k] & 0x7fffffff];
          const float dx = c.z - w.x, dy = c.w - w.y;
          q = fmaxf(q, fmaf(dx, dx, dy * dy));
        }
      }
      const float res = (cs + sqrtf(q)) / a.g32.width[i];
      return static_cast<unsigned long long>(__double_as_longlong(widen_exact(1.0f / res)));
    }
  }
  return kInfBits;
}

// kMinBlocks > 0: register-capped builds for blocks of up to kCappedBlock
// threads with kMinBlocks resident per SM (launch-shape variants 2 and 3)
template <bool kBatch, int kMinBlocks = 0>
__global__ void __launch_bounds__(kMinBlocks ? kCappedBlock : kMaxBlock, kMinBlocks ? kMinBlocks : 1)
    k_update_mixed(MixedArgs a, int from_unscaled, int do_ext, int do_cells) {
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  if (kBatch && do_ext && !from_unscaled && !a.batch_keep_dt) {
    for (int p = t0; p < a.n_problems; p += stride) {
      const double dt = a.cfl * __longlong_as_double(static_cast<long long>(a.dtmin_p[p]));
      a.dt_p[p] = dt;
      a.time_p[p] += dt;
      a.dtmin_p[p] = kInfBits;
    }
  }
  unsigned long long bits = kInfBits;
  for (int i = t0; i < a.mesh.n; i += stride) {
    const unsigned long long b = k_update_mixed_item<kBatch>(a, i, from_unscaled, do_ext, do_cells);
    bits = b < bits ? b : bits;
  }
  if (!kBatch && a.cfl_next) grid_min_times(a.status, bits, a.cfl, &a.status->dt_next, &a.status->dt_next32);
}

// The batch run as one persistent launch (cooperative: every block is
// resident).  Each step runs the per-phase kernels' items in their order --
// CFL (each problem's minimum), slopes, faces (scaled by the problem's dt),
// each problem's dt and time, the cell update -- with a grid barrier between
// phases, so every cell and face gets the same operations on the same inputs
// as with one launch per phase (bit-identical results).  dt_trace[k] keeps
// problem 0's dt of step k.
__global__ void __launch_bounds__(kPersistBlock, 4)
    k_run32_persistent(MixedArgs a, int n_steps, int step0, GridBarrier* gb, int missing, double* dt_trace) {
  __shared__ unsigned int s_gen;
  __shared__ int s_ok;
  if (threadIdx.x == 0) s_gen = *reinterpret_cast<volatile unsigned int*>(&gb->gen);
  __syncthreads();
  unsigned int gen = s_gen;
  const unsigned int expected = gridDim.x + static_cast<unsigned int>(missing);
  const MeshDev& m = a.mesh;
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  for (int k = 0; k < n_steps; ++k) {
    a.step = step0 + k < 0x1fff ? step0 + k : 0x1fff;
    // CFL: each problem's minimum bound (k_cfl32's batch branch)
    for (int base = blockIdx.x * blockDim.x; base < m.n; base += stride) {
      const int t = base + threadIdx.x;
      const float x = t < m.n ? cfl32_cell<true>(a, t) : __int_as_float(0x7f800000);
      problem_min(a.dtmin_p, t < m.n ? a.cell_problem[t] : -1,
                  static_cast<unsigned long long>(__double_as_longlong(widen_exact(x))));
    }
    if (!grid_sync(gb, gen, expected, s_ok, a.status, a.step)) return;
    for (int i = t0; i < m.n; i += stride) k_slopes32_item<true, 1>(a, i);
    if (!grid_sync(gb, gen, expected, s_ok, a.status, a.step)) return;
    for (int e = t0; e < m.e; e += stride) k_faces32_lgi_item<true, true>(a, e);
    if (!grid_sync(gb, gen, expected, s_ok, a.status, a.step)) return;
    // each problem's dt and time (k_update_mixed's batch branch), the update
    for (int p = t0; p < a.n_problems; p += stride) {
      const double dt = a.cfl * __longlong_as_double(static_cast<long long>(a.dtmin_p[p]));
      a.dt_p[p] = dt;
      a.time_p[p] += dt;
      a.dtmin_p[p] = kInfBits;
      if (p == 0 && dt_trace) dt_trace[k] = dt;
    }
    for (int i = t0; i < m.n; i += stride) k_update_mixed_item<true>(a, i, 0, 1, 1);
    if (!grid_sync(gb, gen, expected, s_ok, a.status, a.step)) return;
  }
}

__global__ void __launch_bounds__(kPersistBlock) k_barrier_check(GridBarrier* gb, int missing, DevStatus* st) {
  __shared__ unsigned int s_gen;
  __shared__ int s_ok;
  if (threadIdx.x == 0) s_gen = *reinterpret_cast<volatile unsigned int*>(&gb->gen);
  __syncthreads();
  unsigned int gen = s_gen;
  grid_sync(gb, gen, gridDim.x + static_cast<unsigned int>(missing), s_ok, st, 0);
}

inline int blocks(int n) { return (n + kBlock - 1) / kBlock; }

}  // namespace

cudaError_t launch_geom32(const MixedGeomArgs& a, cudaStream_t s) {
  const int work = a.e > a.m ? (a.e > a.n ? a.e : a.n) : (a.m > a.n ? a.m : a.n);
  const int nb = blocks(work > 0 ? work : 1);
  k_geom32<<<nb < 4096 ? nb : 4096, kBlock, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_geom32_direct(const GeomArgs& ga, const MixedGeomArgs& a, cudaStream_t s) {
  if (a.e > 0) k_geom_faces32<<<blocks(a.e), kBlock, 0, s>>>(ga, a);
  const int work = a.n > a.g ? a.n : a.g;
  if (work > 0) k_geom_cells32<<<blocks(work), kBlock, 0, s>>>(ga, a);
  return cudaGetLastError();
}

cudaError_t launch_run32_persistent(const MixedArgs& a, int n_steps, int step0, GridBarrier* gb, int missing,
                                   double* dt_trace, cudaStream_t s, int* grid_out) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_run32_persistent, kPersistBlock, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorCooperativeLaunchTooLarge;
  // every block resident; no more blocks than the largest phase has items for
  const int work = a.mesh.e > a.mesh.n ? a.mesh.e : a.mesh.n;
  int grid = per_sm * sms;
  const int need = (work + kPersistBlock - 1) / kPersistBlock;
  if (need < grid) grid = need > 0 ? need : 1;
  if (grid_out) *grid_out = grid;
  e = cudaMemsetAsync(gb, 0, sizeof(GridBarrier), s);
  if (e != cudaSuccess) return e;
  MixedArgs ac = a;
  void* args[] = {&ac, &n_steps, &step0, &gb, &missing, &dt_trace};
  return cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(k_run32_persistent), dim3(grid),
                                     dim3(kPersistBlock), args, 0, s);
}

cudaError_t launch_barrier_check(GridBarrier* gb, int missing, DevStatus* st, cudaStream_t s) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaMemsetAsync(gb, 0, sizeof(GridBarrier), s);
  if (e != cudaSuccess) return e;
  void* args[] = {&gb, &missing, &st};
  return cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(k_barrier_check), dim3(2 * sms),
                                     dim3(kPersistBlock), args, 0, s);
}

cudaError_t launch_cells_to32(const double* c64, float4* c32, int n, cudaStream_t s) {
  if (n > 0) k_cells_to32<<<blocks(n), kBlock, 0, s>>>(c64, c32, n);
  return cudaGetLastError();
}
cudaError_t launch_cells_to64(const float4* c32, double* c64, int n, cudaStream_t s) {
  if (n > 0) k_cells_to64<<<blocks(n), kBlock, 0, s>>>(c32, c64, n);
  return cudaGetLastError();
}
cudaError_t launch_vec2_to32(const double* v64, float2* v32, int n, cudaStream_t s) {
  if (n > 0) k_vec2_to32<<<blocks(n), kBlock, 0, s>>>(v64, v32, n);
  return cudaGetLastError();
}
cudaError_t launch_flux_to64(const float4* f32, double* f64, int n, cudaStream_t s) {
  if (n > 0) k_flux_to64<<<blocks(n), kBlock, 0, s>>>(f32, f64, n);
  return cudaGetLastError();
}
cudaError_t launch_flux_to32(const double* f64, float4* f32, int n, cudaStream_t s) {
  if (n > 0) k_flux_to32<<<blocks(n), kBlock, 0, s>>>(f64, f32, n);
  return cudaGetLastError();
}

cudaError_t launch_cfl32(const MixedArgs& a, cudaStream_t s, bool fill_ghosts) {
  const int total = a.mesh.n + (fill_ghosts ? a.mesh.g : 0);
  if (a.cell_problem)
    k_cfl32<true><<<grid_of(a.shapes.cfl, total), a.shapes.cfl.block, 0, s>>>(a, fill_ghosts ? 1 : 0);
  else
    k_cfl32<false><<<grid_of(a.shapes.cfl, total), a.shapes.cfl.block, 0, s>>>(a, fill_ghosts ? 1 : 0);
  return cudaGetLastError();
}
cudaError_t launch_ghost_fill32(const MixedArgs& a, cudaStream_t s) {
  if (a.mesh.g > 0) k_ghost_fill32<<<blocks(a.mesh.g), kBlock, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch_slopes32_trace(const MixedArgs& a, double* slopes64, SlopeTrace* trace, cudaStream_t s) {
  if (a.mesh.n > 0) k_slopes32_trace<<<(a.mesh.n + kBlock - 1) / kBlock, kBlock, 0, s>>>(a, slopes64, trace);
  return cudaGetLastError();
}

cudaError_t launch_slopes32(const MixedArgs& a, cudaStream_t s) {
  if (a.mesh.n > 0) {
    const LaunchShape& sh = a.shapes.slopes;
    const int nb = grid_of(sh, a.mesh.n), bs = sh.block;
    const bool b = a.cell_problem != nullptr;
    // builds: 0 plain, 1 neighbour loops unrolled by 2, 2 and 3 register-capped
    // for 5 and 6 resident blocks of up to 256 threads, 4 neighbours prefetched
    switch (sh.variant) {
      case 4: b ? k_slopes32_pf<true><<<nb, bs, 0, s>>>(a) : k_slopes32_pf<false><<<nb, bs, 0, s>>>(a); break;
      case 1: b ? k_slopes32<true, 0, 2><<<nb, bs, 0, s>>>(a) : k_slopes32<false, 0, 2><<<nb, bs, 0, s>>>(a); break;
      case 2: b ? k_slopes32<true, 5, 1><<<nb, bs, 0, s>>>(a) : k_slopes32<false, 5, 1><<<nb, bs, 0, s>>>(a); break;
      case 3: b ? k_slopes32<true, 6, 1><<<nb, bs, 0, s>>>(a) : k_slopes32<false, 6, 1><<<nb, bs, 0, s>>>(a); break;
      default: b ? k_slopes32<true, 0, 1><<<nb, bs, 0, s>>>(a) : k_slopes32<false, 0, 1><<<nb, bs, 0, s>>>(a);
    }
  }
  return cudaGetLastError();
}
cudaError_t launch_faces32(const MixedArgs& a, cudaStream_t s, bool scaled) {
  if (a.mesh.e == 0) return cudaSuccess;
  const int nb = grid_of(a.shapes.faces, a.mesh.e), bs = a.shapes.faces.block;
  const bool b = a.cell_problem != nullptr;
  if (a.order == 1) {
    if (scaled)
      b ? k_faces32_pcm<true, true><<<nb, bs, 0, s>>>(a) : k_faces32_pcm<true, false><<<nb, bs, 0, s>>>(a);
    else
      b ? k_faces32_pcm<false, true><<<nb, bs, 0, s>>>(a) : k_faces32_pcm<false, false><<<nb, bs, 0, s>>>(a);
  } else if (a.shapes.faces.variant == 1) {
    // two threads per face: the one-thread-per-item grid covers 2 e threads
    const int np = grid_of(a.shapes.faces, 2 * a.mesh.e);
    if (scaled)
      b ? k_faces32_lgi_pair<true, true><<<np, bs, 0, s>>>(a) : k_faces32_lgi_pair<true, false><<<np, bs, 0, s>>>(a);
    else
      b ? k_faces32_lgi_pair<false, true><<<np, bs, 0, s>>>(a) : k_faces32_lgi_pair<false, false><<<np, bs, 0, s>>>(a);
  } else {
    if (scaled)
      b ? k_faces32_lgi<true, true><<<nb, bs, 0, s>>>(a) : k_faces32_lgi<true, false><<<nb, bs, 0, s>>>(a);
    else
      b ? k_faces32_lgi<false, true><<<nb, bs, 0, s>>>(a) : k_faces32_lgi<false, false><<<nb, bs, 0, s>>>(a);
  }
  return cudaGetLastError();
}
cudaError_t launch_update_mixed(const MixedArgs& a, cudaStream_t s, bool from_unscaled, bool extensive, bool cells) {
  const int work = a.cell_problem && a.n_problems > a.mesh.n ? a.n_problems : a.mesh.n;
  if (work > 0) {
    const LaunchShape& sh = a.shapes.update;
    const int nb = grid_of(sh, work), bs = sh.block;
    const int fu = from_unscaled ? 1 : 0, ex = extensive ? 1 : 0, ce = cells ? 1 : 0;
    const bool b = a.cell_problem != nullptr;
    // builds: 0 plain, 2 and 3 register-capped for 5 and 6 resident blocks
    // of up to 256 threads
    switch (sh.variant) {
      case 2:
        b ? k_update_mixed<true, 5><<<nb, bs, 0, s>>>(a, fu, ex, ce) : k_update_mixed<false, 5><<<nb, bs, 0, s>>>(a, fu, ex, ce);
        break;
      case 3:
        b ? k_update_mixed<true, 6><<<nb, bs, 0, s>>>(a, fu, ex, ce) : k_update_mixed<false, 6><<<nb, bs, 0, s>>>(a, fu, ex, ce);
        break;
      default:
        b ? k_update_mixed<true><<<nb, bs, 0, s>>>(a, fu, ex, ce) : k_update_mixed<false><<<nb, bs, 0, s>>>(a, fu, ex, ce);
    }
  }
  return cudaGetLastError();
}

}  // namespace rg
