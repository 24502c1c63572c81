// rg_adjoint.cu -- forward side of the differentiated step (FP64, compiled
// without FMA contraction like rg_fp64.cu):
//
//   k_record_slopes  LinearGaussImproved slopes of W_k, as rg_fp64.cu's
//                    k_slopes computes them, plus the limiter trace the
//                    reverse slope kernel needs (SlopeTrace)
//   k_tl_*           tangent-linear model: the same formulas on dual numbers
//                    (value, tangent).  The value parts follow the production
//                    kernels' operation order, so a tangent run reproduces the
//                    plain FP64 trajectory bit for bit.
//
// Branches (shock test, limiter thresholds and candidates, neighbour max/min,
// HLLC wave speeds and region) are decided on the values; the tangents are
// the derivatives of the branch taken.  Only periodic meshes (every ghost a
// copy of its source cell, no self-mirror neighbours) are differentiated.
#include <math.h>

#include "rg_adjoint.cuh"
#include "rg_div.cuh"

namespace rg {
namespace {

constexpr int kBlock = 256;

// ---------------------------------------------------------------- dual numbers

struct Dual {
  double v, d;
};
using ::rg::quot;  // the double overload, beside the Dual ones below
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return Dual{a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return Dual{a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return Dual{a.v * b.v, a.d * b.v + a.v * b.d}; }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
  const double q = quot(a.v, b.v);
  return Dual{q, quot(a.d - q * b.d, b.v)};
}
__device__ __forceinline__ Dual operator*(Dual a, double b) { return Dual{a.v * b, a.d * b}; }
__device__ __forceinline__ Dual operator*(double a, Dual b) { return Dual{a * b.v, a * b.d}; }
__device__ __forceinline__ Dual operator/(Dual a, double b) { return Dual{quot(a.v, b), quot(a.d, b)}; }
// quotients of the templated code: rg::quot for double, the operators for Dual
__device__ __forceinline__ Dual quot(Dual a, Dual b) { return a / b; }
__device__ __forceinline__ Dual quot(Dual a, double b) { return a / b; }
__device__ __forceinline__ Dual operator-(Dual a, double b) { return Dual{a.v - b, a.d}; }
__device__ __forceinline__ Dual dsqrt(Dual a) {
  const double s = root(a.v);
  return Dual{s, quot(a.d, 2.0 * s)};
}
__device__ __forceinline__ double dsqrt(double a) { return root(a); }
__device__ __forceinline__ double val(double x) { return x; }
__device__ __forceinline__ double val(Dual x) { return x.v; }
__device__ __forceinline__ double tan_of(Dual x) { return x.d; }
__device__ __forceinline__ double tan_of(double) { return 0.0; }
template <class T>
__device__ __forceinline__ T constant(double x);
template <>
__device__ __forceinline__ double constant<double>(double x) { return x; }
template <>
__device__ __forceinline__ Dual constant<Dual>(double x) { return Dual{x, 0.0}; }

// {density, pressure, vx, vy}
template <class T>
struct V4 {
  T v[4];
};

__device__ __forceinline__ void load_raw(const double* c, int i, double o[4]) {
  const double2 a = reinterpret_cast<const double2*>(c)[2 * i];
  const double2 b = reinterpret_cast<const double2*>(c)[2 * i + 1];
  o[0] = a.x;
  o[1] = a.y;
  o[2] = b.x;
  o[3] = b.y;
}
__device__ __forceinline__ void store_raw(double* c, int i, double a, double b, double x, double y) {
  reinterpret_cast<double2*>(c)[2 * i] = make_double2(a, b);
  reinterpret_cast<double2*>(c)[2 * i + 1] = make_double2(x, y);
}

// record i of a 4-double array with (for Dual) its tangent record
template <class T>
__device__ __forceinline__ V4<T> load4(const double* c, const double* dc, int i);
template <>
__device__ __forceinline__ V4<double> load4<double>(const double* c, const double*, int i) {
  V4<double> r;
  load_raw(c, i, r.v);
  return r;
}
template <>
__device__ __forceinline__ V4<Dual> load4<Dual>(const double* c, const double* dc, int i) {
  double x[4], t[4];
  load_raw(c, i, x);
  load_raw(dc, i, t);
  return V4<Dual>{{{x[0], t[0]}, {x[1], t[1]}, {x[2], t[2]}, {x[3], t[3]}}};
}

// state of point p: a real cell, or the source of a periodic ghost
// (PeriodicGhostGenerator.cpp:3-17 copies the source cell)
__device__ __forceinline__ int source_of(const MeshDev& m, int p) { return p < m.n ? p : m.ghost_source[p - m.n]; }
__device__ __forceinline__ int entry_source(const AdjArgs& a, int k) {
  return source_of(a.mesh, static_cast<int>(a.geom.nbr[k] & kNbrIdMask));
}

// ---------------------------------------------------------------- slopes

// LinearGaussImproved.cpp:67-134 (naive slope), :136-157 (is_shock),
// :174-399 (the two limiters) for a real cell with no self-mirror
// neighbour, in the operation order of rg_fp64.cu's k_slopes.
template <class T, bool kTrace>
__device__ void lgi_slope(const AdjArgs& a, int i, V4<T>& sx, V4<T>& sy) {
  const MeshDev& m = a.mesh;
  const V4<T> cell = load4<T>(a.cells, a.dcells, i);
  const int b = m.cell_off[i], nn = m.cell_off[i + 1] - b;
  const dbl4 mi = a.geom.minv[i];
  V4<T> vx, vy;
#pragma unroll
  for (int q = 0; q < 4; ++q) vx.v[q] = vy.v[q] = constant<T>(0.0);
  for (int k = 0; k < nn; ++k) {
    const V4<T> nb = load4<T>(a.cells, a.dcells, entry_source(a, b + k));
    const double2 h = a.geom.hr[b + k];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (k == 0) {
        vx.v[q] = cell.v[q] * h.x;
        vy.v[q] = cell.v[q] * h.y;
      } else {
        vx.v[q] = vx.v[q] + cell.v[q] * h.x;
        vy.v[q] = vy.v[q] + cell.v[q] * h.y;
      }
      vy.v[q] = vy.v[q] + nb.v[q] * h.y;
      vx.v[q] = vx.v[q] + nb.v[q] * h.x;
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    sx.v[q] = vx.v[q] * mi.x + vy.v[q] * mi.y;
    sy.v[q] = vy.v[q] * mi.w + vx.v[q] * mi.z;
  }
  SlopeTrace* tr = kTrace ? a.trace + i : nullptr;
  if (kTrace) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      tr->naive[q] = val(sx.v[q]);
      tr->naive[4 + q] = val(sy.v[q]);
    }
  }
  int code[4] = {kTraceNone, kTraceNone, kTraceNone, kTraceNone};
  double dphi_at[4] = {0, 0, 0, 0};
  T psi[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) psi[q] = constant<T>(1.0);
  if (a.slf) {
    double cq_[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) cq_[q] = val(cell.v[q]);
    // is_shock: (div v)*width < -delta_v*cs, or some neighbour pressure ratio < delta_p
    const double lhs = (val(sx.v[2]) + val(sy.v[3])) * a.geom.width[i];
    bool shock = lhs < (-a.delta_v) * root(quot(a.gamma * cq_[1], cq_[0]));
    if (!shock && nn == 0) shock = 1.0 < a.delta_p;
    for (int k = 0; k < nn && !shock; ++k) {
      const double np_ = a.cells[4 * entry_source(a, b + k) + 1];
      const double num = cq_[1] > np_ ? np_ : cq_[1];
      const double den = cq_[1] > np_ ? cq_[1] : np_;
      shock = quot(num, den) < a.delta_p;
    }
    // neighbour max / min (the first strict improvement is kept, as std::max/min)
    double cmax[4], cmin[4];
    int amax[4] = {-1, -1, -1, -1}, amin[4] = {-1, -1, -1, -1};
#pragma unroll
    for (int q = 0; q < 4; ++q) cmax[q] = cmin[q] = cq_[q];
    for (int k = 0; k < nn; ++k) {
      double nv[4];
      load_raw(a.cells, entry_source(a, b + k), nv);
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
    }
    const double f = shock ? 0.1 : 0.05;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const double cq = cq_[q];
      const double maxd = cmax[q] - cq, mind = cmin[q] - cq;
      const double thr = f * smax(fabs(maxd), fabs(mind));
      // the numerators as functions of the state: neighbour (or cell) minus cell
      T nmax = constant<T>(0.0), nmin = constant<T>(0.0);
      if (amax[q] >= 0) nmax = load4<T>(a.cells, a.dcells, entry_source(a, b + amax[q])).v[q] - cell.v[q];
      if (amin[q] >= 0) nmin = load4<T>(a.cells, a.dcells, entry_source(a, b + amin[q])).v[q] - cell.v[q];
      for (int k = 0; k < nn; ++k) {
        const int e = m.cell_faces[b + k];
        const double2 dm = (a.geom.nbr[b + k] & kNbrFirst) ? a.geom.dm0[e] : a.geom.dm1[e];
        T cv = cell.v[q] + sx.v[q] * dm.x;
        cv = cv + sy.v[q] * dm.y;
        const T dphi = cv - cell.v[q];
        const double dv = val(dphi);
        if (!(abs_gt(dv, thr) || prod_neg(val(cv), cq))) continue;  // integer-pipe tests (rg_convert.cuh)
        if (!shock) {
          const bool use_abs = q >= 2;
          const double t1 = use_abs ? fabs(1e-9 * cq) : 1e-9 * cq;
          const double t2 = use_abs ? -fabs(1e-9 * cq) : -1e-9 * cq;
          if (dv > t1 || dv < t2) {
            const bool up = dv > t1;
            const T cand = quot(up ? nmax : nmin, dphi);
            if (val(cand) < val(psi[q])) {
              psi[q] = cand;
              const int ex = up ? amax[q] : amin[q];
              code[q] = k | ((up ? 0 : 1) << 8) | ((ex + 1) << 16);
              dphi_at[q] = dv;
            }
          }
        } else if (fabs(dv) > 1e-9 * cq) {
          const T nb = load4<T>(a.cells, a.dcells, entry_source(a, b + k)).v[q];
          const T cand = quot(a.theta * (nb - cell.v[q]), dphi);
          const bool clamp = val(cand) < 0.0;  // std::max(cand, 0)
          const T x = clamp ? constant<T>(0.0) : cand;
          if (val(x) < val(psi[q])) {
            psi[q] = x;
            code[q] = k | ((clamp ? 3 : 2) << 8) | ((k + 1) << 16);
            dphi_at[q] = dv;
          }
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    sx.v[q] = sx.v[q] * psi[q];
    sy.v[q] = sy.v[q] * psi[q];
  }
  if (kTrace) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      tr->psi[q] = val(psi[q]);
      tr->dphi[q] = dphi_at[q];
      tr->code[q] = code[q];
    }
  }
}

template <class T>
__device__ __forceinline__ void store_slope(const AdjArgs& a, int i, const V4<T>& sx, const V4<T>& sy) {
  store_raw(a.slopes, 2 * i, val(sx.v[0]), val(sx.v[1]), val(sx.v[2]), val(sx.v[3]));
  store_raw(a.slopes, 2 * i + 1, val(sy.v[0]), val(sy.v[1]), val(sy.v[2]), val(sy.v[3]));
  if (a.dslopes) {
    store_raw(a.dslopes, 2 * i, tan_of(sx.v[0]), tan_of(sx.v[1]), tan_of(sx.v[2]), tan_of(sx.v[3]));
    store_raw(a.dslopes, 2 * i + 1, tan_of(sy.v[0]), tan_of(sy.v[1]), tan_of(sy.v[2]), tan_of(sy.v[3]));
  }
}

__global__ void __launch_bounds__(kBlock) k_record_slopes(AdjArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.mesh.n) return;
  V4<double> sx, sy;
  lgi_slope<double, true>(a, i, sx, sy);
  store_slope(a, i, sx, sy);
}

__global__ void __launch_bounds__(kBlock) k_tl_slopes(AdjArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.mesh.n) return;
  V4<Dual> sx, sy;
  lgi_slope<Dual, false>(a, i, sx, sy);
  store_slope(a, i, sx, sy);
}

// ---------------------------------------------------------------- faces

// hydrodynamic_variables.cpp:261-265 TotalEnergyDensity: d*(0.5*|v|^2 + e)
// with |v| = sqrt(vx^2 + vy^2) squared again; the tangent uses |v|^2 directly
// (the square root has no derivative at rest).
__device__ __forceinline__ double ted(double d, double vx, double vy, double e) {
  const double s = root(vx * vx + vy * vy);
  return d * (0.5 * (s * s) + e);
}
__device__ __forceinline__ Dual ted(Dual d, Dual vx, Dual vy, Dual e) {
  const double v = ted(d.v, vx.v, vy.v, e.v);
  const double k2 = vx.v * vx.v + vy.v * vy.v;
  const double dk2 = 2.0 * (vx.v * vx.d + vy.v * vy.d);
  return Dual{v, d.d * (0.5 * k2 + e.v) + d.v * (0.5 * dk2 + e.d)};
}

// Hllc (hllc.cpp:97-154, massflux, face at rest) between the rotated states
// and the rotation back (simple_flux_calculator.cpp:130-165); the result is
// {mass, energy, px, py}.  Returns false on invalid wave speeds.
template <class T>
__device__ bool face_flux(const AdjArgs& a, int e, const V4<T>& L, const V4<T>& R, T out[4]) {
  const double g = a.gamma;
  const double2 n = a.geom.nrm[e], p = a.geom.par[e];
  const double na = a.geom.nabs[e], pa = a.geom.area[e];
  const T le = quot(quot(L.v[1], L.v[0]), g - 1), lc = dsqrt(quot(g * L.v[1], L.v[0]));
  const T re = quot(quot(R.v[1], R.v[0]), g - 1), rc = dsqrt(quot(g * R.v[1], R.v[0]));
  const T lu = quot(L.v[2] * n.x + L.v[3] * n.y, na), lv = quot(L.v[2] * p.x + L.v[3] * p.y, pa);
  const T ru = quot(R.v[2] * n.x + R.v[3] * n.y, na), rv = quot(R.v[2] * p.x + R.v[3] * p.y, pa);
  const T a1 = lu - lc, b1 = ru - rc, a2 = lu + lc, b2 = ru + rc;
  const T sl = val(b1) < val(a1) ? b1 : a1;
  const T sr = val(a2) < val(b2) ? b2 : a2;
  const T ss = (R.v[1] - L.v[1] + L.v[0] * lu * (sl - lu) - R.v[0] * ru * (sr - ru)) /
               (L.v[0] * (sl - lu) - R.v[0] * (sr - ru));
  const bool use_left = val(sl) > 0 || (val(sl) <= 0 && val(ss) >= 0);
  const bool use_right = !use_left && ((val(ss) < 0 && val(sr) >= 0) || val(sr) < 0);
  if (!use_left && !use_right) return false;
  const T qd = use_left ? L.v[0] : R.v[0], qp = use_left ? L.v[1] : R.v[1];
  const T qu = use_left ? lu : ru, qv = use_left ? lv : rv, qe = use_left ? le : re;
  const T sk = use_left ? sl : sr;
  const T ek = ted(qd, qu, qv, qe);
  const T dsp = qd * qu;
  T fm = dsp, fmx = qp + qu * dsp, fmy = qv * dsp, fen = (ek + qp) * qu;
  if (use_left ? !(val(sl) > 0) : !(val(sr) < 0)) {
    const T ds = quot(qd * (sk - qu), sk - ss);
    const T use = quot(ek * ds, qd) + ds * (ss - qu) * (ss + quot(quot(qp, qd), sk - qu));
    fm = fm + sk * (ds - qd);
    fmx = fmx + (ds * ss - qu * qd) * sk;
    fmy = fmy + (ds * qv - qv * qd) * sk;
    fen = fen + sk * (use - ek);
  }
  out[0] = fm;
  out[1] = fen;
  out[2] = quot(n.x * fmx, na) + quot(p.x * fmy, pa);
  out[3] = quot(n.y * fmx, na) + quot(p.y * fmy, pa);
  return true;
}

// LinearGaussImproved.cpp:570-634 face state: the source cell plus its slope
// times (face centroid - centre of mass of the side's point)
__device__ __forceinline__ V4<Dual> face_state(const AdjArgs& a, int pid, double2 dm) {
  const int sid = source_of(a.mesh, pid);
  V4<Dual> c = load4<Dual>(a.cells, a.dcells, sid);
  const V4<Dual> gx = load4<Dual>(a.slopes, a.dslopes, 2 * sid), gy = load4<Dual>(a.slopes, a.dslopes, 2 * sid + 1);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    c.v[q] = c.v[q] + gx.v[q] * dm.x;
    c.v[q] = c.v[q] + gy.v[q] * dm.y;
  }
  return c;
}

__global__ void __launch_bounds__(kBlock) k_tl_faces(AdjArgs a) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.mesh.e) return;
  const int2 fc = a.mesh.face_cells[e];
  const V4<Dual> l = face_state(a, fc.x, a.geom.dm0[e]), r = face_state(a, fc.y, a.geom.dm1[e]);
  Dual f[4];
  if (!face_flux<Dual>(a, e, l, r, f)) {
    record_error(a.status, 0, RG_ERR_HLLC_WAVE_SPEEDS, 3, e, 0.0);
    return;
  }
  const double s = a.dt * a.geom.area[e];  // simple_extensive_updater.cpp:26-27
  store_raw(a.flux, e, f[0].v * s, f[1].v * s, f[2].v * s, f[3].v * s);
  store_raw(a.dflux, e, f[0].d * s, f[1].d * s, f[2].d * s, f[3].d * s);
}

// ---------------------------------------------------------------- cells

// SimpleExtensiveUpdater gather and SimpleCellUpdater::regular_update
// (simple_cell_updater.cpp:22-59) with their tangents.
__global__ void __launch_bounds__(kBlock) k_tl_update(AdjArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const MeshDev& m = a.mesh;
  if (i >= m.n) return;
  double u[4], du[4];
  load_raw(a.ext_rw, i, u);
  load_raw(a.dext, i, du);
  for (int k = m.cell_off[i]; k < m.cell_off[i + 1]; ++k) {
    const int e = m.cell_faces[k];
    double f[4], df[4];
    load_raw(a.flux, e, f);
    load_raw(a.dflux, e, df);
    const bool first = a.geom.nbr[k] & kNbrFirst;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (first) {
        u[q] -= f[q];
        du[q] -= df[q];
      } else {
        u[q] += f[q];
        du[q] += df[q];
      }
    }
  }
  store_raw(a.ext_rw, i, u[0], u[1], u[2], u[3]);
  store_raw(a.dext, i, du[0], du[1], du[2], du[3]);
  const double V = m.cd_volume[i];
  const double mass = u[0], en = u[1];
  const double d = quot(mass, V);
  if (d < 0) {
    record_error(a.status, 0, RG_ERR_NEGATIVE_DENSITY, 5, i, d);
    return;
  }
  const double vx = quot(u[2], mass), vy = quot(u[3], mass);
  const double energy = quot(en, mass) - 0.5 * (vx * vx + vy * vy);
  if (energy < 0) {
    record_error(a.status, 0, RG_ERR_NEGATIVE_ENERGY, 5, i, energy);
    return;
  }
  store_raw(a.cells_out, i, d, (a.gamma - 1) * energy * d, vx, vy);
  const double dd = quot(du[0], V);
  const double dvx = quot(du[2] - vx * du[0], mass), dvy = quot(du[3] - vy * du[0], mass);
  const double de = quot(du[1] - quot(en, mass) * du[0], mass) - (vx * dvx + vy * dvy);
  store_raw(a.dcells_out, i, dd, (a.gamma - 1) * (de * d + energy * dd), dvx, dvy);
}

// hdsim2d.cpp:41-67 init_extensives with its tangent
__global__ void __launch_bounds__(kBlock) k_tl_init(AdjArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.mesh.n) return;
  double c[4], t[4];
  load_raw(a.cells, i, c);
  load_raw(a.dcells, i, t);
  const double V = a.mesh.cd_volume[i];
  const double mass = V * c[0];
  const double k2 = c[2] * c[2] + c[3] * c[3];
  store_raw(a.ext_rw, i, mass, quot(quot(c[1], c[0]), a.gamma - 1) * mass + 0.5 * mass * k2, c[2] * mass, c[3] * mass);
  const double dm = V * t[0];
  // E = V p / (gamma - 1) + V d |v|^2 / 2
  const double dE = quot(V * t[1], a.gamma - 1) + 0.5 * V * t[0] * k2 + V * c[0] * (c[2] * t[2] + c[3] * t[3]);
  store_raw(a.dext, i, dm, dE, t[2] * mass + c[2] * dm, t[3] * mass + c[3] * dm);
}

inline int blocks(int n) { return (n + kBlock - 1) / kBlock; }

}  // namespace

cudaError_t adj_launch_record_slopes(const AdjArgs& a, cudaStream_t s) {
  k_record_slopes<<<blocks(a.mesh.n), kBlock, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t tl_launch_init(const AdjArgs& a, cudaStream_t s) {
  k_tl_init<<<blocks(a.mesh.n), kBlock, 0, s>>>(a);
  return cudaGetLastError();
}

// One tangent-linear step: slopes and their tangents, fluxes, then the
// update (extensives in place, cells and tangents into cells_out/dcells_out).
cudaError_t tl_launch_step(const AdjArgs& a, cudaStream_t s) {
  k_tl_slopes<<<blocks(a.mesh.n), kBlock, 0, s>>>(a);
  k_tl_faces<<<blocks(a.mesh.e), kBlock, 0, s>>>(a);
  k_tl_update<<<blocks(a.mesh.n), kBlock, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace rg
