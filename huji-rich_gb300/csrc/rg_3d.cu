// rg_3d.cu -- FP64 kernels of the 3D first-order path (HDSim3D on a fixed
// mesh), compiled without FMA contraction: every operation rounds as the
// reference's does, in its evaluation order.
//
//   k3_cfl     per cell width/(|v| + c), grid minimum, times cfl
//              (CourantFriedrichsLewy.cpp:23-46)
//   k3_faces   per face FirstOrderHydroFlux (FirstOrderHydroFlux.cpp:42-114):
//              rigid wall against the reflected state on boundary faces, Hllc
//              on (v.n, |v - (v.n)n|) in the bulk, momentum rebuilt along the
//              normal and the donor's tangential direction; optionally times
//              dt*area (hdsim_3d.cpp:63-76)
//   k3_update  per cell: the face deltas in ascending face order (the order
//              update_extensive applies them to the cell), then
//              extensive/volume and DefaultCellUpdater
//              (default_cell_updater.cpp:5-14, ideal_gas.cpp:18-23)
//   k3_init    ExtensiveGenerator (extensive_generator.cpp:3-28)
#include <math.h>

#include "rg_3d.cuh"
#include "rg_hllc.cuh"

namespace rg {
namespace {

constexpr int kBlock = 256;

struct V3 {
  double x, y, z;
};
// Vector3D.cpp: abs, ScalarProd, d*v (v.x*d), v/d, -, +
__device__ __forceinline__ double vabs(V3 v) { return root(v.x * v.x + v.y * v.y + v.z * v.z); }
__device__ __forceinline__ double vdot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 vscale(double d, V3 v) { return V3{v.x * d, v.y * d, v.z * d}; }
__device__ __forceinline__ V3 vdiv(V3 v, double d) { return V3{quot(v.x, d), quot(v.y, d), quot(v.z, d)}; }
__device__ __forceinline__ V3 vsub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 vadd(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }

struct Cell3 {
  double d, p;
  V3 v;
};
__device__ __forceinline__ Cell3 load_cell3(const double* c, int i) {
  const double2* r = reinterpret_cast<const double2*>(c) + 3 * i;
  const double2 a = r[0], b = r[1], cz = r[2];
  return Cell3{a.x, a.y, V3{b.x, b.y, cz.x}};
}
__device__ __forceinline__ void store6(double* out, int i, double a, double b, double c, double d, double e) {
  double2* r = reinterpret_cast<double2*>(out) + 3 * i;
  r[0] = make_double2(a, b);
  r[1] = make_double2(c, d);
  r[2] = make_double2(e, 0.0);
}

__device__ __forceinline__ double dp2e(double g, double d, double p) { return quot(quot(p, d), g - 1); }
__device__ __forceinline__ double dp2c(double g, double d, double p) { return root(quot(g * p, d)); }

// FirstOrderHydroFlux.cpp:32-40 calc_primitive: (d, p, (v.n, |v - (v.n)n|), e, c)
__device__ __forceinline__ Prim prim3(double g, const Cell3& c, V3 n) {
  const double sp = vdot(c.v, n);
  return Prim{c.d, c.p, sp, vabs(vsub(c.v, vscale(sp, n))), dp2e(g, c.d, c.p), dp2c(g, c.d, c.p)};
}

// FirstOrderHydroFlux.cpp:16-30 GetParallel
__device__ __forceinline__ V3 parallel3(V3 vel, V3 n) {
  V3 par = vsub(vel, vscale(vdot(vel, n), n));
  const double p = vabs(par);
  const double v = vabs(vel);
  if (1e-9 > fabs(v - 0)) return par;
  return p < 1e-8 * v ? vdiv(par, v) : vdiv(par, p);
}

// Vector3D.cpp:203-206 Reflect: v - 2*ScalarProd(v,n)*n/pow(abs(n),2)
__device__ __forceinline__ V3 reflect3(V3 v, V3 n) {
  const double s = 2 * vdot(v, n);
  const double a = vabs(n);
  return vsub(v, vdiv(vscale(s, n), a * a));
}

// ---------------------------------------------------------------- mesh checks

// Every index of a packed 3D mesh, before any other kernel uses it.
__global__ void __launch_bounds__(kBlock) k3_validate(Mesh3Dev m, DevStatus* st) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < m.e) {
    const int2 fc = m.face_cells[t];
    if (fc.x < -1 || fc.x >= m.n || fc.y < -1 || fc.y >= m.n || (fc.x < 0 && fc.y < 0))
      record_error(st, 0, RG_ERR_INVALID_ARGUMENT, 0, t, fc.x < -1 || fc.x >= m.n ? fc.x : fc.y);
  }
  if (t < m.n) {
    const int b = m.cell_off[t], e1 = m.cell_off[t + 1];
    if (b < 0 || e1 < b || e1 > m.m)
      record_error(st, 0, RG_ERR_INVALID_ARGUMENT, 2, t, e1);
    else
      for (int k = b; k < e1; ++k) {
        const int f = m.cell_faces[k];
        if (f < 0 || f >= m.e) {
          record_error(st, 0, RG_ERR_INVALID_ARGUMENT, 2, t, f);
          break;
        }
        const int2 fc = m.face_cells[f];
        if (fc.x != t && fc.y != t) {
          record_error(st, 0, RG_ERR_INVALID_ARGUMENT, 2, t, f);
          break;
        }
      }
  }
}

// Unit normals (FirstOrderHydroFlux.cpp:11-14 normalize) and the CSR signs.
__global__ void __launch_bounds__(kBlock) k3_geometry(Mesh3Dev m, dbl4* nhat, int* fsign) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < m.e) {
    const V3 n{m.normal[3 * t], m.normal[3 * t + 1], m.normal[3 * t + 2]};
    const V3 u = vdiv(n, vabs(n));
    nhat[t] = make_dbl4(u.x, u.y, u.z, 0.0);
  }
  if (t < m.n)
    for (int k = m.cell_off[t]; k < m.cell_off[t + 1]; ++k) {
      const int f = m.cell_faces[k];
      fsign[k] = f | (m.face_cells[f].x == t ? static_cast<int>(0x80000000u) : 0);
    }
}

// ---------------------------------------------------------------- step

__global__ void __launch_bounds__(kBlock) k3_cfl(Step3Args a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long bits = kInfBits;
  if (i < a.mesh.n) {
    const Cell3 c = load_cell3(a.cells, i);
    const double b = quot(a.mesh.width[i], vabs(c.v) + dp2c(a.gamma, c.d, c.p));
    bits = static_cast<unsigned long long>(__double_as_longlong(b));
  }
  grid_min_times(a.status, bits, a.cfl, &a.status->dt);
}

template <bool kScaled>
__global__ void __launch_bounds__(kBlock) k3_faces(Step3Args a) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= a.mesh.e) return;
  const int2 fc = a.mesh.face_cells[f];
  const dbl4 nn = a.nhat[f];
  const V3 n{nn.x, nn.y, nn.z};
  Cons sol;
  V3 par;
  if (fc.x < 0 || fc.y < 0) {
    // CalcRigidWall: the real cell against its reflection
    const bool real_first = fc.x >= 0;
    const Cell3 real = load_cell3(a.cells, real_first ? fc.x : fc.y);
    const Prim preal = prim3(a.gamma, real, n);
    par = parallel3(real.v, n);
    Cell3 other = real;
    other.v = reflect3(real.v, n);
    const Prim pghost = prim3(a.gamma, other, n);
    const bool ok = real_first ? hllc(preal, pghost, 0.0, sol, a.status, a.step, f)
                               : hllc(pghost, preal, 0.0, sol, a.status, a.step, f);
    if (!ok) return;
  } else {
    // CalcSingleFluxInBulk
    double fv = 0.0;
    if (a.fvel) fv = vdot(V3{a.fvel[3 * f], a.fvel[3 * f + 1], a.fvel[3 * f + 2]}, n);
    const Cell3 ca = load_cell3(a.cells, fc.x), cb = load_cell3(a.cells, fc.y);
    if (!hllc(prim3(a.gamma, ca, n), prim3(a.gamma, cb, n), fv, sol, a.status, a.step, f)) return;
    par = parallel3(sol.m > 0 ? ca.v : cb.v, n);
  }
  // Conserved3D(sol.Mass, sol.Momentum.x*normal + sol.Momentum.y*parallel, sol.Energy)
  const V3 mom = vadd(vscale(sol.mx, n), vscale(sol.my, par));
  if (kScaled) {
    const double s = (a.dt_from_device ? a.status->dt : a.dt_host) * a.mesh.area[f];
    store6(a.fluxes, f, s * sol.m, s * mom.x, s * mom.y, s * mom.z, s * sol.en);
  } else {
    store6(a.fluxes, f, sol.m, mom.x, mom.y, mom.z, sol.en);
  }
}

__global__ void __launch_bounds__(kBlock) k3_update(Step3Args a, int from_unscaled, int do_ext, int do_cells) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const Mesh3Dev& m = a.mesh;
  if (i >= m.n) return;
  const double2* e2 = reinterpret_cast<const double2*>(a.ext) + 3 * i;
  const double2 e01 = e2[0], e23 = e2[1], e45 = e2[2];
  double u[5] = {e01.x, e01.y, e23.x, e23.y, e45.x};
  if (do_ext) {
    const double dt = from_unscaled ? (a.dt_from_device ? a.status->dt : a.dt_host) : 0.0;
    for (int k = m.cell_off[i]; k < m.cell_off[i + 1]; ++k) {
      const int fs = a.fsign[k];
      const int f = fs & 0x7fffffff;
      const double2* fl = reinterpret_cast<const double2*>(a.fluxes) + 3 * f;
      const double2 f01 = fl[0], f23 = fl[1], f45 = fl[2];
      double d[5] = {f01.x, f01.y, f23.x, f23.y, f45.x};
      if (from_unscaled) {
        const double s = dt * m.area[f];  // dt*GetArea()*flux (hdsim_3d.cpp:69)
#pragma unroll
        for (int q = 0; q < 5; ++q) d[q] = s * d[q];
      }
#pragma unroll
      for (int q = 0; q < 5; ++q) u[q] = fs < 0 ? u[q] - d[q] : u[q] + d[q];
    }
    store6(a.ext, i, u[0], u[1], u[2], u[3], u[4]);
  }
  if (do_cells) {
    const double V = m.volume[i];
    const double density = quot(u[0], V);
    const V3 vel = vdiv(V3{quot(u[1], V), quot(u[2], V), quot(u[3], V)}, density);
    const double thermal = quot(u[4], V) - 0.5 * density * vdot(vel, vel);
    const double eint = quot(thermal, density);
    if (eint < 0) {
      record_error(a.status, a.step, RG_ERR_NEGATIVE_ENERGY, 5, i, eint);
      return;
    }
    store6(a.cells, i, density, (a.gamma - 1) * eint * density, vel.x, vel.y, vel.z);
  }
}

__global__ void __launch_bounds__(kBlock) k3_init(Step3Args a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.mesh.n) return;
  const Cell3 c = load_cell3(a.cells, i);
  const double V = a.mesh.volume[i];
  const V3 mom = vscale(c.d, c.v);
  const double en = c.d * (0.5 * vdot(c.v, c.v) + dp2e(a.gamma, c.d, c.p));
  store6(a.ext, i, V * c.d, mom.x * V, mom.y * V, mom.z * V, V * en);
}

inline int blocks(int n) { return n > 0 ? (n + kBlock - 1) / kBlock : 1; }

}  // namespace

cudaError_t launch3_validate(const Mesh3Dev& m, DevStatus* st, cudaStream_t s) {
  k3_validate<<<blocks(m.e > m.n ? m.e : m.n), kBlock, 0, s>>>(m, st);
  return cudaGetLastError();
}

cudaError_t launch3_geometry(const Mesh3Dev& m, dbl4* nhat, int* fsign, cudaStream_t s) {
  k3_geometry<<<blocks(m.e > m.n ? m.e : m.n), kBlock, 0, s>>>(m, nhat, fsign);
  return cudaGetLastError();
}

cudaError_t launch3_init_extensives(const Step3Args& a, cudaStream_t s) {
  k3_init<<<blocks(a.mesh.n), kBlock, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch3_cfl(const Step3Args& a, cudaStream_t s) {
  k3_cfl<<<blocks(a.mesh.n), kBlock, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch3_faces(const Step3Args& a, bool scaled, cudaStream_t s) {
  if (a.mesh.e == 0) return cudaSuccess;
  if (scaled)
    k3_faces<true><<<blocks(a.mesh.e), kBlock, 0, s>>>(a);
  else
    k3_faces<false><<<blocks(a.mesh.e), kBlock, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch3_update(const Step3Args& a, bool from_unscaled, bool do_ext, bool do_cells, cudaStream_t s) {
  k3_update<<<blocks(a.mesh.n), kBlock, 0, s>>>(a, from_unscaled ? 1 : 0, do_ext ? 1 : 0, do_cells ? 1 : 0);
  return cudaGetLastError();
}

}  // namespace rg
