// rg_3d_mixed.cu -- FP32-mixed kernels of the 3D first-order path: the
// per-face work (primitives along the normal, Hllc, tangential rebuild) and
// the CFL bound in FP32 with FMA; each cell's FP32 face fluxes summed in
// float-float in ascending face order and added to the FP64 extensives, and
// the internal energy E/m - v^2/2 formed in FP64 (its cancellation at high
// Mach numbers).  Same structure as the FP64 kernels in rg_3d.cu.
#include <math.h>

#include "rg_3d.cuh"
#include "rg_convert.cuh"
#include "rg_hllc.cuh"

namespace rg {
namespace {

constexpr int kBlock = 256;

struct F3 {
  float x, y, z;
};
__device__ __forceinline__ float fabs3(F3 v) { return sqrtf(v.x * v.x + v.y * v.y + v.z * v.z); }
__device__ __forceinline__ float fdot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 fscale(float d, F3 v) { return F3{v.x * d, v.y * d, v.z * d}; }
__device__ __forceinline__ F3 fsub(F3 a, F3 b) { return F3{a.x - b.x, a.y - b.y, a.z - b.z}; }

struct C3 {
  float d, p;
  F3 v;
};
__device__ __forceinline__ C3 load32(const Mixed3Args& a, int i) {
  const float4 c = a.cells32[i];
  return C3{c.x, c.y, F3{c.z, c.w, a.vz32[i]}};
}

__device__ __forceinline__ PrimT<float> prim32(float g, const C3& c, F3 n) {
  const float sp = fdot(c.v, n);
  return PrimT<float>{c.d, c.p, sp, fabs3(fsub(c.v, fscale(sp, n))), c.p / c.d / (g - 1.0f), sqrtf(g * c.p / c.d)};
}

// FirstOrderHydroFlux.cpp:16-30 GetParallel
__device__ __forceinline__ F3 parallel32(F3 vel, F3 n) {
  const F3 par = fsub(vel, fscale(fdot(vel, n), n));
  const float p = fabs3(par), v = fabs3(vel);
  if (1e-9f > v) return par;
  return fscale(1.0f / (p < 1e-8f * v ? v : p), par);
}

// Vector3D.cpp:203-206 Reflect about a unit normal
__device__ __forceinline__ F3 reflect32(F3 v, F3 n) { return fsub(v, fscale(2.0f * fdot(v, n), n)); }

// float -> double on the integer pipe (exact for normal floats, zeros,
// infinities, NaN; subnormals become signed zeros)
__device__ __forceinline__ double widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned ex = (u >> 23) & 0xffu;
  const unsigned dex = ex == 0u ? 0u : (ex == 0xffu ? 0x7ffu : ex + 896u);
  const unsigned mant = ex == 0u ? 0u : (u & 0x7fffffu);
  return __hiloint2double(static_cast<int>((u & 0x80000000u) | (dex << 20) | (mant >> 3)),
                          static_cast<int>(mant << 29));
}
__device__ __forceinline__ void two_sum(float& s, float& c, float x) {
  const float t = s + x;
  const float bb = t - s;
  c += (s - (t - bb)) + (x - bb);
  s = t;
}

__global__ void __launch_bounds__(kBlock) k3m_geometry(Mesh3Dev m, const dbl4* nhat, float4* n32, float* a32,
                                                       float* w32) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < m.e) {
    const dbl4 v = nhat[t];
    n32[t] = make_float4(narrow(v.x), narrow(v.y), narrow(v.z), 0.0f);
    a32[t] = narrow(m.area[t]);
  }
  if (t < m.n) w32[t] = narrow(m.width[t]);
}

__global__ void __launch_bounds__(kBlock) k3m_to32(const double* c64, float4* c32, float* vz, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* c = c64 + 6 * i;
  c32[i] = make_float4(narrow(c[0]), narrow(c[1]), narrow(c[2]), narrow(c[3]));
  vz[i] = narrow(c[4]);
}

__global__ void __launch_bounds__(kBlock) k3m_to64(const float4* c32, const float* vz, double* c64, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 c = c32[i];
  double* o = c64 + 6 * i;
  o[0] = c.x;
  o[1] = c.y;
  o[2] = c.z;
  o[3] = c.w;
  o[4] = vz[i];
  o[5] = 0.0;
}

__global__ void __launch_bounds__(kBlock) k3m_flux_to64(const float4* f32, const float* fen, double* f64, int e) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= e) return;
  const float4 v = f32[f];
  double* o = f64 + 6 * f;
  o[0] = v.x;
  o[1] = v.y;
  o[2] = v.z;
  o[3] = v.w;
  o[4] = fen[f];
  o[5] = 0.0;
}

__global__ void __launch_bounds__(kBlock) k3m_cfl(Mixed3Args a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long bits = kInfBits;
  if (i < a.mesh.n) {
    const C3 c = load32(a, i);
    const float b = a.width32[i] / (fabs3(c.v) + sqrtf(a.gamma * c.p / c.d));
    bits = static_cast<unsigned long long>(__double_as_longlong(widen_exact(b)));
  }
  grid_min_times(a.status, bits, a.cfl, &a.status->dt, &a.status->dt32);
}

template <bool kScaled>
__global__ void __launch_bounds__(kBlock) k3m_faces(Mixed3Args a) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= a.mesh.e) return;
  const int2 fc = a.mesh.face_cells[f];
  const float4 nn = a.nhat32[f];
  const F3 n{nn.x, nn.y, nn.z};
  ConsT<float> sol;
  F3 par;
  if (fc.x < 0 || fc.y < 0) {
    const bool real_first = fc.x >= 0;
    const C3 real = load32(a, real_first ? fc.x : fc.y);
    C3 other = real;
    other.v = reflect32(real.v, n);
    const PrimT<float> pr = prim32(a.gamma, real, n), pg = prim32(a.gamma, other, n);
    par = parallel32(real.v, n);
    const bool ok = real_first ? hllc(pr, pg, 0.0f, sol, a.status, a.step, f) : hllc(pg, pr, 0.0f, sol, a.status, a.step, f);
    if (!ok) return;
    // the reflected state carries the same density, pressure and normal speed
    // magnitude: the exact mass and energy fluxes through a wall at rest are 0
    sol.m = 0.0f;
    sol.en = 0.0f;
  } else {
    float fv = 0.0f;
    if (a.fvel) fv = fdot(F3{a.fvel[3 * f], a.fvel[3 * f + 1], a.fvel[3 * f + 2]}, n);
    const C3 ca = load32(a, fc.x), cb = load32(a, fc.y);
    if (!hllc(prim32(a.gamma, ca, n), prim32(a.gamma, cb, n), fv, sol, a.status, a.step, f)) return;
    par = parallel32(sol.m > 0.0f ? ca.v : cb.v, n);
  }
  const F3 mom{fmaf(sol.my, par.x, sol.mx * n.x), fmaf(sol.my, par.y, sol.mx * n.y), fmaf(sol.my, par.z, sol.mx * n.z)};
  const float s = kScaled ? (a.dt_from_device ? a.status->dt32 : a.dt32) * a.area32[f] : 1.0f;
  a.flux32[f] = make_float4(s * sol.m, s * mom.x, s * mom.y, s * mom.z);
  a.fen32[f] = s * sol.en;
}

__global__ void __launch_bounds__(kBlock) k3m_update(Mixed3Args a, int from_unscaled, int do_ext, int do_cells) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const Mesh3Dev& m = a.mesh;
  if (i >= m.n) return;
  double2* e2 = reinterpret_cast<double2*>(a.ext) + 3 * i;
  const double2 e01 = e2[0], e23 = e2[1], e45 = e2[2];
  double u[5] = {e01.x, e01.y, e23.x, e23.y, e45.x};
  if (do_ext) {
    float s[5] = {0, 0, 0, 0, 0}, c[5] = {0, 0, 0, 0, 0};
    const float dt = from_unscaled ? (a.dt_from_device ? a.status->dt32 : a.dt32) : 1.0f;
    for (int k = m.cell_off[i]; k < m.cell_off[i + 1]; ++k) {
      const int fs = a.fsign[k];
      const int f = fs & 0x7fffffff;
      const float4 v = a.flux32[f];
      float d[5] = {v.x, v.y, v.z, v.w, a.fen32[f]};
      const float sc = from_unscaled ? dt * a.area32[f] : 1.0f;
#pragma unroll
      for (int q = 0; q < 5; ++q) {
        // a separately rounded product (no contraction into the sum): the
        // fused step's pre-scaled fluxes give the same terms
        const float x = __fmul_rn(d[q], sc);
        two_sum(s[q], c[q], fs < 0 ? -x : x);
      }
    }
#pragma unroll
    for (int q = 0; q < 5; ++q) u[q] += widen(s[q]) + widen(c[q]);
    e2[0] = make_double2(u[0], u[1]);
    e2[1] = make_double2(u[2], u[3]);
    e2[2] = make_double2(u[4], 0.0);
  }
  if (do_cells) {
    const double V = m.volume[i];
    const float mf = narrow(u[0]);
    // 1/m from the FP32 reciprocal and one Newton step
    double r = widen(1.0f / mf);
    r = r * (2.0 - u[0] * r);
    const double vx = u[1] * r, vy = u[2] * r, vz = u[3] * r;
    const double eint = u[4] * r - 0.5 * (vx * vx + vy * vy + vz * vz);  // FP64: the cancellation
    if (eint < 0) {
      record_error(a.status, a.step, RG_ERR_NEGATIVE_ENERGY, 5, i, eint);
      return;
    }
    // m / V in FP32 from the rounded mass and volume (the result is stored in FP32)
    const float d = mf / narrow(V);
    a.cells32[i] = make_float4(d, (a.gamma - 1.0f) * narrow(eint) * d, narrow(vx), narrow(vy));
    a.vz32[i] = narrow(vz);
  }
}

__global__ void __launch_bounds__(kBlock) k3m_d2f(const double* a, float* b, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = narrow(a[i]);
}

inline int blocks(int n) { return n > 0 ? (n + kBlock - 1) / kBlock : 1; }

}  // namespace

cudaError_t launch3m_d2f(const double* a, float* b, int n, cudaStream_t s) {
  k3m_d2f<<<blocks(n), kBlock, 0, s>>>(a, b, n);
  return cudaGetLastError();
}

cudaError_t launch3m_geometry(const Mesh3Dev& m, const dbl4* nhat, float4* nhat32, float* area32, float* width32,
                              cudaStream_t s) {
  k3m_geometry<<<blocks(m.e > m.n ? m.e : m.n), kBlock, 0, s>>>(m, nhat, nhat32, area32, width32);
  return cudaGetLastError();
}
cudaError_t launch3m_cells_to32(const double* c64, float4* c32, float* vz32, int n, cudaStream_t s) {
  k3m_to32<<<blocks(n), kBlock, 0, s>>>(c64, c32, vz32, n);
  return cudaGetLastError();
}
cudaError_t launch3m_cells_to64(const float4* c32, const float* vz32, double* c64, int n, cudaStream_t s) {
  k3m_to64<<<blocks(n), kBlock, 0, s>>>(c32, vz32, c64, n);
  return cudaGetLastError();
}
cudaError_t launch3m_flux_to64(const float4* f32, const float* fen32, double* f64, int e, cudaStream_t s) {
  k3m_flux_to64<<<blocks(e), kBlock, 0, s>>>(f32, fen32, f64, e);
  return cudaGetLastError();
}
cudaError_t launch3m_cfl(const Mixed3Args& a, cudaStream_t s) {
  k3m_cfl<<<blocks(a.mesh.n), kBlock, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch3m_faces(const Mixed3Args& a, bool scaled, cudaStream_t s) {
  if (a.mesh.e == 0) return cudaSuccess;
  if (scaled)
    k3m_faces<true><<<blocks(a.mesh.e), kBlock, 0, s>>>(a);
  else
    k3m_faces<false><<<blocks(a.mesh.e), kBlock, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch3m_update(const Mixed3Args& a, bool from_unscaled, bool do_ext, bool do_cells, cudaStream_t s) {
  k3m_update<<<blocks(a.mesh.n), kBlock, 0, s>>>(a, from_unscaled ? 1 : 0, do_ext ? 1 : 0, do_cells ? 1 : 0);
  return cudaGetLastError();
}

}  // namespace rg
