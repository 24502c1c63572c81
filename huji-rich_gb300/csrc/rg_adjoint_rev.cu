// rg_adjoint_rev.cu -- hand-written reverse sweep of one differentiated step
// (FP64; rg_adjoint_rev32.cu builds the face and cell kernels again in FP32
// for the FP32-mixed adjoint).  With Ubar_{k+1} = dL/dU_{k+1} given, one reverse step is
//     Wbar_k = G'(W_k)^T Ubar_{k+1}
//     Ubar_k = Ubar_{k+1} + C'(U_k)^T Wbar_k      (k > 0)
//     dL/dW_0 = Wbar_0 + I'(W_0)^T Ubar_1          (k = 0)
// and G'^T runs as three kernels, each a gather with no atomics:
//   k_adj_faces  per face: the flux adjoint dt*area*(Ubar[second] -
//                Ubar[first]) (the transposed SimpleExtensiveUpdater
//                gather) through the rotation back, HLLC (the primal's wave
//                speed and region branches) and the rotation into the face
//                frame, to the adjoints of the face's two reconstructed states
//   k_adj_cell   per cell: gathers the adjoints of the face states built
//                from it (its own sides and those of the periodic ghosts it
//                is the source of) into its state and slope adjoints, then
//                reverses the limiter (the active candidate in the trace:
//                psi = numerator/dphi, a subgradient at switches) and the
//                Green-Gauss slope; the shares of its neighbours are written
//                per CSR entry
//   k_adj_update gathers the CSR-entry shares addressed to the cell (the
//                reverse adjacency, ascending), adds its own share and
//                applies C'^T (or I'^T for the first step)
// The branches are re-evaluated from the stored forward state; this file
// lets the compiler contract multiply-adds, so a re-evaluation can differ
// from the forward only at an exact tie, where either side is a valid
// one-sided derivative.
#include <math.h>

#include "rg_adjoint.cuh"
#include "rg_div.cuh"

#ifndef RG_ADJ_REAL
#define RG_ADJ_REAL double
#define RG_ADJ_FP64 1
#endif

namespace rg {
namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ void load_raw(const double* c, int i, double o[4]) {
  const double2 a = reinterpret_cast<const double2*>(c)[2 * i];
  const double2 b = reinterpret_cast<const double2*>(c)[2 * i + 1];
  o[0] = a.x;
  o[1] = a.y;
  o[2] = b.x;
  o[3] = b.y;
}
__device__ __forceinline__ void store_raw(double* c, int i, const double v[4]) {
  reinterpret_cast<double2*>(c)[2 * i] = make_double2(v[0], v[1]);
  reinterpret_cast<double2*>(c)[2 * i + 1] = make_double2(v[2], v[3]);
}
__device__ __forceinline__ int source_of(const MeshDev& m, int p) { return p < m.n ? p : m.ghost_source[p - m.n]; }

// Working precision of the face and cell reverse kernels: double here;
// rg_adjoint_rev32.cu compiles them again with float (the FP32-mixed
// adjoint), loading and storing the same FP64 arrays.
using real = RG_ADJ_REAL;
struct rv2 {
  real x, y;
};
__device__ __forceinline__ rv2 r2(double2 v) { return rv2{static_cast<real>(v.x), static_cast<real>(v.y)}; }
__device__ __forceinline__ void load_r(const double* c, int i, real o[4]) {
  double t[4];
  load_raw(c, i, t);
#pragma unroll
  for (int q = 0; q < 4; ++q) o[q] = static_cast<real>(t[q]);
}
__device__ __forceinline__ void store_r(double* c, int i, const real v[4]) {
  const double t[4] = {v[0], v[1], v[2], v[3]};
  store_raw(c, i, t);
}

#if RG_ADJ_FP64
// Periodic meshes only: every ghost has a source, no CSR entry is a
// self-mirror and no cell uses the boundary slope.
__global__ void __launch_bounds__(kBlock) k_adj_check(AdjArgs a) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < a.mesh.m && (a.geom.nbr[t] & kNbrMirror)) record_error(a.status, 0, RG_ERR_INVALID_ARGUMENT, 0, t, 0.0);
  if (t < a.mesh.n && (a.geom.cflags[t] & kCellBoundarySlope))
    record_error(a.status, 0, RG_ERR_INVALID_ARGUMENT, 1, t, 0.0);
}

// C'(U)^T w for SimpleCellUpdater (d = m/V, v = P/m, e = E/m - |v|^2/2,
// p = (gamma-1) e d), added to ub.
__device__ __forceinline__ void cell_update_transpose(double gamma, double V, const double u[4], const double w[4],
                                                      double ub[4]) {
  const double mass = u[0], en = u[1];
  const double d = quot(mass, V), vx = quot(u[2], mass), vy = quot(u[3], mass);
  const double e = quot(en, mass) - 0.5 * (vx * vx + vy * vy);
  const double be = w[1] * (gamma - 1) * d;
  const double bd = w[0] + w[1] * (gamma - 1) * e;
  const double bvx = w[2] - be * vx, bvy = w[3] - be * vy;
  ub[0] += quot(bd, V) - quot(quot(be * en, mass) + bvx * vx + bvy * vy, mass);
  ub[1] += quot(be, mass);
  ub[2] += quot(bvx, mass);
  ub[3] += quot(bvy, mass);
}

__global__ void __launch_bounds__(kBlock) k_adj_seed(AdjArgs a, const double* wbar, double* ubar) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.mesh.n) return;
  double u[4], w[4], ub[4] = {0, 0, 0, 0};
  load_raw(a.ext, i, u);
  load_raw(wbar, i, w);
  cell_update_transpose(a.gamma, a.mesh.cd_volume[i], u, w, ub);
  store_raw(ubar, i, ub);
}

#endif  // RG_ADJ_FP64

// Reverse of primitive conversion, rotation into the face frame, Hllc
// (hllc.cpp:97-154, massflux, face at rest) and the rotation back: from fb
// (adjoint of {mass, energy, px, py}) to the adjoints of the two states.
__device__ void hllc_reverse(real g, rv2 n, real na, rv2 p, real pa, const real L[4], const real R[4],
                             const real fb[4], real lb[4], real rb[4]) {
  // forward values
  const real dL = L[0], pL = L[1], dR = R[0], pR = R[1];
  const real eL = quot(quot(pL, dL), g - real(1)), cL = root(quot(g * pL, dL));
  const real eR = quot(quot(pR, dR), g - real(1)), cR = root(quot(g * pR, dR));
  const real lu = quot(L[2] * n.x + L[3] * n.y, na), lv = quot(L[2] * p.x + L[3] * p.y, pa);
  const real ru = quot(R[2] * n.x + R[3] * n.y, na), rv = quot(R[2] * p.x + R[3] * p.y, pa);
  const bool sl_right = (ru - cR) < (lu - cL);
  const real sl = sl_right ? ru - cR : lu - cL;
  const bool sr_right = (lu + cL) < (ru + cR);
  const real sr = sr_right ? ru + cR : lu + cL;
  const real num = pR - pL + dL * lu * (sl - lu) - dR * ru * (sr - ru);
  const real den = dL * (sl - lu) - dR * (sr - ru);
  const real ss = quot(num, den);
  const bool left = sl > 0 || (sl <= 0 && ss >= 0);
  const bool star = left ? !(sl > 0) : !(sr < 0);
  const real qd = left ? dL : dR, qp = left ? pL : pR, qe = left ? eL : eR;
  const real qu = left ? lu : ru, qv = left ? lv : rv, sk = left ? sl : sr;
  const real k2 = qu * qu + qv * qv;
  const real ek = qd * (real(0.5) * k2 + qe);
  // adjoint of the face-frame flux {fm, fmx, fmy, fen}
  const real bfm = fb[0], bfen = fb[1];
  const real bfmx = quot(n.x * fb[2] + n.y * fb[3], na);
  const real bfmy = quot(p.x * fb[2] + p.y * fb[3], pa);
  real bd = 0, bp = 0, bu = 0, bv = 0, be = 0, bek = 0, bsk = 0, bss = 0;
  if (star) {
    // ds = qd K/D, use = ek ds/qd + ds A B with K = sk - qu, D = sk - ss,
    // A = ss - qu, B = ss + Q, Q = qp/(qd K); fluxes gain sk*(u* - u)
    const real K = sk - qu, D = sk - ss;
    const real ds = quot(qd * K, D);
    const real Q = quot(quot(qp, qd), K);
    const real A = ss - qu, B = ss + Q;
    const real use = quot(ek * ds, qd) + ds * A * B;
    bsk += bfm * (ds - qd) + bfmx * (ds * ss - qu * qd) + bfmy * (ds * qv - qv * qd) + bfen * (use - ek);
    real bds = (bfm + bfmx * ss + bfmy * qv) * sk;
    bd -= (bfm + bfmx * qu + bfmy * qv) * sk;
    bu -= bfmx * qd * sk;
    bv += bfmy * (ds - qd) * sk;
    bss += bfmx * ds * sk;
    const real buse = bfen * sk;
    bek -= bfen * sk;
    bek += quot(buse * ds, qd);
    bds += buse * (quot(ek, qd) + A * B);
    bd -= quot(buse * ek * ds, qd * qd);
    const real bA = buse * ds * B, bB = buse * ds * A;
    bss += bA + bB;
    bu -= bA;
    bp += quot(bB, qd * K);
    bd -= quot(bB * Q, qd);
    real bK = quot(-bB * Q, K);
    bd += quot(bds * K, D);
    bK += quot(bds * qd, D);
    const real bD = quot(-bds * ds, D);
    bsk += bK + bD;
    bu -= bK;
    bss -= bD;
  }
  // physical flux along the normal: fm = qd qu, fmx = qp + qu qd qu,
  // fmy = qv qd qu, fen = (ek + qp) qu; ek = qd (|v|^2/2 + qe)
  bd += bfm * qu + bfmx * qu * qu + bfmy * qv * qu;
  bu += bfm * qd + real(2.0) * bfmx * qd * qu + bfmy * qv * qd + bfen * (ek + qp);
  bv += bfmy * qd * qu;
  bp += bfmx + bfen * qu;
  bek += bfen * qu;
  bd += bek * (real(0.5) * k2 + qe);
  bu += bek * qd * qu;
  bv += bek * qd * qv;
  be += bek * qd;
  // distribute to the chosen side, then the wave-speed paths
  real bdL = 0, bpL = 0, buL = 0, bvL = 0, beL = 0, bcL = 0;
  real bdR = 0, bpR = 0, buR = 0, bvR = 0, beR = 0, bcR = 0;
  real bsl = 0, bsr = 0;
  if (left) {
    bdL = bd, bpL = bp, buL = bu, bvL = bv, beL = be, bsl = bsk;
  } else {
    bdR = bd, bpR = bp, buR = bu, bvR = bv, beR = be, bsr = bsk;
  }
  // ss = num/den
  const real bnum = quot(bss, den), bden = quot(-bss * ss, den);
  bpR += bnum;
  bpL -= bnum;
  bdL += bnum * lu * (sl - lu) + bden * (sl - lu);
  buL += bnum * dL * (sl - real(2.0) * lu) - bden * dL;
  bsl += (bnum * lu + bden) * dL;
  bdR -= bnum * ru * (sr - ru) + bden * (sr - ru);
  buR -= bnum * dR * (sr - real(2.0) * ru) - bden * dR;
  bsr -= (bnum * ru + bden) * dR;
  // sl = min(lu - cL, ru - cR), sr = max(lu + cL, ru + cR)
  if (sl_right) {
    buR += bsl;
    bcR -= bsl;
  } else {
    buL += bsl;
    bcL -= bsl;
  }
  if (sr_right) {
    buR += bsr;
    bcR += bsr;
  } else {
    buL += bsr;
    bcL += bsr;
  }
  // e = p/(d (gamma-1)), c = sqrt(gamma p/d)
  bpL += quot(beL, dL * (g - real(1))) + quot(bcL * g, real(2.0) * cL * dL);
  bdL -= quot(beL * eL, dL) + quot(bcL * cL, real(2.0) * dL);
  bpR += quot(beR, dR * (g - real(1))) + quot(bcR * g, real(2.0) * cR * dR);
  bdR -= quot(beR * eR, dR) + quot(bcR * cR, real(2.0) * dR);
  // rotation into the face frame: u = v.n/|n|, v_t = v.par/|par|
  lb[0] = bdL;
  lb[1] = bpL;
  lb[2] = quot(buL * n.x, na) + quot(bvL * p.x, pa);
  lb[3] = quot(buL * n.y, na) + quot(bvL * p.y, pa);
  rb[0] = bdR;
  rb[1] = bpR;
  rb[2] = quot(buR * n.x, na) + quot(bvR * p.x, pa);
  rb[3] = quot(buR * n.y, na) + quot(bvR * p.y, pa);
}

__device__ __forceinline__ void face_state(const AdjArgs& a, int pid, rv2 dm, real c[4]) {
  const int sid = source_of(a.mesh, pid);
  real gx[4], gy[4];
  load_r(a.cells, sid, c);
  load_r(a.slopes, 2 * sid, gx);
  load_r(a.slopes, 2 * sid + 1, gy);
#pragma unroll
  for (int q = 0; q < 4; ++q) c[q] = c[q] + gx[q] * dm.x + gy[q] * dm.y;
}

__global__ void __launch_bounds__(kBlock) k_adj_faces(AdjArgs a, const double* ubar) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const MeshDev& m = a.mesh;
  if (e >= m.e) return;
  const int2 fc = m.face_cells[e];
  // the transposed gather of the extensive update stays in FP64
  const double s = a.dt * a.geom.area[e];
  double fbd[4] = {0, 0, 0, 0};
  if (fc.y < m.n) {
    double u[4];
    load_raw(ubar, fc.y, u);
#pragma unroll
    for (int q = 0; q < 4; ++q) fbd[q] += u[q];
  }
  if (fc.x < m.n) {
    double u[4];
    load_raw(ubar, fc.x, u);
#pragma unroll
    for (int q = 0; q < 4; ++q) fbd[q] -= u[q];
  }
  real fb[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) fb[q] = static_cast<real>(fbd[q] * s);
  real L[4], R[4], lb[4], rb[4];
  face_state(a, fc.x, r2(a.geom.dm0[e]), L);
  face_state(a, fc.y, r2(a.geom.dm1[e]), R);
  hllc_reverse(static_cast<real>(a.gamma), r2(a.geom.nrm[e]), static_cast<real>(a.geom.nabs[e]), r2(a.geom.par[e]),
               static_cast<real>(a.geom.area[e]), L, R, fb, lb, rb);
  store_r(a.side_bar, 2 * e, lb);
  store_r(a.side_bar, 2 * e + 1, rb);
}

__global__ void __launch_bounds__(kBlock) k_adj_cell(AdjArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const MeshDev& m = a.mesh;
  if (i >= m.n) return;
  // face-state adjoints -> state adjoint w and slope adjoints bx, by
  real w[4] = {0, 0, 0, 0}, bx[4] = {0, 0, 0, 0}, by[4] = {0, 0, 0, 0};
  for (int k = a.side_off[i]; k < a.side_off[i + 1]; ++k) {
    const int s = a.sides[k];
    const int e = s >> 1;
    const rv2 dm = r2((s & 1) ? a.geom.dm1[e] : a.geom.dm0[e]);
    real sb[4];
    load_r(a.side_bar, s, sb);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      w[q] += sb[q];
      bx[q] += sb[q] * dm.x;
      by[q] += sb[q] * dm.y;
    }
  }
  // limiter: s = naive*psi
  const SlopeTrace& tr = a.trace[i];
  const int b = m.cell_off[i], nn = m.cell_off[i + 1] - b;
  real bnx[4], bny[4], extra[4];
  int ex_at[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int code = tr.code[q];
    const int k = code & 0xff;
    bnx[q] = bx[q];
    bny[q] = by[q];
    extra[q] = 0;
    ex_at[q] = -1;
    if (k == kTraceNone) continue;
    const int kind = (code >> 8) & 3;
    const real psi = static_cast<real>(tr.psi[q]);
    bnx[q] = bx[q] * psi;
    bny[q] = by[q] * psi;
    if (kind == 3) continue;  // clamped to zero: no dependence
    // psi = N/D with D = naive_x dm.x + naive_y dm.y (the centroid difference)
    // and N = coef*(W[neighbour] - W[cell])
    const real nx = static_cast<real>(tr.naive[q]), ny = static_cast<real>(tr.naive[4 + q]);
    const real bpsi = bx[q] * nx + by[q] * ny;
    const real D = static_cast<real>(tr.dphi[q]);
    const real bN = quot(bpsi, D), bD = quot(-bpsi * psi, D);
    const int e = m.cell_faces[b + k];
    const rv2 dm = r2((a.geom.nbr[b + k] & kNbrFirst) ? a.geom.dm0[e] : a.geom.dm1[e]);
    bnx[q] += bD * dm.x;
    bny[q] += bD * dm.y;
    const int ex = (code >> 16) - 1;
    if (ex >= 0) {
      extra[q] = (kind == 2 ? static_cast<real>(a.theta) : real(1)) * bN;
      ex_at[q] = ex;
      w[q] -= extra[q];
    }
  }
  // naive slope: nx = vx*mi.x + vy*mi.y, ny = vx*mi.z + vy*mi.w,
  // v = sum_k h_k (W[cell] + W[neighbour k])
  const dbl4 mid = a.geom.minv[i];
  const real mix = static_cast<real>(mid.x), miy = static_cast<real>(mid.y), miz = static_cast<real>(mid.z),
             miw = static_cast<real>(mid.w);
  real bvx[4], bvy[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    bvx[q] = bnx[q] * mix + bny[q] * miz;
    bvy[q] = bnx[q] * miy + bny[q] * miw;
  }
  for (int k = 0; k < nn; ++k) {
    const rv2 h = r2(a.geom.hr[b + k]);
    real c[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      c[q] = bvx[q] * h.x + bvy[q] * h.y;
      w[q] += c[q];
      if (ex_at[q] == k) c[q] += extra[q];
    }
    store_r(a.entry_bar, b + k, c);
  }
  store_r(a.self_bar, i, w);
}

#if RG_ADJ_FP64
__global__ void __launch_bounds__(kBlock) k_adj_update(AdjArgs a, const double* ubar_in, double* ubar_out,
                                                       double* grad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const MeshDev& m = a.mesh;
  if (i >= m.n) return;
  double w[4];
  load_raw(a.self_bar, i, w);
  for (int k = a.target_off[i]; k < a.target_off[i + 1]; ++k) {
    double c[4];
    load_raw(a.entry_bar, a.targets[k], c);
#pragma unroll
    for (int q = 0; q < 4; ++q) w[q] += c[q];
  }
  double ub[4];
  load_raw(ubar_in, i, ub);
  const double V = m.cd_volume[i];
  if (grad) {
    // U_0 = I(W_0): mass = V d, E = V p/(gamma-1) + V d |v|^2/2, P = mass v
    double c[4];
    load_raw(a.cells, i, c);
    const double k2 = c[2] * c[2] + c[3] * c[3];
    const double mass = V * c[0];
    double g[4];
    g[0] = w[0] + V * (ub[0] + 0.5 * k2 * ub[1] + c[2] * ub[2] + c[3] * ub[3]);
    g[1] = w[1] + quot(V, a.gamma - 1) * ub[1];
    g[2] = w[2] + mass * (c[2] * ub[1] + ub[2]);
    g[3] = w[3] + mass * (c[3] * ub[1] + ub[3]);
    store_raw(grad, i, g);
    return;
  }
  double u[4];
  load_raw(a.ext, i, u);
  cell_update_transpose(a.gamma, V, u, w, ub);
  store_raw(ubar_out, i, ub);
}

#endif  // RG_ADJ_FP64

inline int blocks(int n) { return (n + kBlock - 1) / kBlock; }

}  // namespace

#if RG_ADJ_FP64
cudaError_t adj_launch_check(const AdjArgs& a, cudaStream_t s) {
  const int n = a.mesh.m > a.mesh.n ? a.mesh.m : a.mesh.n;
  k_adj_check<<<blocks(n), kBlock, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t adj_launch_seed(const AdjArgs& a, const double* wbar, double* ubar, cudaStream_t s) {
  k_adj_seed<<<blocks(a.mesh.n), kBlock, 0, s>>>(a, wbar, ubar);
  return cudaGetLastError();
}

cudaError_t adj_launch_update(const AdjArgs& a, const double* ubar_in, double* ubar_out, double* grad,
                              cudaStream_t s) {
  k_adj_update<<<blocks(a.mesh.n), kBlock, 0, s>>>(a, ubar_in, ubar_out, grad);
  return cudaGetLastError();
}

cudaError_t adj_launch_reverse(const AdjArgs& a, const double* ubar_in, double* ubar_out, double* grad,
                               cudaStream_t s) {
  k_adj_faces<<<blocks(a.mesh.e), kBlock, 0, s>>>(a, ubar_in);
  k_adj_cell<<<blocks(a.mesh.n), kBlock, 0, s>>>(a);
  return adj_launch_update(a, ubar_in, ubar_out, grad, s);
}
#else
cudaError_t adj_launch_reverse32(const AdjArgs& a, const double* ubar_in, double* ubar_out, double* grad,
                                 cudaStream_t s) {
  k_adj_faces<<<blocks(a.mesh.e), kBlock, 0, s>>>(a, ubar_in);
  k_adj_cell<<<blocks(a.mesh.n), kBlock, 0, s>>>(a);
  return adj_launch_update(a, ubar_in, ubar_out, grad, s);
}
#endif

}  // namespace rg
