// rg_adjoint_rev.cu -- hand-written reverse sweep of one differentiated step
// (FP64).  With Ubar_{k+1} = dL/dU_{k+1} given, one reverse step is
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
  const double d = mass / V, vx = u[2] / mass, vy = u[3] / mass;
  const double e = en / mass - 0.5 * (vx * vx + vy * vy);
  const double be = w[1] * (gamma - 1) * d;
  const double bd = w[0] + w[1] * (gamma - 1) * e;
  const double bvx = w[2] - be * vx, bvy = w[3] - be * vy;
  ub[0] += bd / V - (be * en / mass + bvx * vx + bvy * vy) / mass;
  ub[1] += be / mass;
  ub[2] += bvx / mass;
  ub[3] += bvy / mass;
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

// Reverse of primitive conversion, rotation into the face frame, Hllc
// (hllc.cpp:97-154, massflux, face at rest) and the rotation back: from fb
// (adjoint of {mass, energy, px, py}) to the adjoints of the two states.
__device__ void hllc_reverse(double g, double2 n, double na, double2 p, double pa, const double L[4],
                             const double R[4], const double fb[4], double lb[4], double rb[4]) {
  // forward values
  const double dL = L[0], pL = L[1], dR = R[0], pR = R[1];
  const double eL = pL / dL / (g - 1), cL = sqrt(g * pL / dL);
  const double eR = pR / dR / (g - 1), cR = sqrt(g * pR / dR);
  const double lu = (L[2] * n.x + L[3] * n.y) / na, lv = (L[2] * p.x + L[3] * p.y) / pa;
  const double ru = (R[2] * n.x + R[3] * n.y) / na, rv = (R[2] * p.x + R[3] * p.y) / pa;
  const bool sl_right = (ru - cR) < (lu - cL);
  const double sl = sl_right ? ru - cR : lu - cL;
  const bool sr_right = (lu + cL) < (ru + cR);
  const double sr = sr_right ? ru + cR : lu + cL;
  const double num = pR - pL + dL * lu * (sl - lu) - dR * ru * (sr - ru);
  const double den = dL * (sl - lu) - dR * (sr - ru);
  const double ss = num / den;
  const bool left = sl > 0 || (sl <= 0 && ss >= 0);
  const bool star = left ? !(sl > 0) : !(sr < 0);
  const double qd = left ? dL : dR, qp = left ? pL : pR, qe = left ? eL : eR;
  const double qu = left ? lu : ru, qv = left ? lv : rv, sk = left ? sl : sr;
  const double k2 = qu * qu + qv * qv;
  const double ek = qd * (0.5 * k2 + qe);
  // adjoint of the face-frame flux {fm, fmx, fmy, fen}
  const double bfm = fb[0], bfen = fb[1];
  const double bfmx = (n.x * fb[2] + n.y * fb[3]) / na;
  const double bfmy = (p.x * fb[2] + p.y * fb[3]) / pa;
  double bd = 0, bp = 0, bu = 0, bv = 0, be = 0, bek = 0, bsk = 0, bss = 0;
  if (star) {
    // ds = qd K/D, use = ek ds/qd + ds A B with K = sk - qu, D = sk - ss,
    // A = ss - qu, B = ss + Q, Q = qp/(qd K); fluxes gain sk*(u* - u)
    const double K = sk - qu, D = sk - ss;
    const double ds = qd * K / D;
    const double Q = qp / qd / K;
    const double A = ss - qu, B = ss + Q;
    const double use = ek * ds / qd + ds * A * B;
    bsk += bfm * (ds - qd) + bfmx * (ds * ss - qu * qd) + bfmy * (ds * qv - qv * qd) + bfen * (use - ek);
    double bds = (bfm + bfmx * ss + bfmy * qv) * sk;
    bd -= (bfm + bfmx * qu + bfmy * qv) * sk;
    bu -= bfmx * qd * sk;
    bv += bfmy * (ds - qd) * sk;
    bss += bfmx * ds * sk;
    const double buse = bfen * sk;
    bek -= bfen * sk;
    bek += buse * ds / qd;
    bds += buse * (ek / qd + A * B);
    bd -= buse * ek * ds / (qd * qd);
    const double bA = buse * ds * B, bB = buse * ds * A;
    bss += bA + bB;
    bu -= bA;
    bp += bB / (qd * K);
    bd -= bB * Q / qd;
    double bK = -bB * Q / K;
    bd += bds * K / D;
    bK += bds * qd / D;
    const double bD = -bds * ds / D;
    bsk += bK + bD;
    bu -= bK;
    bss -= bD;
  }
  // physical flux along the normal: fm = qd qu, fmx = qp + qu qd qu,
  // fmy = qv qd qu, fen = (ek + qp) qu; ek = qd (|v|^2/2 + qe)
  bd += bfm * qu + bfmx * qu * qu + bfmy * qv * qu;
  bu += bfm * qd + 2.0 * bfmx * qd * qu + bfmy * qv * qd + bfen * (ek + qp);
  bv += bfmy * qd * qu;
  bp += bfmx + bfen * qu;
  bek += bfen * qu;
  bd += bek * (0.5 * k2 + qe);
  bu += bek * qd * qu;
  bv += bek * qd * qv;
  be += bek * qd;
  // distribute to the chosen side, then the wave-speed paths
  double bdL = 0, bpL = 0, buL = 0, bvL = 0, beL = 0, bcL = 0;
  double bdR = 0, bpR = 0, buR = 0, bvR = 0, beR = 0, bcR = 0;
  double bsl = 0, bsr = 0;
  if (left) {
    bdL = bd, bpL = bp, buL = bu, bvL = bv, beL = be, bsl = bsk;
  } else {
    bdR = bd, bpR = bp, buR = bu, bvR = bv, beR = be, bsr = bsk;
  }
  // ss = num/den
  const double bnum = bss / den, bden = -bss * ss / den;
  bpR += bnum;
  bpL -= bnum;
  bdL += bnum * lu * (sl - lu) + bden * (sl - lu);
  buL += bnum * dL * (sl - 2.0 * lu) - bden * dL;
  bsl += (bnum * lu + bden) * dL;
  bdR -= bnum * ru * (sr - ru) + bden * (sr - ru);
  buR -= bnum * dR * (sr - 2.0 * ru) - bden * dR;
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
  bpL += beL / (dL * (g - 1)) + bcL * g / (2.0 * cL * dL);
  bdL -= beL * eL / dL + bcL * cL / (2.0 * dL);
  bpR += beR / (dR * (g - 1)) + bcR * g / (2.0 * cR * dR);
  bdR -= beR * eR / dR + bcR * cR / (2.0 * dR);
  // rotation into the face frame: u = v.n/|n|, v_t = v.par/|par|
  lb[0] = bdL;
  lb[1] = bpL;
  lb[2] = buL * n.x / na + bvL * p.x / pa;
  lb[3] = buL * n.y / na + bvL * p.y / pa;
  rb[0] = bdR;
  rb[1] = bpR;
  rb[2] = buR * n.x / na + bvR * p.x / pa;
  rb[3] = buR * n.y / na + bvR * p.y / pa;
}

__device__ __forceinline__ void face_state(const AdjArgs& a, int pid, double2 dm, double c[4]) {
  const int sid = source_of(a.mesh, pid);
  double gx[4], gy[4];
  load_raw(a.cells, sid, c);
  load_raw(a.slopes, 2 * sid, gx);
  load_raw(a.slopes, 2 * sid + 1, gy);
#pragma unroll
  for (int q = 0; q < 4; ++q) c[q] = c[q] + gx[q] * dm.x + gy[q] * dm.y;
}

__global__ void __launch_bounds__(kBlock) k_adj_faces(AdjArgs a, const double* ubar) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const MeshDev& m = a.mesh;
  if (e >= m.e) return;
  const int2 fc = m.face_cells[e];
  const double s = a.dt * a.geom.area[e];
  double fb[4] = {0, 0, 0, 0};
  if (fc.y < m.n) {
    double u[4];
    load_raw(ubar, fc.y, u);
#pragma unroll
    for (int q = 0; q < 4; ++q) fb[q] += u[q];
  }
  if (fc.x < m.n) {
    double u[4];
    load_raw(ubar, fc.x, u);
#pragma unroll
    for (int q = 0; q < 4; ++q) fb[q] -= u[q];
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) fb[q] *= s;
  double L[4], R[4], lb[4], rb[4];
  face_state(a, fc.x, a.geom.dm0[e], L);
  face_state(a, fc.y, a.geom.dm1[e], R);
  hllc_reverse(a.gamma, a.geom.nrm[e], a.geom.nabs[e], a.geom.par[e], a.geom.area[e], L, R, fb, lb, rb);
  store_raw(a.side_bar, 2 * e, lb);
  store_raw(a.side_bar, 2 * e + 1, rb);
}

__global__ void __launch_bounds__(kBlock) k_adj_cell(AdjArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const MeshDev& m = a.mesh;
  if (i >= m.n) return;
  // face-state adjoints -> state adjoint w and slope adjoints bx, by
  double w[4] = {0, 0, 0, 0}, bx[4] = {0, 0, 0, 0}, by[4] = {0, 0, 0, 0};
  for (int k = a.side_off[i]; k < a.side_off[i + 1]; ++k) {
    const int s = a.sides[k];
    const int e = s >> 1;
    const double2 dm = (s & 1) ? a.geom.dm1[e] : a.geom.dm0[e];
    double sb[4];
    load_raw(a.side_bar, s, sb);
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
  double bnx[4], bny[4], extra[4];
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
    const double psi = tr.psi[q];
    bnx[q] = bx[q] * psi;
    bny[q] = by[q] * psi;
    if (kind == 3) continue;  // clamped to zero: no dependence
    // psi = N/D with D = naive_x dm.x + naive_y dm.y (the centroid difference)
    // and N = coef*(W[neighbour] - W[cell])
    const double nx = tr.naive[q], ny = tr.naive[4 + q];
    const double bpsi = bx[q] * nx + by[q] * ny;
    const double D = tr.dphi[q];
    const double bN = bpsi / D, bD = -bpsi * psi / D;
    const int e = m.cell_faces[b + k];
    const double2 dm = (a.geom.nbr[b + k] & kNbrFirst) ? a.geom.dm0[e] : a.geom.dm1[e];
    bnx[q] += bD * dm.x;
    bny[q] += bD * dm.y;
    const int ex = (code >> 16) - 1;
    if (ex >= 0) {
      extra[q] = (kind == 2 ? a.theta : 1.0) * bN;
      ex_at[q] = ex;
      w[q] -= extra[q];
    }
  }
  // naive slope: nx = vx*mi.x + vy*mi.y, ny = vx*mi.z + vy*mi.w,
  // v = sum_k h_k (W[cell] + W[neighbour k])
  const dbl4 mi = a.geom.minv[i];
  double bvx[4], bvy[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    bvx[q] = bnx[q] * mi.x + bny[q] * mi.z;
    bvy[q] = bnx[q] * mi.y + bny[q] * mi.w;
  }
  for (int k = 0; k < nn; ++k) {
    const double2 h = a.geom.hr[b + k];
    double c[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      c[q] = bvx[q] * h.x + bvy[q] * h.y;
      w[q] += c[q];
      if (ex_at[q] == k) c[q] += extra[q];
    }
    store_raw(a.entry_bar, b + k, c);
  }
  store_raw(a.self_bar, i, w);
}

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
    g[1] = w[1] + V / (a.gamma - 1) * ub[1];
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

inline int blocks(int n) { return (n + kBlock - 1) / kBlock; }

}  // namespace

cudaError_t adj_launch_check(const AdjArgs& a, cudaStream_t s) {
  const int n = a.mesh.m > a.mesh.n ? a.mesh.m : a.mesh.n;
  k_adj_check<<<blocks(n), kBlock, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t adj_launch_seed(const AdjArgs& a, const double* wbar, double* ubar, cudaStream_t s) {
  k_adj_seed<<<blocks(a.mesh.n), kBlock, 0, s>>>(a, wbar, ubar);
  return cudaGetLastError();
}

cudaError_t adj_launch_reverse(const AdjArgs& a, const double* ubar_in, double* ubar_out, double* grad,
                               cudaStream_t s) {
  k_adj_faces<<<blocks(a.mesh.e), kBlock, 0, s>>>(a, ubar_in);
  k_adj_cell<<<blocks(a.mesh.n), kBlock, 0, s>>>(a);
  k_adj_update<<<blocks(a.mesh.n), kBlock, 0, s>>>(a, ubar_in, ubar_out, grad);
  return cudaGetLastError();
}

}  // namespace rg
