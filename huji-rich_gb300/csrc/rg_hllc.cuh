// rg_hllc.cuh -- the Hllc Riemann solver (source/newtonian/common/hllc.cpp),
// templated on the real type: double for the plain path, shared by the 2D
// kernels (rg_fp64.cu) and the 3D first-order kernels (rg_3d.cu), both
// compiled with --fmad=false so every operation rounds as the reference's;
// float for the FP32-mixed 3D kernels (rg_3d_mixed.cu).  FP64 quotients are
// formed by rg::div_rn (rg_div.cuh: the same bits as the IEEE division).
#pragma once
#include "rg_div.cuh"
#include "rg_internal.cuh"

namespace rg {

template <class R>
struct PrimT {
  R d, p, vx, vy, e, c;
};
template <class R>
struct ConsT {
  R m, mx, my, en;
};
using Prim = PrimT<double>;
using Cons = ConsT<double>;

// hydrodynamic_variables.cpp:261-265 TotalEnergyDensity (pow(x,2) is x*x)
template <class R>
__device__ __forceinline__ R ted(const PrimT<R>& p) {
  const R s = root(p.vx * p.vx + p.vy * p.vy);
  return p.d * (R(0.5) * (s * s) + p.e);
}

// hllc.cpp:97-154 with massflux_ = true; the frame normal is (1,0), so
// Primitive2Flux's n/abs(n) is (1,0) exactly.  Only the branch's starred
// state is formed; the others do not reach the result.
template <class R>
__device__ __forceinline__ bool hllc(PrimT<R> l, PrimT<R> r, R velocity, ConsT<R>& f, DevStatus* status, int step,
                                     int face) {
  if (isnan(r.vx)) {
    record_error(status, step, RG_ERR_HLLC_NAN, 3, face, r.vx);
    return false;
  }
  // local.Velocity -= velocity*(1,0): the y part subtracts a zero, which can
  // only change the sign of a zero result, and is left out; so is the whole
  // boost for a face at rest (velocity +-0)
  const bool moving = velocity != R(0);
  if (moving) {
    l.vx -= velocity;
    r.vx -= velocity;
  }
  // :27-43 estimate_wave_speeds
  const R a1 = l.vx - l.c, b1 = r.vx - r.c, a2 = l.vx + l.c, b2 = r.vx + r.c;
  const R sl = b1 < a1 ? b1 : a1;  // std::min
  const R sr = a2 < b2 ? b2 : a2;  // std::max
  const R ss = quot(r.p - l.p + l.d * l.vx * (sl - l.vx) - r.d * r.vx * (sr - r.vx),
                    l.d * (sl - l.vx) - r.d * (sr - r.vx));
  const bool use_left = sl > R(0) || (sl <= R(0) && ss >= R(0));
  const bool use_right = !use_left && ((ss < R(0) && sr >= R(0)) || sr < R(0));
  if (!use_left && !use_right) {
    record_error(status, step, RG_ERR_HLLC_WAVE_SPEEDS, 3, face, ss);
    return false;
  }
  const PrimT<R>& q = use_left ? l : r;
  const R sk = use_left ? sl : sr;
  const R e_k = ted(q);
  // :281-290 Primitive2Flux along (1,0)
  // Primitive2Flux along n = (1,0): v.n = vx (the vy*0 term only changes the
  // sign of a zero), momentum (p + vx*d*vx, vy*d*vx)
  const R dsp = q.d * q.vx;
  ConsT<R> fk{dsp, q.p + q.vx * dsp, q.vy * dsp, (e_k + q.p) * q.vx};
  const bool star = use_left ? !(sl > R(0)) : !(sr < R(0));
  if (star) {
    // :76-92 starred_state, and fk + sk*(us - u) with u = Primitive2Conserved (:267-272)
    const R ds = quot(q.d * (sk - q.vx), sk - ss);
    const R usm = ds, usx = ds * ss, usy = ds * q.vy;
    const R use = quot(e_k * ds, q.d) + ds * (ss - q.vx) * (ss + quot(quot(q.p, q.d), sk - q.vx));
    fk.m = fk.m + sk * (usm - q.d);
    fk.mx = fk.mx + (usx - q.vx * q.d) * sk;
    fk.my = fk.my + (usy - q.vy * q.d) * sk;
    fk.en = fk.en + sk * (use - e_k);
  }
  // :150-152 back to the lab frame along the normal
  if (moving) {
    fk.en += fk.mx * velocity + R(0.5) * fk.m * velocity * velocity;
    fk.mx += velocity * fk.m;
  }
  f = fk;
  return true;
}

// LagrangianHLLC.cpp:85-175 (FP64): Hllc's flux for massflux = true, with
// `energy` the internal energy the flux carries across the face (:126-149);
// for massflux = false the same solve in the frame of the contact that
// estimate_wave_speeds gives for the boosted states (:108-115), `energy`
// that contact speed.  The (1,0)-frame terms that only change the sign of a
// zero are left out as in hllc(); ScalarProd(v, (1,0)) is formed in full.
__device__ __forceinline__ bool lagrangian_hllc(Prim l, Prim r, double velocity, bool massflux, Cons& f,
                                                double& energy, DevStatus* status, int step, int face) {
  if (isnan(r.vx)) {
    record_error(status, step, RG_ERR_HLLC_NAN, 3, face, r.vx);
    return false;
  }
  if (velocity != 0.0) {
    l.vx -= velocity;
    r.vx -= velocity;
  }
  double en = 0.0;
  if (!massflux) {
    const double a1 = l.vx - l.c, b1 = r.vx - r.c, a2 = l.vx + l.c, b2 = r.vx + r.c;
    const double sl2 = b1 < a1 ? b1 : a1, sr2 = a2 < b2 ? b2 : a2;
    const double ss2 = quot(r.p - l.p + l.d * l.vx * (sl2 - l.vx) - r.d * r.vx * (sr2 - r.vx),
                            l.d * (sl2 - l.vx) - r.d * (sr2 - r.vx));
    l.vx -= ss2;
    r.vx -= ss2;
    velocity += ss2;
    en = ss2;
  }
  const double a1 = l.vx - l.c, b1 = r.vx - r.c, a2 = l.vx + l.c, b2 = r.vx + r.c;
  const double sl = b1 < a1 ? b1 : a1;
  const double sr = a2 < b2 ? b2 : a2;
  const double ss = quot(r.p - l.p + l.d * l.vx * (sl - l.vx) - r.d * r.vx * (sr - r.vx),
                         l.d * (sl - l.vx) - r.d * (sr - r.vx));
  const bool use_left = sl > 0.0 || (sl <= 0.0 && ss >= 0.0);
  const bool use_right = !use_left && ((ss < 0.0 && sr >= 0.0) || sr < 0.0);
  if (!use_left && !use_right) {
    record_error(status, step, RG_ERR_HLLC_WAVE_SPEEDS, 3, face, ss);
    return false;
  }
  const Prim& q = use_left ? l : r;
  const double sk = use_left ? sl : sr;
  const double e_k = ted(q);
  const double dsp = q.d * q.vx;
  Cons fk{dsp, q.p + q.vx * dsp, q.vy * dsp, (e_k + q.p) * q.vx};
  const bool star = use_left ? !(sl > 0.0) : !(sr < 0.0);
  // ScalarProd(local.Velocity, (1,0))
  const double sp = q.vx * 1.0 + q.vy * 0.0;
  if (star) {
    const double ds = quot(q.d * (sk - q.vx), sk - ss);
    const double usm = ds, usx = ds * ss, usy = ds * q.vy;
    const double use = quot(e_k * ds, q.d) + ds * (ss - q.vx) * (ss + quot(quot(q.p, q.d), sk - q.vx));
    fk.m = fk.m + sk * (usm - q.d);
    fk.mx = fk.mx + (usx - q.vx * q.d) * sk;
    fk.my = fk.my + (usy - q.vy * q.d) * sk;
    fk.en = fk.en + sk * (use - e_k);
    if (massflux) {
      const double frac = quot(sk - q.vx, sk - ss) - 1.0;
      en = use_left ? sp * q.e * q.d + sk * q.e * frac * q.d : (sp * q.e + sk * q.e * frac) * q.d;
    }
  } else if (massflux) {
    en = sp * q.e * q.d;
  }
  if (velocity != 0.0) {
    fk.en += fk.mx * velocity + 0.5 * fk.m * velocity * velocity;
    fk.mx += velocity * fk.m;
  }
  f = fk;
  energy = en;
  return true;
}

}  // namespace rg
