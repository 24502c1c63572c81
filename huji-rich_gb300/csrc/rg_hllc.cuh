// rg_hllc.cuh -- the FP64 Hllc Riemann solver of the plain path, shared by
// the 2D kernels (rg_fp64.cu) and the 3D first-order kernels (rg_3d.cu);
// both reference paths call the same Hllc (source/newtonian/common/hllc.cpp).
// Compile with --fmad=false: every operation rounds as the reference's.
#pragma once
#include "rg_internal.cuh"

namespace rg {

struct Prim { double d, p, vx, vy, e, c; };
struct Cons { double m, mx, my, en; };

// hydrodynamic_variables.cpp:261-265 TotalEnergyDensity (pow(x,2) is x*x)
__device__ __forceinline__ double ted(const Prim& p) {
  const double s = sqrt(p.vx * p.vx + p.vy * p.vy);
  return p.d * (0.5 * (s * s) + p.e);
}

// hllc.cpp:97-154 with massflux_ = true; the frame normal is (1,0), so
// Primitive2Flux's n/abs(n) is (1,0) exactly.  Only the branch's starred
// state is formed; the others do not reach the result.
__device__ __forceinline__ bool hllc(Prim l, Prim r, double velocity, Cons& f, DevStatus* status, int step,
                                     int face) {
  if (isnan(r.vx)) {
    record_error(status, step, RG_ERR_HLLC_NAN, 3, face, r.vx);
    return false;
  }
  // local.Velocity -= velocity*(1,0): the y part subtracts a zero, which can
  // only change the sign of a zero result, and is left out; so is the whole
  // boost for a face at rest (velocity +-0)
  const bool moving = velocity != 0.0;
  if (moving) {
    l.vx -= velocity;
    r.vx -= velocity;
  }
  // :27-43 estimate_wave_speeds
  const double sl = smin(l.vx - l.c, r.vx - r.c);
  const double sr = smax(l.vx + l.c, r.vx + r.c);
  const double ss = (r.p - l.p + l.d * l.vx * (sl - l.vx) - r.d * r.vx * (sr - r.vx)) /
                    (l.d * (sl - l.vx) - r.d * (sr - r.vx));
  const bool use_left = sl > 0 || (sl <= 0 && ss >= 0);
  const bool use_right = !use_left && ((ss < 0 && sr >= 0) || sr < 0);
  if (!use_left && !use_right) {
    record_error(status, step, RG_ERR_HLLC_WAVE_SPEEDS, 3, face, ss);
    return false;
  }
  const Prim& q = use_left ? l : r;
  const double sk = use_left ? sl : sr;
  const double e_k = ted(q);
  // :281-290 Primitive2Flux along (1,0)
  // Primitive2Flux along n = (1,0): v.n = vx (the vy*0 term only changes the
  // sign of a zero), momentum (p + vx*d*vx, vy*d*vx)
  const double dsp = q.d * q.vx;
  Cons fk{dsp, q.p + q.vx * dsp, q.vy * dsp, (e_k + q.p) * q.vx};
  const bool star = use_left ? !(sl > 0) : !(sr < 0);
  if (star) {
    // :76-92 starred_state, and fk + sk*(us - u) with u = Primitive2Conserved (:267-272)
    const double ds = q.d * (sk - q.vx) / (sk - ss);
    const double usm = ds, usx = ds * ss, usy = ds * q.vy;
    const double use = e_k * ds / q.d + ds * (ss - q.vx) * (ss + q.p / q.d / (sk - q.vx));
    fk.m = fk.m + sk * (usm - q.d);
    fk.mx = fk.mx + (usx - q.vx * q.d) * sk;
    fk.my = fk.my + (usy - q.vy * q.d) * sk;
    fk.en = fk.en + sk * (use - e_k);
  }
  // :150-152 back to the lab frame along the normal
  if (moving) {
    fk.en += fk.mx * velocity + 0.5 * fk.m * velocity * velocity;
    fk.mx += velocity * fk.m;
  }
  f = fk;
  return true;
}

}  // namespace rg
