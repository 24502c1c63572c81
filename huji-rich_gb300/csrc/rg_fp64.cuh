// rg_fp64.cuh -- device helpers shared by the plain-FP64 kernels
// (rg_fp64.cu) and the tracer kernels (rg_tracers.cu): cell records, ghost
// and point states, the FP32 screening of FP64 limiter quotients and one
// component of each LinearGaussImproved limiter.  Both units are compiled
// with --fmad=false.
#pragma once
#include <math.h>

#include "rg_div.cuh"
#include "rg_internal.cuh"

namespace rg {
namespace {

struct Cell { double d, p, vx, vy; };

__device__ __forceinline__ Cell load_cell(const double* cells, int i) {
  const double2 a = reinterpret_cast<const double2*>(cells)[2 * i];
  const double2 b = reinterpret_cast<const double2*>(cells)[2 * i + 1];
  return Cell{a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ void store4(double* out, int i, double a, double b, double c, double d) {
  reinterpret_cast<double2*>(out)[2 * i] = make_double2(a, b);
  reinterpret_cast<double2*>(out)[2 * i + 1] = make_double2(c, d);
}
// computational_cell_2d.cpp:59-68 ComputationalCellAddMult
__device__ __forceinline__ void addmult(Cell& r, const Cell& o, double s) {
  r.d += o.d * s;
  r.p += o.p * s;
  r.vx += o.vx * s;
  r.vy += o.vy * s;
}

// Per-problem parameters of a batch (kBatch) or the handle's single values.
template <bool kBatch>
__device__ __forceinline__ double gamma_at(const StepArgs& a, int point) {
  return kBatch ? a.gamma_p[a.cell_problem[point]] : a.gamma;
}
template <bool kBatch>
__device__ __forceinline__ double scaled_dt(const StepArgs& a, int point) {
  if (kBatch) return a.cfl * __longlong_as_double(static_cast<long long>(a.dtmin_p[a.cell_problem[point]]));
  return a.dt_from_device ? a.status->dt : a.dt_host;
}

// Ghost state (LinearGaussImproved.cpp:543-550 new_cells[ghost]):
// RigidWallGenerator.cpp:17-37 reflects the real neighbour's velocity,
// PeriodicGhostGenerator.cpp:3-17 copies the source cell.
__device__ __forceinline__ Cell ghost_state(const StepArgs& a, int g) {
  Cell c = load_cell(a.cells, a.geom.ghost_real[g]);
  if (a.ghost_kind != RG_GHOST_PERIODIC) {
    const double2 u = a.geom.ghost_unit[g];
    const double s = 2 * (c.vx * u.x + c.vy * u.y);
    c.vx -= u.x * s;
    c.vy -= u.y * s;
  }
  return c;
}
__device__ __forceinline__ void fill_ghost(const StepArgs& a, int g) {
  const Cell c = ghost_state(a, g);
  store4(a.cells, a.mesh.n + g, c.d, c.p, c.vx, c.vy);
}
// State of point p: a real cell's record, or a ghost's state formed from the
// current state of its cell (the per-step kernels read no ghost records)
__device__ __forceinline__ Cell point_state(const StepArgs& a, int p) {
  return p < a.mesh.n ? load_cell(a.cells, p) : ghost_state(a, p - a.mesh.n);
}
// dm0[e] or dm1[e] (centroid minus the first / second cell's CM), chosen by pointer
__device__ __forceinline__ double2 centroid_offset(const GeomDev& g, uint32_t w, int e) {
  return ((w & kNbrFirst) ? g.dm0 : g.dm1)[e];
}

// The cell whose tracers and stickers point p carries: p itself, or the
// cell a ghost copies (RigidWallGenerator.cpp:17-37 and
// PeriodicGhostGenerator.cpp:3-17 copy the whole ComputationalCell).
__device__ __forceinline__ int copied_cell(const StepArgs& a, int p) {
  return p < a.mesh.n ? p : a.geom.ghost_real[p - a.mesh.n];
}
// point p carries LinearGaussImproved's skip_key sticker (:192-193, :314-315, :339-340)
__device__ __forceinline__ bool skipped(const StepArgs& a, int p) {
  return a.skip_mask != 0 && (a.stickers[copied_cell(a, p)] & a.skip_mask) != 0;
}

__device__ __forceinline__ double step_dt(const StepArgs& a) {
  return a.dt_from_device ? a.status->dt : a.dt_host;
}

// LagrangianExtensiveUpdater.cpp:32-56 for cell i: dV, dV_ws over the cell's
// faces in face order, and the factor (V + dV) / (V + dV + dV_ws) that every
// extensive of the cell (its tracers included) is multiplied by
__device__ __forceinline__ double lag_factor(const StepArgs& a, int i) {
  const MeshDev& m = a.mesh;
  const double dtl = step_dt(a);
  double dv = 0.0, dvw = 0.0;
  for (int k = m.cell_off[i]; k < m.cell_off[i + 1]; ++k) {
    const int e = m.cell_faces[k];
    const double ar = a.geom.xarea[e];
    const double t1 = ar * dtl * a.lag_ev[e], t2 = ar * dtl * a.lag_ws[e];
    if (a.geom.nbr[k] & kNbrFirst) {
      dv += t1;
      dvw += t2;
    } else {
      dv -= t1;
      dvw -= t2;
    }
  }
  const double vol = m.cd_volume[i];
  return quot(vol + dv, vol + dv + dvw);
}

// FP32 screening of FP64 quotients.  GB300 issues 64 FP32 operations per FP64
// one, so a decision that only needs to know on which side of a threshold a
// correctly rounded FP64 quotient lies is taken from an FP32 estimate when
// the estimate is clear of the threshold by more than its error, and from the
// exact FP64 division otherwise.  For |a|,|b| in [2^-120, 2^120] the
// estimate float(a)/float(b) is within 4 * 2^-24 < 2.5e-7 (relative) of
// a/b; the margins below are 1e-6, with float(t) itself within 6e-8 of t.
// The range tests, the roundings to float and the limiter's |dphi| > thr and
// sign-of-product tests run on the integer pipe (rg_convert.cuh).
__device__ __forceinline__ bool fp32_safe(double a) { return abs_within(a, 1e-36, 1e36); }

// The limiter's running minimum psi is carried as its bit pattern (selections
// on the integer pipe) with psi_f = float(psi) beside it.
constexpr uint64_t kOneBits = 0x3ff0000000000000ull;  // 1.0

// psi_f = float(psi) is a usable screen when psi is 0 or a normal float.
__device__ __forceinline__ bool psi_screenable(uint64_t psi, float psi_f) {
  return psi_f >= 1e-30f || (psi & kMagMask) == 0u;
}

// smin(psi, num/den) for num/den >= 0 (or NaN, which smin ignores), psi >= 0:
// skips the division when the quotient is provably >= psi.
__device__ __forceinline__ void min_quotient(double num, double den, uint64_t& psi, float& psi_f) {
  if (fp32_safe(num) && fp32_safe(den) && psi_screenable(psi, psi_f)) {
    const float qf = narrow(num) / narrow(den);
    if (qf >= psi_f * 1.000001f) return;
  }
  const double q = quot(num, den);
  const uint64_t uq = conv_dbits(q);
  if (lt_u(uq, psi)) {
    psi = uq;
    psi_f = narrow(q);
  }
}

// one component of the ordinary limiter, LinearGaussImproved.cpp:232-267.
// thr = 0.05*max(|maxd|,|mind|) (per cell); maxd >= 0 >= mind, so both
// candidate quotients are >= 0.  The comparisons run on the integer pipe
// (rg_convert.cuh); the lower threshold -1e-9*q (or -|1e-9*q|) is exactly
// the negated upper one, the rounding being sign-symmetric.
__device__ __forceinline__ void limit_comp(double dphi, double cv, double cellv, double thr, double maxd,
                                           double mind, bool use_abs, uint64_t& psi, float& psi_f) {
  if (abs_gt(dphi, thr) || prod_neg(cv, cellv)) {
    const uint64_t t1 = use_abs ? abs_u(1e-9 * cellv) : conv_dbits(1e-9 * cellv);
    const uint64_t ud = conv_dbits(dphi);
    if (lt_u(t1, ud))
      min_quotient(maxd, dphi, psi, psi_f);
    else if (lt_u(ud, t1 ^ 0x8000000000000000ull))
      min_quotient(mind, dphi, psi, psi_f);
  }
}

// one component of the shocked limiter, LinearGaussImproved.cpp:343-366
// (threshold 1e-9*q without abs for every hydro component, as the reference
// has it; |1e-9*q| for tracers, :377): psi = smin(psi, smax(theta*(nb-cell)/dphi, 0)).
__device__ __forceinline__ void shocked_comp(double dphi, double cv, double cellv, double thr, double nbv,
                                             double theta, uint64_t& psi, float& psi_f, bool abs_thr = false) {
  if (abs_gt(dphi, thr) || prod_neg(cv, cellv)) {
    if (lt_u(abs_thr ? abs_u(1e-9 * cellv) : conv_dbits(1e-9 * cellv), abs_u(dphi))) {
      const double num = theta * (nbv - cellv);
      const uint64_t un = conv_dbits(num), ud = conv_dbits(dphi);
      // num != 0, neither NaN, (num < 0) != (dphi < 0)
      const bool num_neg = (un >> 63) != 0u, dphi_neg = (ud >> 63) != 0u && (ud & kMagMask) != 0u;
      if ((un & kMagMask) != 0u && !nan_bits(un) && !nan_bits(ud) && num_neg != dphi_neg) {
        // negative quotient: smax(., 0) gives 0
        if (lt_u(0u, psi)) {
          psi = 0u;
          psi_f = 0.0f;
        }
        return;
      }
      if (num != 0 && fp32_safe(num) && fp32_safe(dphi) && psi_screenable(psi, psi_f)) {
        const float qf = narrow(num) / narrow(dphi);
        if (qf >= psi_f * 1.000001f) return;
      }
      const double q = quot(num, dphi);
      const uint64_t ux = max_first_u(conv_dbits(q), 0u);
      if (lt_u(ux, psi)) {
        psi = ux;
        psi_f = narrow(conv_double_bits(ux));
      }
    }
  }
}

}  // namespace
}  // namespace rg
