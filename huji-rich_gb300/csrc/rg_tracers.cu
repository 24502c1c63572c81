// rg_tracers.cu -- tracer passes of the FP64 path (ComputationalCell::tracers,
// Extensive::tracers), compiled with --fmad=false like rg_fp64.cu.
//
// Every ComputationalCell / Extensive operation of the reference applies to
// each tracer exactly as to a hydro field (computational_cell_2d.cpp:20-110,
// extensive.cpp), with the same geometric scalars, so each tracer pass runs
// after its hydro pass and reads what that pass decided:
//   k_tr_slopes   per cell: LinearGaussImproved slope of every tracer
//                 (:67-134 / :401-422), zero outside calc_tracers (:470-479),
//                 the limiter chosen by the hydro shock test (:481-492)
//   k_tr_faces_*  per face: mass flux (kept by the hydro face kernel) times
//                 the upwind side's tracer (modular_flux_calculator.cpp:24-35,
//                 simple_flux_calculator.cpp:193-213)
//   k_tr_update   per cell: ascending-face gather of the tracer fluxes
//                 (simple_extensive_updater.cpp:11-35), then tracer =
//                 extensive / mass and the "Entropy" tracer
//                 (simple_cell_updater.cpp:22-59), or the old tracers of a
//                 SkipUpdate cell
// Tracers are cell-major (cell i's tracer j at i*nt + j).  The per-cell
// kernels are instantiated for each tracer count NT (1..kMaxTracers) so their
// loops over tracers have exact compile-time bounds: the per-cell arrays stay
// in registers and no FP64 work is spent on absent tracers.
#include <math.h>

#include "rg_fp64.cuh"

namespace rg {
namespace {

constexpr int kTrBlock = 256;

__device__ __forceinline__ const double* tracers_of(const StepArgs& a, const TracerArgs& t, int p) {
  return t.tr + static_cast<size_t>(copied_cell(a, p)) * t.nt;
}

// LinearGaussImproved.cpp:425-494 calc_slope, tracer part, for cell i.
template <int NT>
__global__ void __launch_bounds__(kTrBlock) k_tr_slopes(StepArgs a, TracerArgs t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const MeshDev& m = a.mesh;
  if (i >= m.n) return;
  constexpr int nt = NT;
  constexpr int kMaxTracers = NT;
  const int b = m.cell_off[i], nn = m.cell_off[i + 1] - b;
  const dbl4 mi = a.geom.minv[i];
  double ct[kMaxTracers], sx[kMaxTracers], sy[kMaxTracers];
#pragma unroll
  for (int j = 0; j < kMaxTracers; ++j) {
    ct[j] = j < nt ? t.tr[static_cast<size_t>(i) * nt + j] : 0.0;
    sx[j] = sy[j] = 0.0;
  }
  if (a.geom.cflags[i] & kCellBoundarySlope) {
    // :401-422 GetBoundarySlope: PhiS += (nb - cell)*(cm_nb - cm_cell)
    double py[kMaxTracers], px[kMaxTracers];
#pragma unroll
    for (int j = 0; j < kMaxTracers; ++j) py[j] = px[j] = 0.0;
    for (int k = 0; k < nn; ++k) {
      const double* nb = tracers_of(a, t, static_cast<int>(a.geom.nbr[b + k] & kNbrIdMask));
      const double2 h = a.geom.hr[b + k];
#pragma unroll
      for (int j = 0; j < kMaxTracers; ++j) {
        if (j < nt) {
          const double df = nb[j] - ct[j];
          py[j] = py[j] + df * h.y;
          px[j] = px[j] + df * h.x;
        }
      }
    }
    const double sxsy = mi.x, sx2 = mi.y, sy2 = mi.z, den = mi.w;
#pragma unroll
    for (int j = 0; j < kMaxTracers; ++j) {
      sx[j] = quot(py[j] * sxsy - px[j] * sy2, den);
      sy[j] = quot(px[j] * sxsy - py[j] * sx2, den);
    }
  } else {
    // :80-133 calc_naive_slope with the mesh's 0.5*r_ij and inverse matrix
    double vx[kMaxTracers], vy[kMaxTracers];
#pragma unroll
    for (int j = 0; j < kMaxTracers; ++j) vx[j] = vy[j] = 0.0;
    for (int k = 0; k < nn; ++k) {
      const double* nb = tracers_of(a, t, static_cast<int>(a.geom.nbr[b + k] & kNbrIdMask));
      const double2 h = a.geom.hr[b + k];
#pragma unroll
      for (int j = 0; j < kMaxTracers; ++j) {
        if (j < nt) {
          if (k == 0) {
            vx[j] = ct[j] * h.x;
            vy[j] = ct[j] * h.y;
          } else {
            vx[j] += ct[j] * h.x;
            vy[j] += ct[j] * h.y;
          }
          const double q = nb[j];
          vy[j] += q * h.y;
          vx[j] += q * h.x;
        }
      }
    }
#pragma unroll
    for (int j = 0; j < kMaxTracers; ++j) {
      sx[j] = vx[j] * mi.x;
      sy[j] = vy[j] * mi.w;
      sx[j] += vy[j] * mi.y;
      sy[j] += vx[j] * mi.z;
    }
  }
  // :470-479 tracers outside calc_tracers get zero slopes
#pragma unroll
  for (int j = 0; j < kMaxTracers; ++j)
    if (!((t.limited >> j) & 1u)) sx[j] = sy[j] = 0.0;
  if (a.slf) {
    const bool shock = a.shock[i] != 0;
    uint64_t cmax[kMaxTracers], cmin[kMaxTracers];  // bit patterns
#pragma unroll
    for (int j = 0; j < kMaxTracers; ++j) cmax[j] = cmin[j] = conv_dbits(ct[j]);
    for (int k = 0; k < nn; ++k) {
      const uint32_t w = a.geom.nbr[b + k];
      if (!shock && (w & kNbrMirror)) continue;  // :194-195
      if (skipped(a, static_cast<int>(w & kNbrIdMask))) continue;
      const double* nb = tracers_of(a, t, static_cast<int>(w & kNbrIdMask));
#pragma unroll
      for (int j = 0; j < kMaxTracers; ++j) {
        if (j < nt) {
          cmax[j] = max_first_u(cmax[j], conv_dbits(nb[j]));
          cmin[j] = min_first_u(cmin[j], conv_dbits(nb[j]));
        }
      }
    }
    const double f = shock ? 0.1 : 0.05;
    double maxd[kMaxTracers], mind[kMaxTracers], thr[kMaxTracers];
    uint64_t psi[kMaxTracers];
    float pf[kMaxTracers];
#pragma unroll
    for (int j = 0; j < kMaxTracers; ++j) {
      maxd[j] = conv_double_bits(cmax[j]) - ct[j];
      mind[j] = conv_double_bits(cmin[j]) - ct[j];
      thr[j] = f * conv_double_bits(max_first_u(abs_u(maxd[j]), abs_u(mind[j])));
      psi[j] = kOneBits;
      pf[j] = 1.0f;
    }
    for (int k = 0; k < nn; ++k) {
      const uint32_t w = a.geom.nbr[b + k];
      const int other = static_cast<int>(w & kNbrIdMask);
      if (shock && skipped(a, other)) continue;  // :339-340
      const int e = m.cell_faces[b + k];
      const double2 dm = centroid_offset(a.geom, w, e);
      const double* nb = tracers_of(a, t, other);
#pragma unroll
      for (int j = 0; j < kMaxTracers; ++j) {
        if (j < nt) {
          double cv = ct[j];
          cv += sx[j] * dm.x;
          cv += sy[j] * dm.y;
          const double dphi = cv - ct[j];
          if (!shock)
            limit_comp(dphi, cv, ct[j], thr[j], maxd[j], mind[j], true, psi[j], pf[j]);  // :268-283
          else
            shocked_comp(dphi, cv, ct[j], thr[j], nb[j], a.theta, psi[j], pf[j], true);  // :367-385
        }
      }
    }
#pragma unroll
    for (int j = 0; j < kMaxTracers; ++j) {
      sx[j] *= conv_double_bits(psi[j]);
      sy[j] *= conv_double_bits(psi[j]);
    }
  }
  double* o = t.tr_slopes + static_cast<size_t>(i) * 2 * nt;
#pragma unroll
  for (int j = 0; j < kMaxTracers; ++j) {
    if (j < nt) {
      o[j] = sx[j];
      o[nt + j] = sy[j];
    }
  }
}

// dt*area of face e (simple_extensive_updater.cpp:26-27); in a batch the dt
// of the problem of the face's real side, as the hydro face kernel scales it
__device__ __forceinline__ double tr_scale(const StepArgs& a, int e) {
  if (a.cell_problem) {
    const int2 fc = a.mesh.face_cells[e];
    return scaled_dt<true>(a, fc.x < a.mesh.n ? fc.x : fc.y) * a.geom.xarea[e];
  }
  return scaled_dt<false>(a, 0) * a.geom.xarea[e];
}

// ModularFluxCalculator tracer fluxes: Mass * (Mass > 0 ? first : second)
// side's LinearGaussImproved value (:570-590 real sides; :596-634 ghost sides:
// the copied cell's tracers plus the periodic source's gradient, or a zero
// gradient at rigid walls, RigidWallGenerator.cpp:39-54).
template <bool kScaled>
__global__ void __launch_bounds__(kTrBlock) k_tr_faces_lgi(StepArgs a, TracerArgs t) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const MeshDev& m = a.mesh;
  if (e >= m.e) return;
  const int nt = t.nt;
  const int2 fc = m.face_cells[e];
  const double mass = a.mflux[e];
  const bool first = mass > 0;
  const int pid = first ? fc.x : fc.y;
  const double2 dm = first ? a.geom.dm0[e] : a.geom.dm1[e];
  const int src = copied_cell(a, pid);
  const bool zero_grad = pid >= m.n && a.ghost_kind != RG_GHOST_PERIODIC;
  const double* q = t.tr + static_cast<size_t>(src) * nt;
  const double* g = t.tr_slopes + static_cast<size_t>(src) * 2 * nt;
  const double s = kScaled ? tr_scale(a, e) : 1.0;
  double* o = t.tr_flux + static_cast<size_t>(e) * nt;
  for (int j = 0; j < nt; ++j) {
    double v = q[j];
    v += (zero_grad ? 0.0 : g[j]) * dm.x;
    v += (zero_grad ? 0.0 : g[nt + j]) * dm.y;
    const double f = mass * v;
    o[j] = kScaled ? f * s : f;
  }
}

// The condition/action fluxes' tracer part: Mass times the tracers of the
// side the face's action chose (a.tr_side): that neighbour's own cell (a
// ghost's cell, as the hydro state), or its LinearGaussImproved face value as
// k_tr_faces_lgi forms it.  Faces with no action carry none.
template <bool kScaled>
__global__ void __launch_bounds__(kTrBlock) k_tr_faces_cas(StepArgs a, TracerArgs t) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const MeshDev& m = a.mesh;
  if (e >= m.e) return;
  const int nt = t.nt;
  const unsigned char side = a.tr_side[e];
  double* o = t.tr_flux + static_cast<size_t>(e) * nt;
  if (!(side & (kTrSideFirst | kTrSideSecond))) {
    for (int j = 0; j < nt; ++j) o[j] = 0.0;
    return;
  }
  const int2 fc = m.face_cells[e];
  const double mass = a.mflux[e];
  const bool first = (side & kTrSideFirst) != 0;
  const int pid = first ? fc.x : fc.y;
  const double s = kScaled ? tr_scale(a, e) : 1.0;
  if (side & kTrSideFace) {
    const double2 dm = (first ? a.geom.dm0 : a.geom.dm1)[e];
    const int src = copied_cell(a, pid);
    const bool zero_grad = pid >= m.n && a.ghost_kind != RG_GHOST_PERIODIC;
    const double* q = t.tr + static_cast<size_t>(src) * nt;
    const double* g = t.tr_slopes + static_cast<size_t>(src) * 2 * nt;
    for (int j = 0; j < nt; ++j) {
      double v = q[j];
      v += (zero_grad ? 0.0 : g[j]) * dm.x;
      v += (zero_grad ? 0.0 : g[nt + j]) * dm.y;
      const double f = mass * v;
      o[j] = kScaled ? f * s : f;
    }
  } else {
    const double* q = t.tr + static_cast<size_t>(orig_of(m, pid)) * nt;
    for (int j = 0; j < nt; ++j) {
      const double f = mass * q[j];
      o[j] = kScaled ? f * s : f;
    }
  }
}

// SimpleFluxCalculator calc_tracer_flux (simple_flux_calculator.cpp:193-213):
// Mass * the upwind point's tracer, 0 when that point is a self-mirror ghost
// or Mass is 0; a periodic ghost reads its source cell, as the hydro state does.
template <bool kScaled>
__global__ void __launch_bounds__(kTrBlock) k_tr_faces_pcm(StepArgs a, TracerArgs t) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const MeshDev& m = a.mesh;
  if (e >= m.e) return;
  const int nt = t.nt;
  const int2 fc = m.face_cells[e];
  const double mass = a.mflux[e];
  const bool mirror = orig_of(m, fc.x) == orig_of(m, fc.y);
  int up = -1;
  if (mass > 0 && (fc.x < m.n || !mirror))
    up = fc.x;
  else if (mass < 0 && (fc.y < m.n || !mirror))
    up = fc.y;
  const double s = kScaled ? tr_scale(a, e) : 1.0;
  double* o = t.tr_flux + static_cast<size_t>(e) * nt;
  for (int j = 0; j < nt; ++j) {
    const double f = up >= 0 ? mass * t.tr[static_cast<size_t>(orig_of(m, up)) * nt + j] : 0.0;
    o[j] = kScaled ? f * s : f;
  }
}

// SimpleExtensiveUpdater for the extensive tracers (gather in ascending face
// order) and SimpleCellUpdater's tracer part; runs after the hydro update,
// whose new mass, density and pressure it reads.
template <int NT>
__global__ void __launch_bounds__(kTrBlock) k_tr_update(StepArgs a, TracerArgs t, int from_unscaled, int do_ext,
                                                         int do_cells) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const MeshDev& m = a.mesh;
  if (i >= m.n) return;
  constexpr int nt = NT;
  constexpr int kMaxTracers = NT;
  double te[kMaxTracers];
  double* ext_t = t.tr_ext + static_cast<size_t>(i) * nt;
#pragma unroll
  for (int j = 0; j < kMaxTracers; ++j) te[j] = j < nt ? ext_t[j] : 0.0;
  if (do_ext) {
    const double dt = from_unscaled ? step_dt(a) : 0.0;
    for (int k = m.cell_off[i]; k < m.cell_off[i + 1]; ++k) {
      const int e = m.cell_faces[k];
      const bool minus = (a.geom.nbr[k] & kNbrFirst) != 0;
      const double s = from_unscaled ? dt * a.geom.xarea[e] : 1.0;
      const double* f = t.tr_flux + static_cast<size_t>(e) * nt;
#pragma unroll
      for (int j = 0; j < kMaxTracers; ++j) {
        if (j < nt) {
          const double d = from_unscaled ? f[j] * s : f[j];
          if (minus)
            te[j] -= d;
          else
            te[j] += d;
        }
      }
    }
    if (a.lag_update) {
      // LagrangianExtensiveUpdater scales every extensive of the cell
      const double f = lag_factor(a, i);
#pragma unroll
      for (int j = 0; j < kMaxTracers; ++j)
        if (j < nt) te[j] *= f;
    }
  }
  if (t.tr_ext_avg) {
    // hdsim2d.cpp:311-320 average_extensive: 0.5*(mid + old)
    const double* o = t.tr_ext_avg + static_cast<size_t>(i) * nt;
#pragma unroll
    for (int j = 0; j < kMaxTracers; ++j)
      if (j < nt) te[j] = 0.5 * (te[j] + o[j]);
  }
  const bool frozen = a.frozen_mask && (a.stickers[i] & a.frozen_mask);
  if (do_cells && frozen && t.tr_out) {
    // SkipUpdate keeps the step's old cell, its tracers included
#pragma unroll
    for (int j = 0; j < kMaxTracers; ++j)
      if (j < nt) t.tr_out[static_cast<size_t>(i) * nt + j] = t.tr[static_cast<size_t>(i) * nt + j];
  }
  if (do_cells && !frozen) {
    const double mass = (a.ext_out ? a.ext_out : a.ext)[4 * i];
    double* tr = (t.tr_out ? t.tr_out : t.tr) + static_cast<size_t>(i) * nt;
#pragma unroll
    for (int j = 0; j < kMaxTracers; ++j)
      if (j < nt) tr[j] = quot(te[j], mass);
    if (t.entropy >= 0) {
      // ideal_gas.cpp:52-55 dp2s of the updated cell
      const Cell c = load_cell(a.cells_out ? a.cells_out : a.cells, i);
      const double sv = c.p * pow(c.d, -(a.cell_problem ? a.gamma_p[a.cell_problem[i]] : a.gamma));
      tr[t.entropy] = sv;
#pragma unroll
      for (int j = 0; j < kMaxTracers; ++j)
        if (j == t.entropy) te[j] = sv * mass;
    }
  }
  if (do_ext || (do_cells && t.entropy >= 0) || t.tr_ext_out) {
    double* out = t.tr_ext_out ? t.tr_ext_out + static_cast<size_t>(i) * nt : ext_t;
#pragma unroll
    for (int j = 0; j < kMaxTracers; ++j)
      if (j < nt) out[j] = te[j];
  }
}

// hdsim2d.cpp:56-63 init_extensives: tracer * mass, mass = volume * density
__global__ void __launch_bounds__(kTrBlock) k_tr_init(StepArgs a, TracerArgs t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.mesh.n) return;
  const double mass = a.mesh.cd_volume[i] * load_cell(a.cells, i).d;
  for (int j = 0; j < t.nt; ++j)
    t.tr_ext[static_cast<size_t>(i) * t.nt + j] = t.tr[static_cast<size_t>(i) * t.nt + j] * mass;
}

inline int tr_blocks(int n) { return (n + kTrBlock - 1) / kTrBlock; }

}  // namespace

// kernel K instantiated for NT = t.nt
#define RG_TR_DISPATCH(K, grid, s, ...)                                  \
  switch (t.nt) {                                                         \
    case 1: K<1><<<grid, kTrBlock, 0, s>>>(__VA_ARGS__); break;           \
    case 2: K<2><<<grid, kTrBlock, 0, s>>>(__VA_ARGS__); break;           \
    case 3: K<3><<<grid, kTrBlock, 0, s>>>(__VA_ARGS__); break;           \
    case 4: K<4><<<grid, kTrBlock, 0, s>>>(__VA_ARGS__); break;           \
    case 5: K<5><<<grid, kTrBlock, 0, s>>>(__VA_ARGS__); break;           \
    case 6: K<6><<<grid, kTrBlock, 0, s>>>(__VA_ARGS__); break;           \
    case 7: K<7><<<grid, kTrBlock, 0, s>>>(__VA_ARGS__); break;           \
    case 8: K<8><<<grid, kTrBlock, 0, s>>>(__VA_ARGS__); break;           \
    default: break;                                                       \
  }

cudaError_t launch_tr_slopes(const StepArgs& a, const TracerArgs& t, cudaStream_t s) {
  if (a.mesh.n > 0 && t.nt > 0 && t.nt <= kMaxTracers) {
    RG_TR_DISPATCH(k_tr_slopes, tr_blocks(a.mesh.n), s, a, t)
  }
  return cudaGetLastError();
}

cudaError_t launch_tr_faces(const StepArgs& a, const TracerArgs& t, cudaStream_t s, bool scaled) {
  if (a.mesh.e == 0 || t.nt == 0) return cudaSuccess;
  const int nb = tr_blocks(a.mesh.e);
  if (a.n_rules > 0)
    scaled ? k_tr_faces_cas<true><<<nb, kTrBlock, 0, s>>>(a, t) : k_tr_faces_cas<false><<<nb, kTrBlock, 0, s>>>(a, t);
  else if (a.order == 1)
    scaled ? k_tr_faces_pcm<true><<<nb, kTrBlock, 0, s>>>(a, t) : k_tr_faces_pcm<false><<<nb, kTrBlock, 0, s>>>(a, t);
  else
    scaled ? k_tr_faces_lgi<true><<<nb, kTrBlock, 0, s>>>(a, t) : k_tr_faces_lgi<false><<<nb, kTrBlock, 0, s>>>(a, t);
  return cudaGetLastError();
}

cudaError_t launch_tr_update(const StepArgs& a, const TracerArgs& t, cudaStream_t s, bool from_unscaled,
                             bool extensive, bool cells) {
  if (a.mesh.n > 0 && t.nt > 0 && t.nt <= kMaxTracers) {
    const int fu = from_unscaled ? 1 : 0, ex = extensive ? 1 : 0, ce = cells ? 1 : 0;
    RG_TR_DISPATCH(k_tr_update, tr_blocks(a.mesh.n), s, a, t, fu, ex, ce)
  }
  return cudaGetLastError();
}

cudaError_t launch_tr_init(const StepArgs& a, const TracerArgs& t, cudaStream_t s) {
  if (a.mesh.n > 0 && t.nt > 0) k_tr_init<<<tr_blocks(a.mesh.n), kTrBlock, 0, s>>>(a, t);
  return cudaGetLastError();
}

}  // namespace rg
