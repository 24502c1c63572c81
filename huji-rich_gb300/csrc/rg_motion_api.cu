// rg_motion_api.cu -- C ABI of device-side point motion and geometry
// (include/rich_gb300.h, "Point motion on the device"): hdsim::TimeAdvance's
// first half (hdsim2d.cpp:149-195) enqueued on the handle's stream, the
// kernels in rg_motion.cu.  Point motion reads FP64 cell records; on the
// FP32-mixed path they are widened from the FP32 primitives first, and the
// face velocities are written straight into their FP32 copy (the FP64 ones
// are formed when read back).
#include <cuda_runtime.h>

#include "rg_handle.cuh"
#include "rg_mixed.cuh"
#include "rg_motion.cuh"

using namespace rgh;

namespace {

rg::MotionArgs motion_args(rg_handle* h) {
  rg::MotionArgs mo{};
  mo.kind = h->motion.kind;
  mo.edges = h->motion.edges;
  mo.cold = h->motion.cold;
  mo.fix = h->motion.correct_overshoot;
  mo.chi = h->motion.chi;
  mo.eta = h->motion.eta;
  mo.box = rg::make_dbl4(h->box[0], h->box[1], h->box[2], h->box[3]);
  mo.pv = static_cast<double2*>(h->pv.p);
  mo.ev = static_cast<double2*>(h->ev.p);
  return mo;
}

// FP64 cell records for the motion kernels
rg_status widen_cells(rg_handle* h) {
  if (h->mixed)
    RG_CUDA(h, rg::launch_cells_to64(static_cast<const float4*>(h->cells32.p), static_cast<double*>(h->cells.p),
                                     active_slot(h)->n, h->stream));
  return RG_OK;
}

// face velocities from the point velocities, as the handle's edge velocities
// (an FP32-mixed handle: the FP32 copy; the FP64 one on read-back)
rg_status edges_from_points(rg_handle* h, const rg::StepArgs& a, const rg::MotionArgs& mo) {
  MeshSlot* s = active_slot(h);
  h->ev64_pending = false;
  if (h->motion.kind == RG_MOTION_EULERIAN) {
    // every face velocity is +0 (CalcFaceVelocity of zero velocities): the
    // kernels read none
    RG_CUDA(h, cudaMemsetAsync(h->ev.p, 0, 16 * static_cast<size_t>(s->e), h->stream));
    if (h->mixed) RG_CUDA(h, cudaMemsetAsync(h->ev32.p, 0, 8 * static_cast<size_t>(s->e), h->stream));
    h->ev_zero = true;
  } else if (h->mixed) {
    RG_CUDA(h, rg::launch_edge_velocities32(a, mo, static_cast<float2*>(h->ev32.p), h->stream));
    h->ev64_pending = true;
    h->ev_zero = false;
  } else {
    RG_CUDA(h, rg::launch_edge_velocities(a, mo, h->stream));
    h->ev_zero = false;
  }
  h->have_ev = true;
  h->dt_next_ready = false;
  return RG_OK;
}

rg_status download_pv(rg_handle* h, double* out) {
  if (!out) return RG_OK;
  RG_CUDA(h, cudaMemcpyAsync(out, h->pv.p, 16 * static_cast<size_t>(active_slot(h)->n), cudaMemcpyDeviceToHost,
                             h->stream));
  return RG_OK;
}

rg_status motion_ready(rg_handle* h) {
  if (rg_status st = require(h, true, false, false, false)) return st;
  if (h->external_state) return invalid(h, -1, 0);
  RG_CUDA(h, h->pv.ensure(16 * static_cast<size_t>(active_slot(h)->n)));
  return RG_OK;
}

}  // namespace

extern "C" {

rg_status rg_set_outer_box(rg_handle* h, double left, double right, double down, double up) {
  if (!h) return RG_ERR_INVALID_ARGUMENT;
  if (!(left < right) || !(down < up)) return invalid(h, 0, right - left);
  h->box[0] = left;
  h->box[1] = right;
  h->box[2] = down;
  h->box[3] = up;
  h->have_box = true;
  return RG_OK;
}

rg_status rg_set_point_motion(rg_handle* h, const rg_point_motion* pm) {
  if (!h || !pm) return RG_ERR_INVALID_ARGUMENT;
  if (pm->kind < RG_MOTION_EULERIAN || pm->kind > RG_MOTION_ROUND_CELLS) return invalid(h, 0, pm->kind);
  if (pm->edges != RG_EDGES_STATIONARY_BOX && pm->edges != RG_EDGES_PERIODIC) return invalid(h, 1, pm->edges);
  if (pm->kind == RG_MOTION_ROUND_CELLS && pm->correct_overshoot && !h->have_box) return invalid(h, 2, 0);
  h->motion = *pm;
  return RG_OK;
}

rg_status rg_point_velocities(rg_handle* h, double* pv_out) {
  if (rg_status st = motion_ready(h)) return st;
  h->last = rg_error{};
  RG_TRY(widen_cells(h));
  const rg::StepArgs a = step_args(h);
  const rg::MotionArgs mo = motion_args(h);
  RG_CUDA(h, rg::launch_point_velocities(a, mo, h->stream));
  RG_TRY(edges_from_points(h, a, mo));
  RG_TRY(download_pv(h, pv_out));
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  return RG_OK;
}

rg_status rg_apply_fix(rg_handle* h, double dt, double* pv_out) {
  if (rg_status st = motion_ready(h)) return st;
  h->last = rg_error{};
  RG_TRY(widen_cells(h));
  rg::StepArgs a = step_args(h);
  a.dt_host = dt;
  const rg::MotionArgs mo = motion_args(h);
  RG_CUDA(h, rg::launch_apply_fix(a, mo, h->stream));
  RG_TRY(edges_from_points(h, a, mo));
  RG_TRY(download_pv(h, pv_out));
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  return RG_OK;
}

rg_status rg_get_edge_velocities(rg_handle* h, double* ev) {
  if (rg_status st = require(h, false, false, true, false)) return st;
  if (!ev) return RG_ERR_INVALID_ARGUMENT;
  if (h->ev64_pending) {
    // the FP64 face velocities of the last device motion (FP32-mixed)
    RG_CUDA(h, rg::launch_edge_velocities(step_args(h), motion_args(h), h->stream));
    h->ev64_pending = false;
  }
  RG_CUDA(h, cudaMemcpyAsync(ev, h->ev.p, 16 * static_cast<size_t>(active_slot(h)->e), cudaMemcpyDeviceToHost,
                             h->stream));
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  return RG_OK;
}

rg_status rg_set_physical_geometry(rg_handle* h, const rg_physical_geometry* pg) {
  if (!h || !pg) return RG_ERR_INVALID_ARGUMENT;
  if (pg->kind != RG_GEOMETRY_SLAB && pg->kind != RG_GEOMETRY_CYLINDRICAL) return invalid(h, 0, pg->kind);
  if (pg->kind == RG_GEOMETRY_CYLINDRICAL && !(pg->direction[0] != 0 || pg->direction[1] != 0))
    return invalid(h, 1, 0);
  h->pgeo = *pg;
  return RG_OK;
}

rg_status rg_get_geometry(rg_handle* h, double* volume, double* cm_xy, double* cd_volume, double* cd_area) {
  if (rg_status st = require(h, false, false, false, false)) return st;
  if (cd_area) RG_TRY(ensure_geom64(h));
  MeshSlot* s = active_slot(h);
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  const size_t n = static_cast<size_t>(s->n), np = n + static_cast<size_t>(s->g);
  if (cd_area) RG_CUDA(h, cudaMemcpy(cd_area, s->geom.xarea, 8 * static_cast<size_t>(s->e), cudaMemcpyDeviceToHost));
  if (volume) RG_CUDA(h, cudaMemcpy(volume, s->mesh.volume, 8 * n, cudaMemcpyDeviceToHost));
  if (cm_xy) RG_CUDA(h, cudaMemcpy(cm_xy, s->mesh.cms, 16 * np, cudaMemcpyDeviceToHost));
  if (cd_volume) RG_CUDA(h, cudaMemcpy(cd_volume, s->mesh.cd_volume, 8 * n, cudaMemcpyDeviceToHost));
  return RG_OK;
}

rg_status rg_advance_begin(rg_handle* h, double* dt_out, double* pv_out) {
  if (rg_status st = motion_ready(h)) return st;
  if (rg_status st = require(h, true, true, false, false)) return st;
  if (rg_status st = require_tracers(h, true)) return st;
  if (rg_status st = mesh_error(h)) return st;
  if (h->n_problems > 0 || h->heun) return invalid(h, -2, 0);
  h->last = rg_error{};
  RG_TRY(reset_status(h, h->d_status, h->stream));
  RG_TRY(widen_cells(h));
  const rg::MotionArgs mo = motion_args(h);
  {
    // PointMotion::operator(), EdgeVelocityCalculator, SimpleCFL
    const rg::StepArgs a0 = step_args(h);
    RG_CUDA(h, rg::launch_point_velocities(a0, mo, h->stream));
    RG_TRY(edges_from_points(h, a0, mo));
  }
  const bool o2 = h->cfg.order == 2;
  if (h->mixed) {
    RG_CUDA(h, rg::launch_cfl32(mixed_args(h), h->stream, false));
  } else {
    rg::StepArgs ac = step_args(h);
    RG_CUDA(h, rg::launch_cfl(ac, h->stream, false));
  }
  if (h->motion.kind == RG_MOTION_ROUND_CELLS && (h->motion.cold || h->motion.correct_overshoot)) {
    // ApplyFix with the device dt, face velocities again (the other motions'
    // ApplyFix leaves the velocities, point_motion.cpp:5-9)
    rg::StepArgs a1 = step_args(h);
    a1.dt_from_device = 1;
    RG_CUDA(h, rg::launch_apply_fix(a1, mo, h->stream));
    RG_TRY(edges_from_points(h, a1, mo));
  }
  // fluxes (dt*area scaled) and the extensive update
  if (h->mixed) {
    rg::MixedArgs m = mixed_args(h);
    m.dt32_from_device = 1;
    const bool tr = h->tcfg.n_tracers > 0;
    rg::StepArgs a64 = step_args(h);
    a64.dt_from_device = 1;
    const rg::TracerArgs ta = tracer_args(h);
    if (o2) {
      RG_CUDA(h, rg::launch_ghost_fill32(m, h->stream));
      RG_CUDA(h, rg::launch_slopes32(m, h->stream));
      if (tr) RG_CUDA(h, rg::launch_tr_slopes(a64, ta, h->stream));
    }
    RG_CUDA(h, rg::launch_faces32(m, h->stream, true));
    if (tr) RG_CUDA(h, rg::launch_tr_faces(a64, ta, h->stream, true));
    RG_CUDA(h, rg::launch_update_mixed(m, h->stream, false, true, false));
    if (tr) RG_CUDA(h, rg::launch_tr_update(a64, ta, h->stream, false, true, false));
  } else {
    rg::StepArgs a = step_args(h);
    a.dt_from_device = 1;
    const bool tr = h->tcfg.n_tracers > 0;
    const rg::TracerArgs ta = tracer_args(h);
    if (o2) {
      RG_CUDA(h, rg::launch_ghost_fill(a, h->stream));
      RG_CUDA(h, rg::launch_slopes(a, h->stream));
      if (tr) RG_CUDA(h, rg::launch_tr_slopes(a, ta, h->stream));
    }
    RG_CUDA(h, rg::launch_faces(a, h->stream, true));
    if (tr) RG_CUDA(h, rg::launch_tr_faces(a, ta, h->stream, true));
    RG_CUDA(h, rg::launch_update(a, h->stream, false, true, false));
    if (tr) RG_CUDA(h, rg::launch_tr_update(a, ta, h->stream, false, true, false));
  }
  RG_TRY(download_pv(h, pv_out));
  h->have_fluxes = false;
  h->dt_next_ready = false;
  const rg_status st = collect(h, h->d_status, h->stream);
  if (dt_out) *dt_out = h->last_dt;
  return st;
}

}  // extern "C"
