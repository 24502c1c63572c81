// rg_capi.cu -- the C ABI (include/rich_gb300.h): handle, mesh upload,
// state transfer and the plugin operations, on top of the kernels in
// rg_fp64.cu.
//
// Streams: every kernel of a handle runs on its compute stream.  Meshes are
// double-buffered: rg_upload_mesh copies into the slot the compute stream is
// not using, on a separate upload stream, computes that slot's geometry there
// and makes the compute stream wait for it, so an upload overlaps whatever
// compute work is still in flight on the previous mesh.
//
// Every index of a mesh is checked on the host before it is copied: the
// kernels index with them unchecked.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

#include "rg_handle.cuh"
#include "rg_motion.cuh"

using rg::DevStatus;

using namespace rgh;

namespace rgh {

rg_status cuda_fail(rg_handle* h, cudaError_t e) {
  if (h) {
    h->last = rg_error{RG_ERR_CUDA, 0, static_cast<int64_t>(e), 0.0};
  }
  cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? RG_ERR_OUT_OF_MEMORY : RG_ERR_CUDA;
}

rg_status invalid(rg_handle* h, int64_t index, double value) {
  if (h) h->last = rg_error{RG_ERR_INVALID_ARGUMENT, 0, index, value};
  return RG_ERR_INVALID_ARGUMENT;
}

}  // namespace rgh

namespace {

// Host-side checks of a packed mesh view that need no O(size) pass: counts,
// pointers and the CSR length.  Every index is checked on the device
// (k_validate) before any other kernel uses the mesh.
rg_status check_view(rg_handle* h, const rg_mesh_view* v, bool device_geometry) {
  if (!v || v->n_cells <= 0 || v->n_ghosts < 0 || v->n_faces < 0) return invalid(h, -1, 0);
  if (static_cast<int64_t>(v->n_cells) + v->n_ghosts > static_cast<int64_t>(rg::kNbrIdMask))
    return invalid(h, -2, 0);
  if (!v->point_xy || !v->face_cells || !v->face_vertices || !v->cell_face_offset || !v->cell_faces)
    return invalid(h, -3, 0);
  if (!device_geometry && (!v->cm_xy || !v->volume || !v->cd_volume)) return invalid(h, -3, 0);
  // rigid-wall ghost CMs are reflected about the box's sides
  if (device_geometry && v->n_ghosts > 0 && h->cfg.ghost_kind != RG_GHOST_PERIODIC && !h->have_box)
    return invalid(h, -5, 0);
  if (v->n_ghosts > 0 && (!v->ghost_source || !v->ghost_face)) return invalid(h, -3, 0);
  const int m = v->cell_face_offset[v->n_cells];
  if (v->cell_face_offset[0] != 0 || m < 0 || m > 2 * v->n_faces) return invalid(h, -4, m);
  return RG_OK;
}

bool is_pinned(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// memcpy split over a few threads for the large arrays of a mesh.
void par_memcpy(void* dst, const void* src, size_t bytes) {
  const size_t kChunk = size_t(4) << 20;
  const unsigned hw = std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
  const size_t parts = std::min<size_t>(hw, (bytes + kChunk - 1) / kChunk);
  if (parts <= 1) {
    std::memcpy(dst, src, bytes);
    return;
  }
  std::vector<std::thread> pool;
  const size_t per = (bytes + parts - 1) / parts;
  for (size_t k = 0; k < parts; ++k) {
    const size_t off = k * per;
    if (off >= bytes) break;
    const size_t len = std::min(per, bytes - off);
    pool.emplace_back([=] { std::memcpy(static_cast<char*>(dst) + off, static_cast<const char*>(src) + off, len); });
  }
  for (auto& t : pool) t.join();
}

void fill_views(MeshSlot& s) {
  void* b = s.buf.p;
  const SlotLayout& L = s.lay;
  s.mesh.n = s.n;
  s.mesh.g = s.g;
  s.mesh.e = s.e;
  s.mesh.m = s.m;
  s.mesh.points = at<double2>(b, L.points);
  s.mesh.cms = at<double2>(b, L.cms);
  s.mesh.volume = at<double>(b, L.volume);
  s.mesh.cd_volume = at<double>(b, L.cd_volume);
  s.mesh.ghost_source = at<int>(b, L.ghost_source);
  s.mesh.ghost_face = at<int>(b, L.ghost_face);
  s.mesh.face_cells = at<int2>(b, L.face_cells);
  s.mesh.face_vertices = at<rg::dbl4>(b, L.face_vertices);
  s.mesh.cell_off = at<int>(b, L.cell_off);
  s.mesh.cell_faces = at<int>(b, L.cell_faces);
  s.geom.area = at<double>(b, L.area);
  s.geom.nrm = at<double2>(b, L.nrm);
  s.geom.nabs = at<double>(b, L.nabs);
  s.geom.par = at<double2>(b, L.par);
  s.geom.dm0 = at<double2>(b, L.dm0);
  s.geom.dm1 = at<double2>(b, L.dm1);
  s.geom.dab = at<double>(b, L.dab);
  s.geom.xarea = L.own_xarea ? at<double>(b, L.xarea) : s.geom.area;
  s.geom.width = at<double>(b, L.width);
  s.geom.minv = at<rg::dbl4>(b, L.minv);
  s.geom.cflags = at<int>(b, L.cflags);
  s.geom.nbr = at<uint32_t>(b, L.nbr);
  s.geom.hr = at<double2>(b, L.hr);
  s.geom.ghost_real = at<int>(b, L.ghost_real);
  s.geom.ghost_unit = at<double2>(b, L.ghost_unit);
  s.geom.cell_order = at<int>(b, L.cell_order);
  s.g32.nrm = at<float2>(b, L.nrm32);
  s.g32.nabs = at<float>(b, L.nabs32);
  s.g32.par = at<float2>(b, L.par32);
  s.g32.area = at<float>(b, L.area32);
  s.g32.xarea = L.own_xarea ? at<float>(b, L.xarea32) : s.g32.area;
  s.g32.dm0 = at<float2>(b, L.dm0_32);
  s.g32.dm1 = at<float2>(b, L.dm1_32);
  s.g32.width = at<float>(b, L.width32);
  s.g32.minv = at<float4>(b, L.minv32);
  s.g32.ent = at<float4>(b, L.ent32);
  s.g32.fsign = at<int>(b, L.fsign32);
  s.g32.ghost_unit = at<float2>(b, L.gunit32);
  s.g32.inv_cd_volume = at<float>(b, L.icdv32);
}

}  // namespace

namespace rgh {

rg_status reset_status(rg_handle* h, DevStatus* st, cudaStream_t s) {
  // error part only: err_key = ~0, err_status = lock = 0
  RG_CUDA(h, cudaMemsetAsync(&st->err_key, 0xff, sizeof(unsigned long long), s));
  RG_CUDA(h, cudaMemsetAsync(&st->err_status, 0, 2 * sizeof(int), s));
  return RG_OK;
}

// Reads the status block after the stream is idle; returns the error (if any).
rg_status collect(rg_handle* h, DevStatus* st, cudaStream_t s) {
  DevStatus* hs = static_cast<DevStatus*>(h->host_status.p);
  RG_CUDA(h, cudaMemcpyAsync(hs, st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
  RG_CUDA(h, cudaStreamSynchronize(s));
  RG_CUDA(h, cudaGetLastError());
  h->last_dt = hs->dt;
  if (hs->err_key != ~0ull) {
    const unsigned long long key = hs->err_key;
    h->last = rg_error{hs->err_status, static_cast<int32_t>((key >> rg::kKeyPhaseShift) & 0xf),
                       static_cast<int64_t>(key & rg::kKeyIndexMask), hs->err_value};
    if (h->last.status == 0) h->last.status = RG_ERR_CUDA;  // key won a lock race; value stale
    return static_cast<rg_status>(h->last.status);
  }
  return RG_OK;
}

MeshSlot* active_slot(rg_handle* h) { return h->active < 0 ? nullptr : &h->slots[h->active]; }

rg::StepArgs step_args(rg_handle* h) {
  MeshSlot* s = active_slot(h);
  rg::StepArgs a{};
  a.mesh = s->mesh;
  a.geom = s->geom;
  a.gamma = h->cfg.gamma;
  a.cfl = h->cfg.cfl;
  a.order = h->cfg.order;
  a.ghost_kind = h->cfg.ghost_kind;
  a.slf = h->cfg.slope_limiter;
  a.delta_v = h->cfg.delta_v;
  a.theta = h->cfg.theta;
  a.delta_p = h->cfg.delta_p;
  a.cells = static_cast<double*>(h->cells.p);
  a.ext = static_cast<double*>(h->ext.p);
  a.ev = static_cast<const double*>(h->ev.p);
  a.slopes = static_cast<double*>(h->slopes.p);
  a.fluxes = static_cast<double*>(h->fluxes.p);
  a.status = h->d_status;
  a.dt_host = 0;
  a.dt_from_device = 0;
  a.step = 0;
  a.shapes = h->shapes64;
  a.ev_zero = h->ev_zero && !h->external_state;
  if (h->n_problems > 0) {
    a.cell_problem = static_cast<const int*>(h->cell_problem.p);
    a.gamma_p = static_cast<const double*>(h->gamma_p.p);
    a.dtmin_p = static_cast<unsigned long long*>(h->dtmin_p.p);
    a.time_p = static_cast<double*>(h->time_p.p);
    a.dt_p = static_cast<double*>(h->dt_p.p);
    a.n_problems = h->n_problems;
  }
  a.n_rules = h->n_rules;
  for (int k = 0; k < h->n_rules; ++k) {
    const rg_flux_rule& r = h->rules[k];
    a.rules[k][0] = r.sequence;
    a.rules[k][1] = r.condition;
    a.rules[k][2] = r.sticker;
    a.rules[k][3] = r.action;
    a.rules[k][4] = r.ratchet_in;
    a.rules[k][5] = r.massflux;
  }
  if (h->lag_rule && h->lag_ws.p) {
    a.lag_ws = static_cast<double*>(h->lag_ws.p);
    a.lag_ev = static_cast<double*>(h->lag_ev.p);
    a.lag_update = h->lag_update ? 1 : 0;
  }
  if (tracers_on(h)) {
    a.stickers = static_cast<const uint32_t*>(h->stickers.p);
    a.skip_mask = h->tcfg.skip_sticker >= 0 ? 1u << h->tcfg.skip_sticker : 0u;
    a.frozen_mask = h->tcfg.frozen_sticker >= 0 ? 1u << h->tcfg.frozen_sticker : 0u;
    if (h->tcfg.n_tracers > 0) {
      a.mflux = static_cast<double*>(h->mflux.p);
      if (h->n_rules > 0) a.tr_side = static_cast<unsigned char*>(h->tr_side.p);
      if (h->cfg.order == 2) a.shock = static_cast<unsigned char*>(h->shock.p);
    }
  }
  return a;
}

}  // namespace rgh

namespace rgh {

rg::MixedArgs mixed_args(rg_handle* h) {
  MeshSlot* s = active_slot(h);
  rg::MixedArgs a{};
  a.mesh = s->mesh;
  a.geom = s->geom;
  a.g32 = s->g32;
  a.gamma = static_cast<float>(h->cfg.gamma);
  a.inv_gm1 = static_cast<float>(1.0 / (h->cfg.gamma - 1.0));
  a.cfl = h->cfg.cfl;
  a.order = h->cfg.order;
  a.ghost_kind = h->cfg.ghost_kind;
  a.slf = h->cfg.slope_limiter;
  a.delta_v = static_cast<float>(h->cfg.delta_v);
  a.theta = static_cast<float>(h->cfg.theta);
  a.delta_p = static_cast<float>(h->cfg.delta_p);
  a.cells32 = static_cast<float4*>(h->cells32.p);
  a.slopes32 = static_cast<float4*>(h->slopes32.p);
  a.flux32 = static_cast<float4*>(h->flux32.p);
  a.ev32 = static_cast<const float2*>(h->ev32.p);
  a.ext = static_cast<double*>(h->ext.p);
  a.status = h->d_status;
  a.dt32 = 0;
  a.dt32_from_device = 0;
  a.step = 0;
  a.shapes = h->shapes32;
  a.ev_zero = h->ev_zero && !h->external_state;
  if (h->n_problems > 0) {
    a.cell_problem = static_cast<const int*>(h->cell_problem.p);
    a.gamma_p = static_cast<const float*>(h->gamma32_p.p);
    a.inv_gm1_p = static_cast<const float*>(h->inv_gm1_32_p.p);
    a.dtmin_p = static_cast<unsigned long long*>(h->dtmin_p.p);
    a.time_p = static_cast<double*>(h->time_p.p);
    a.dt_p = static_cast<double*>(h->dt_p.p);
    a.n_problems = h->n_problems;
  }
  if (tracers_on(h)) {
    a.stickers = static_cast<const uint32_t*>(h->stickers.p);
    a.skip_mask = h->tcfg.skip_sticker >= 0 ? 1u << h->tcfg.skip_sticker : 0u;
    a.frozen_mask = h->tcfg.frozen_sticker >= 0 ? 1u << h->tcfg.frozen_sticker : 0u;
    if (h->tcfg.n_tracers > 0) {
      a.mflux = static_cast<double*>(h->mflux.p);
      if (h->cfg.order == 2) a.shock = static_cast<unsigned char*>(h->shock.p);
    }
  }
  return a;
}

void drop_graph(rg_handle* h) {
  if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
  if (h->graph) cudaGraphDestroy(h->graph);
  h->graph_exec = nullptr;
  h->graph = nullptr;
}

}  // namespace rgh

namespace rgh {

rg_status require(rg_handle* h, bool cells, bool ext, bool ev, bool fluxes) {
  if (!h) return RG_ERR_INVALID_ARGUMENT;
  if (h->active < 0 || (cells && !h->have_cells) || (ext && !h->have_ext) || (ev && !h->have_ev) ||
      (fluxes && !h->have_fluxes)) {
    h->last = rg_error{RG_ERR_NOT_READY, 0, -1, 0};
    return RG_ERR_NOT_READY;
  }
  return RG_OK;
}

rg_status mesh_error(rg_handle* h) {
  MeshSlot* s = active_slot(h);
  if (h->cfg.order == 2 && s->geom_error.status != 0) {
    h->last = s->geom_error;
    return static_cast<rg_status>(s->geom_error.status);
  }
  return RG_OK;
}

}  // namespace rgh

namespace {

// Fused steps (the update computes the next step's dt): one problem, order 2
// (the slopes kernel moves the dt into place before the face kernel reads
// it), no caller access to the device buffers.
bool fusable(const rg_handle* h) { return h->cfg.order == 2 && h->n_problems == 0 && !h->external_state; }

// hdsim::TimeAdvance2Heun on a fixed mesh (hdsim2d.cpp:323-449): dt once;
// pass 1 on the cells writes the mid extensives and mid cells; pass 2 on the
// mid cells continues the mid extensives, averages them with the old ones
// (average_extensive, hdsim2d.cpp:311-320) and updates the cells.
rg_status enqueue_heun(rg_handle* h, int step, cudaEvent_t* ev) {
  const bool o2 = h->cfg.order == 2;
  if (h->mixed) {
    rg::MixedArgs a = mixed_args(h);
    a.dt32_from_device = 1;
    a.step = step;
    float4* mid_c = static_cast<float4*>(h->mid_cells32.p);
    double* mid_e = static_cast<double*>(h->mid_ext.p);
    if (ev) RG_CUDA(h, cudaEventRecord(ev[0], h->stream));
    RG_CUDA(h, rg::launch_cfl32(a, h->stream, o2));
    if (ev) RG_CUDA(h, cudaEventRecord(ev[1], h->stream));
    if (o2) RG_CUDA(h, rg::launch_slopes32(a, h->stream));
    RG_CUDA(h, rg::launch_faces32(a, h->stream, true));
    rg::MixedArgs a1 = a;
    a1.ext_out = mid_e;
    a1.cells32_out = mid_c;
    a1.batch_keep_dt = 1;  // a batch keeps each problem's dt for the second half
    RG_CUDA(h, rg::launch_update_mixed(a1, h->stream, false, true, true));
    if (ev) RG_CUDA(h, cudaEventRecord(ev[2], h->stream));
    rg::MixedArgs a2 = a;
    a2.cells32 = mid_c;
    if (o2) {
      RG_CUDA(h, rg::launch_ghost_fill32(a2, h->stream));
      RG_CUDA(h, rg::launch_slopes32(a2, h->stream));
    }
    RG_CUDA(h, rg::launch_faces32(a2, h->stream, true));
    if (ev) RG_CUDA(h, cudaEventRecord(ev[3], h->stream));
    rg::MixedArgs a3 = a2;
    a3.ext = mid_e;
    a3.ext_out = static_cast<double*>(h->ext.p);
    a3.ext_avg = static_cast<const double*>(h->ext.p);
    a3.cells32_out = static_cast<float4*>(h->cells32.p);
    RG_CUDA(h, rg::launch_update_mixed(a3, h->stream, false, true, true));
    if (ev) RG_CUDA(h, cudaEventRecord(ev[4], h->stream));
  } else {
    rg::StepArgs a = step_args(h);
    a.dt_from_device = 1;
    a.step = step;
    double* mid_c = static_cast<double*>(h->mid_cells.p);
    double* mid_e = static_cast<double*>(h->mid_ext.p);
    // tracers: the same two halves, mid tracers and extensive tracers beside
    // the mid cells and extensives (the tracer kernels of a half run after
    // its hydro kernels, whose mass fluxes and shock decisions they read)
    const bool tr = h->tcfg.n_tracers > 0;
    const rg::TracerArgs ta = tracer_args(h);
    rg::TracerArgs ta1 = ta, ta2 = ta, ta3 = ta;
    ta1.tr_out = ta2.tr = static_cast<double*>(h->mid_tr.p);
    ta1.tr_ext_out = ta3.tr_ext = static_cast<double*>(h->mid_tr_ext.p);
    ta3.tr_ext_out = ta.tr_ext;
    ta3.tr_ext_avg = ta.tr_ext;
    if (ev) RG_CUDA(h, cudaEventRecord(ev[0], h->stream));
    RG_CUDA(h, rg::launch_cfl(a, h->stream, o2));
    if (ev) RG_CUDA(h, cudaEventRecord(ev[1], h->stream));
    if (o2) {
      RG_CUDA(h, rg::launch_slopes(a, h->stream));
      if (tr) RG_CUDA(h, rg::launch_tr_slopes(a, ta, h->stream));
    }
    RG_CUDA(h, rg::launch_faces(a, h->stream, true));
    if (tr) RG_CUDA(h, rg::launch_tr_faces(a, ta, h->stream, true));
    rg::StepArgs a1 = a;
    a1.ext_out = mid_e;
    a1.cells_out = mid_c;
    a1.batch_keep_dt = 1;  // a batch keeps each problem's dt for the second half
    RG_CUDA(h, rg::launch_update(a1, h->stream, false, true, true));
    if (tr) RG_CUDA(h, rg::launch_tr_update(a1, ta1, h->stream, false, true, true));
    if (ev) RG_CUDA(h, cudaEventRecord(ev[2], h->stream));
    rg::StepArgs a2 = a;
    a2.cells = mid_c;
    if (o2) {
      RG_CUDA(h, rg::launch_ghost_fill(a2, h->stream));
      RG_CUDA(h, rg::launch_slopes(a2, h->stream));
      if (tr) RG_CUDA(h, rg::launch_tr_slopes(a2, ta2, h->stream));
    }
    RG_CUDA(h, rg::launch_faces(a2, h->stream, true));
    if (tr) RG_CUDA(h, rg::launch_tr_faces(a2, ta2, h->stream, true));
    if (ev) RG_CUDA(h, cudaEventRecord(ev[3], h->stream));
    rg::StepArgs a3 = a2;
    a3.ext = mid_e;
    a3.ext_out = static_cast<double*>(h->ext.p);
    a3.ext_avg = static_cast<const double*>(h->ext.p);
    a3.cells_out = static_cast<double*>(h->cells.p);
    RG_CUDA(h, rg::launch_update(a3, h->stream, false, true, true));
    if (tr) RG_CUDA(h, rg::launch_tr_update(a3, ta3, h->stream, false, true, true));
    if (ev) RG_CUDA(h, cudaEventRecord(ev[4], h->stream));
  }
  h->have_fluxes = false;
  return RG_OK;
}

// Enqueues one fused step (no host synchronisation).  With ev != nullptr,
// records ev[0..4] around its kernels.
rg_status enqueue_step(rg_handle* h, int step, cudaEvent_t* ev = nullptr) {
  if (h->heun) return enqueue_heun(h, step, ev);
  if (h->mixed) {
    rg::MixedArgs a = mixed_args(h);
    a.dt32_from_device = 1;
    a.step = step;
    const bool fuse = fusable(h), have_dt = fuse && h->dt_next_ready;
    // tracers: the FP64 tracer passes after each FP32 hydro pass, reading
    // its shock decisions and mass fluxes (the dt from the device)
    const bool tr = h->tcfg.n_tracers > 0;
    rg::StepArgs a64 = step_args(h);
    a64.dt_from_device = 1;
    a64.step = step;
    const rg::TracerArgs ta = tracer_args(h);
    if (ev) RG_CUDA(h, cudaEventRecord(ev[0], h->stream));
    if (!have_dt) RG_CUDA(h, rg::launch_cfl32(a, h->stream, false));
    if (ev) RG_CUDA(h, cudaEventRecord(ev[1], h->stream));
    a.take_next_dt = have_dt;
    if (h->cfg.order == 2) RG_CUDA(h, rg::launch_slopes32(a, h->stream));
    a.take_next_dt = 0;
    if (tr && h->cfg.order == 2) RG_CUDA(h, rg::launch_tr_slopes(a64, ta, h->stream));
    if (ev) RG_CUDA(h, cudaEventRecord(ev[2], h->stream));
    RG_CUDA(h, rg::launch_faces32(a, h->stream, true));
    if (tr) RG_CUDA(h, rg::launch_tr_faces(a64, ta, h->stream, true));
    if (ev) RG_CUDA(h, cudaEventRecord(ev[3], h->stream));
    a.cfl_next = fuse;
    RG_CUDA(h, rg::launch_update_mixed(a, h->stream, false, true, true));
    if (tr) {
      // the entropy tracer reads the new cells in FP64
      RG_CUDA(h, rg::launch_cells_to64(static_cast<const float4*>(h->cells32.p), static_cast<double*>(h->cells.p),
                                       active_slot(h)->n, h->stream));
      RG_CUDA(h, rg::launch_tr_update(a64, ta, h->stream, false, true, true));
    }
    if (ev) RG_CUDA(h, cudaEventRecord(ev[4], h->stream));
    h->dt_next_ready = fuse;
    h->have_fluxes = false;
    return RG_OK;
  }
  rg::StepArgs a = step_args(h);
  a.dt_from_device = 1;
  a.step = step;
  const bool fuse = fusable(h), have_dt = fuse && h->dt_next_ready;
  const bool tr = h->tcfg.n_tracers > 0;
  const rg::TracerArgs ta = tracer_args(h);
  if (ev) RG_CUDA(h, cudaEventRecord(ev[0], h->stream));
  if (!have_dt) RG_CUDA(h, rg::launch_cfl(a, h->stream, false));
  if (ev) RG_CUDA(h, cudaEventRecord(ev[1], h->stream));
  a.take_next_dt = have_dt;
  if (h->cfg.order == 2) RG_CUDA(h, rg::launch_slopes(a, h->stream));
  a.take_next_dt = 0;
  if (tr && h->cfg.order == 2) RG_CUDA(h, rg::launch_tr_slopes(a, ta, h->stream));
  if (ev) RG_CUDA(h, cudaEventRecord(ev[2], h->stream));
  RG_CUDA(h, rg::launch_faces(a, h->stream, true));
  if (tr) RG_CUDA(h, rg::launch_tr_faces(a, ta, h->stream, true));
  if (ev) RG_CUDA(h, cudaEventRecord(ev[3], h->stream));
  a.cfl_next = fuse;
  RG_CUDA(h, rg::launch_update(a, h->stream, false, true, true));
  if (tr) RG_CUDA(h, rg::launch_tr_update(a, ta, h->stream, false, true, true));
  if (ev) RG_CUDA(h, cudaEventRecord(ev[4], h->stream));
  h->dt_next_ready = fuse;
  h->have_fluxes = false;  // the buffer now holds dt*area-scaled fluxes
  return RG_OK;
}

// The persistent form takes a batch on the FP32-mixed path, second order,
// hdsim::TimeAdvance, without tracers, stickers or rule tables.
bool persistent_ok(const rg_handle* h) {
  return h->mixed && h->n_problems > 0 && h->cfg.order == 2 && !h->heun && !tracers_on(h) && h->n_rules == 0;
}

// rg_run of a batch as one cooperative launch (RG_STEP_PERSISTENT)
rg_status run_persistent(rg_handle* h, int32_t n_steps, double* dt_out) {
  if (!persistent_ok(h)) return invalid(h, -20, h->step_mode);
  RG_TRY(reset_status(h, h->d_status, h->stream));
  if (n_steps > 0) {
    RG_CUDA(h, h->barrier.ensure(sizeof(rg::GridBarrier)));
    RG_CUDA(h, h->dt_trace.ensure(sizeof(double) * static_cast<size_t>(n_steps)));
    rg::MixedArgs a = mixed_args(h);
    double* trace = static_cast<double*>(h->dt_trace.p);
    RG_CUDA(h, rg::launch_run32_persistent(a, n_steps, 0, static_cast<rg::GridBarrier*>(h->barrier.p), 0, trace,
                                           h->stream, nullptr));
    if (dt_out) {
      RG_CUDA(h, h->host_dts.ensure(sizeof(double) * static_cast<size_t>(n_steps)));
      RG_CUDA(h, cudaMemcpyAsync(h->host_dts.p, trace, sizeof(double) * static_cast<size_t>(n_steps),
                                 cudaMemcpyDeviceToHost, h->stream));
    }
  }
  h->dt_next_ready = false;
  h->have_fluxes = false;
  const rg_status st = collect(h, h->d_status, h->stream);
  if (dt_out && n_steps > 0) std::memcpy(dt_out, h->host_dts.p, sizeof(double) * static_cast<size_t>(n_steps));
  return st;
}

}  // namespace

namespace rgh {

// The per-face and per-cell geometry of slot s on stream st: the FP64 pass
// (and, for the FP32-mixed path, its rounded FP32 copies) when full64, else
// the FP32-mixed path's direct FP32 geometry with the few FP64 arrays its
// motion and neighbour walks read.
rg_status geometry_pass(rg_handle* h, MeshSlot& s, const rg::MeshDev& gm, bool full64, cudaStream_t st) {
  rg::GeomArgs ga{};
  ga.mesh = gm;
  ga.order = h->cfg.order;
  void* b = s.buf.p;
  ga.area = at<double>(b, s.lay.area);
  ga.nrm = at<double2>(b, s.lay.nrm);
  ga.nabs = at<double>(b, s.lay.nabs);
  ga.par = at<double2>(b, s.lay.par);
  ga.dm0 = at<double2>(b, s.lay.dm0);
  ga.dm1 = at<double2>(b, s.lay.dm1);
  ga.dab = at<double>(b, s.lay.dab);
  ga.rij = at<double2>(b, s.lay.rij);
  ga.cij = at<double2>(b, s.lay.cij);
  ga.width = at<double>(b, s.lay.width);
  ga.minv = at<rg::dbl4>(b, s.lay.minv);
  ga.cflags = at<int>(b, s.lay.cflags);
  ga.nbr = at<uint32_t>(b, s.lay.nbr);
  ga.hr = at<double2>(b, s.lay.hr);
  ga.ghost_real = at<int>(b, s.lay.ghost_real);
  ga.ghost_unit = at<double2>(b, s.lay.ghost_unit);
  ga.cell_order = at<int>(b, s.lay.cell_order);
  ga.ghost_kind = h->cfg.ghost_kind;
  ga.status = h->d_geom_status;
  if (full64) RG_CUDA(h, rg::launch_geometry(ga, st));
  s.geom64 = full64;
  if (h->mixed) {
    rg::MixedGeomArgs m32{};
    m32.n = s.n;
    m32.g = s.g;
    m32.e = s.e;
    m32.m = s.m;
    m32.g64 = s.geom;
    m32.nrm = at<float2>(b, s.lay.nrm32);
    m32.nabs = at<float>(b, s.lay.nabs32);
    m32.par = at<float2>(b, s.lay.par32);
    m32.area = at<float>(b, s.lay.area32);
    m32.xarea = s.lay.own_xarea ? at<float>(b, s.lay.xarea32) : m32.area;
    m32.dm0 = at<float2>(b, s.lay.dm0_32);
    m32.dm1 = at<float2>(b, s.lay.dm1_32);
    m32.width = at<float>(b, s.lay.width32);
    m32.minv = at<float4>(b, s.lay.minv32);
    m32.ent = at<float4>(b, s.lay.ent32);
    m32.fsign = at<int>(b, s.lay.fsign32);
    m32.cell_faces = s.mesh.cell_faces;
    m32.ghost_unit = at<float2>(b, s.lay.gunit32);
    m32.inv_cd_volume = at<float>(b, s.lay.icdv32);
    m32.cd_volume = s.mesh.cd_volume;
    m32.invalid = gm.invalid;
    m32.frec = at<float4>(b, s.lay.frec32);
    if (full64) {
      RG_CUDA(h, rg::launch_geom32(m32, st));
    } else {
      RG_CUDA(h, rg::launch_geom_ghosts(ga, st));
      RG_CUDA(h, rg::launch_geom32_direct(ga, m32, st));
    }
  }
  return RG_OK;
}

// The FP64 geometry of the active slot, for the FP64 passes that run on an
// FP32-mixed handle (tracers, differentiation, rg_get_geometry): formed on
// the compute stream once per mesh, with the FP32 copies rounded from it.
rg_status ensure_geom64(rg_handle* h) {
  if (h->active < 0) return RG_OK;
  MeshSlot& s = h->slots[h->active];
  if (s.geom64) return RG_OK;
  RG_CUDA(h, cudaStreamWaitEvent(h->stream, h->ev_uploaded, 0));
  rg::MeshDev gm = s.mesh;
  gm.invalid = nullptr;
  return geometry_pass(h, s, gm, true, h->stream);
}

}  // namespace rgh

extern "C" {

void rg_default_config(rg_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof *c);
  c->gamma = 5.0 / 3.0;
  c->cfl = 0.3;
  c->order = 2;
  c->ghost_kind = RG_GHOST_RIGID_WALL;
  c->slope_limiter = 1;
  c->precision = RG_FP64;
  c->delta_v = 0.2;
  c->theta = 0.5;
  c->delta_p = 0.7;
  c->device = 0;
}

const char* rg_status_string(rg_status s) {
  switch (s) {
    case RG_OK: return "ok";
    case RG_ERR_INVALID_ARGUMENT: return "invalid argument";
    case RG_ERR_CUDA: return "CUDA error";
    case RG_ERR_NOT_READY: return "not ready (mesh or state missing)";
    case RG_ERR_OUT_OF_MEMORY: return "out of device memory";
    case RG_ERR_NEGATIVE_DENSITY: return "Negative density";
    case RG_ERR_NEGATIVE_ENERGY: return "Negative thermal energy";
    case RG_ERR_HLLC_NAN: return "Hllc::Solved entered with nan";
    case RG_ERR_HLLC_WAVE_SPEEDS: return "Invalid wave speeds in hllc solver";
    case RG_ERR_SINGULAR_MATRIX: return "Singular matrix";
    case RG_ERR_TOO_MANY_NEIGHBORS: return "Cell has too many neighbors";
    case RG_ERR_TIMEOUT: return "a device-side wait timed out";
  }
  return "unknown status";
}

rg_status rg_create(const rg_config* cfg, rg_handle** out) {
  if (!cfg || !out) return RG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (cfg->order != 1 && cfg->order != 2) return RG_ERR_INVALID_ARGUMENT;
  if (cfg->ghost_kind != RG_GHOST_RIGID_WALL && cfg->ghost_kind != RG_GHOST_PERIODIC)
    return RG_ERR_INVALID_ARGUMENT;
  if (cfg->precision != RG_FP64 && cfg->precision != RG_FP32_MIXED) return RG_ERR_INVALID_ARGUMENT;
  if (cfg->time_integrator != RG_TIME_ADVANCE && cfg->time_integrator != RG_TIME_ADVANCE_HEUN)
    return RG_ERR_INVALID_ARGUMENT;
  if (!(cfg->gamma > 1.0) || !(cfg->cfl > 0.0)) return RG_ERR_INVALID_ARGUMENT;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= cfg->device || cfg->device < 0) {
    cudaGetLastError();
    return RG_ERR_CUDA;
  }
  rg_handle* h = new (std::nothrow) rg_handle();
  if (!h) return RG_ERR_OUT_OF_MEMORY;
  h->cfg = *cfg;
  h->mixed = cfg->precision == RG_FP32_MIXED;
  h->heun = cfg->time_integrator == RG_TIME_ADVANCE_HEUN;
  auto fail = [&](cudaError_t e) {
    rg_destroy(h);
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? RG_ERR_OUT_OF_MEMORY : RG_ERR_CUDA;
  };
  cudaError_t e;
  if ((e = cudaSetDevice(cfg->device)) != cudaSuccess) return fail(e);
  if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess) return fail(e);
  if ((e = cudaStreamCreateWithFlags(&h->upload_stream, cudaStreamNonBlocking)) != cudaSuccess) return fail(e);
  if ((e = cudaEventCreateWithFlags(&h->ev_uploaded, cudaEventDisableTiming)) != cudaSuccess) return fail(e);
  if ((e = cudaStreamCreateWithFlags(&h->download_stream, cudaStreamNonBlocking)) != cudaSuccess) return fail(e);
  if ((e = cudaEventCreateWithFlags(&h->ev_state, cudaEventDisableTiming)) != cudaSuccess) return fail(e);
  if ((e = cudaEventCreateWithFlags(&h->ev_downloaded, cudaEventDisableTiming)) != cudaSuccess) return fail(e);
  for (auto& s : h->slots)
    if ((e = cudaEventCreateWithFlags(&s.last_use, cudaEventDisableTiming)) != cudaSuccess) return fail(e);
  for (auto& k : h->ev_k)
    if ((e = cudaEventCreateWithFlags(&k, cudaEventDefault)) != cudaSuccess) return fail(e);
  if ((e = h->status_buf.ensure(3 * sizeof(DevStatus))) != cudaSuccess) return fail(e);
  h->d_status = static_cast<DevStatus*>(h->status_buf.p);
  h->d_geom_status = h->d_status + 1;
  h->d_valid_status = h->d_status + 2;
  DevStatus init{};
  init.err_key = ~0ull;
  init.dt_min_bits = rg::kInfBits;
  DevStatus all[3] = {init, init, init};
  if ((e = cudaMemcpy(h->d_status, all, sizeof all, cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e);
  if ((e = h->host_status.ensure(2 * sizeof(DevStatus))) != cudaSuccess) return fail(e);
  *out = h;
  return RG_OK;
}

rg_status rg_destroy(rg_handle* h) {
  if (!h) return RG_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->upload_stream) cudaStreamSynchronize(h->upload_stream);
  if (h->download_stream) cudaStreamSynchronize(h->download_stream);
  for (auto& s : h->slots) {
    s.buf.release();
    if (s.last_use) cudaEventDestroy(s.last_use);
  }
  adjoint_release(h);
  tracer_release(h);
  h->lag_ws.release();
  h->lag_ev.release();
  h->pv.release();
  h->flag_buf.release();
  h->barrier.release();
  h->dt_trace.release();
  h->cells.release();
  h->ext.release();
  h->ev.release();
  h->slopes.release();
  h->fluxes.release();
  h->mid_ext.release();
  h->mid_cells.release();
  h->mid_cells32.release();
  for (DevBuf* b : {&h->cell_problem, &h->problem_offsets, &h->gamma_p, &h->gamma32_p, &h->inv_gm1_32_p,
                    &h->dtmin_p, &h->time_p, &h->dt_p})
    b->release();
  if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
  if (h->graph) cudaGraphDestroy(h->graph);
  h->cells32.release();
  h->slopes32.release();
  h->flux32.release();
  h->ev32.release();
  h->status_buf.release();
  h->staging.release();
  h->host_status.release();
  h->host_dts.release();
  for (auto& k : h->ev_k)
    if (k) cudaEventDestroy(k);
  if (h->ev_uploaded) cudaEventDestroy(h->ev_uploaded);
  if (h->ev_state) cudaEventDestroy(h->ev_state);
  if (h->ev_downloaded) cudaEventDestroy(h->ev_downloaded);
  if (h->stream) cudaStreamDestroy(h->stream);
  if (h->upload_stream) cudaStreamDestroy(h->upload_stream);
  if (h->download_stream) cudaStreamDestroy(h->download_stream);
  cudaGetLastError();
  delete h;
  return RG_OK;
}

rg_status rg_last_error(const rg_handle* h, rg_error* err) {
  if (!h || !err) return RG_ERR_INVALID_ARGUMENT;
  *err = h->last;
  return RG_OK;
}

rg_status rg_upload_mesh(rg_handle* h, const rg_mesh_view* v, uint32_t flags) {
  if (!h) return RG_ERR_INVALID_ARGUMENT;
  h->last = rg_error{};
  h->dt_next_ready = false;
  const auto t0 = std::chrono::steady_clock::now();
  const bool device_geometry = (flags & RG_MESH_DEVICE_GEOMETRY) != 0;
  if (rg_status st = check_view(h, v, device_geometry)) return st;
  RG_CUDA(h, cudaSetDevice(h->cfg.device));
  const int n = v->n_cells, g = v->n_ghosts, e = v->n_faces, m = v->cell_face_offset[n];
  const bool n_changed = h->active >= 0 && active_slot(h)->n != n;
  const int next = h->active < 0 ? 0 : 1 - h->active;
  MeshSlot& s = h->slots[next];
  // the slot may still be read by kernels enqueued on the previous-but-one mesh
  RG_CUDA(h, cudaStreamWaitEvent(h->upload_stream, s.last_use, 0));
  s.lay.compute(n, g, e, m, h->mixed, h->pgeo.kind == RG_GEOMETRY_CYLINDRICAL);
  RG_CUDA(h, cudaStreamSynchronize(h->upload_stream));
  RG_CUDA(h, s.buf.ensure(s.lay.total));
  RG_CUDA(h, h->staging.ensure(s.lay.input_end));
  s.n = n;
  s.g = g;
  s.e = e;
  s.m = m;
  fill_views(s);
  // inputs: straight from the caller's arrays when they are pinned, through
  // the pinned staging buffer otherwise
  char* st = static_cast<char*>(h->staging.p);
  const size_t np = static_cast<size_t>(n) + g;
  struct Part {
    size_t off;
    const void* src;
    size_t bytes;
  } parts[10] = {{s.lay.points, v->point_xy, 16 * np},
                 {s.lay.cms, v->cm_xy, 16 * np},
                 {s.lay.volume, v->volume, 8 * static_cast<size_t>(n)},
                 {s.lay.cd_volume, v->cd_volume, 8 * static_cast<size_t>(n)},
                 {s.lay.ghost_source, v->ghost_source, 4 * static_cast<size_t>(g)},
                 {s.lay.ghost_face, v->ghost_face, 4 * static_cast<size_t>(g)},
                 {s.lay.face_cells, v->face_cells, 8 * static_cast<size_t>(e)},
                 {s.lay.face_vertices, v->face_vertices, 32 * static_cast<size_t>(e)},
                 {s.lay.cell_off, v->cell_face_offset, 4 * (static_cast<size_t>(n) + 1)},
                 {s.lay.cell_faces, v->cell_faces, 4 * static_cast<size_t>(m)}};
  for (const Part& p : parts) {
    if (p.bytes == 0 || p.src == nullptr) continue;  // device geometry: computed below
    if (is_pinned(p.src)) {
      RG_CUDA(h, cudaMemcpyAsync(static_cast<char*>(s.buf.p) + p.off, p.src, p.bytes, cudaMemcpyHostToDevice,
                                 h->upload_stream));
    } else {
      par_memcpy(st + p.off, p.src, p.bytes);
      RG_CUDA(h, cudaMemcpyAsync(static_cast<char*>(s.buf.p) + p.off, st + p.off, p.bytes, cudaMemcpyHostToDevice,
                                 h->upload_stream));
    }
  }
  // every index is checked before any kernel uses it: the validation runs
  // first on the upload stream and the geometry kernels behind it return at
  // once when it has failed, so the host reads both results after one wait
  RG_TRY(reset_status(h, h->d_valid_status, h->upload_stream));
  RG_CUDA(h, rg::launch_validate(s.mesh, h->d_valid_status, h->upload_stream));
  rg::MeshDev gm = s.mesh;
  gm.invalid = &h->d_valid_status->err_key;
  // geometry pass on the upload stream (the per-cell kernels take cells in
  // the per-tile neighbour-count order, computed first)
  RG_TRY(reset_status(h, h->d_geom_status, h->upload_stream));
  RG_CUDA(h, rg::launch_cell_order(gm, at<int>(s.buf.p, s.lay.cell_order), at<int>(s.buf.p, s.lay.cflags),
                                   h->upload_stream));
  if (device_geometry)
    RG_CUDA(h, rg::launch_device_geometry(gm, at<int>(s.buf.p, s.lay.cell_order), at<double2>(s.buf.p, s.lay.cms), at<double>(s.buf.p, s.lay.volume),
                                          at<double>(s.buf.p, s.lay.cd_volume), h->cfg.ghost_kind, h->box,
                                          h->upload_stream));
  if (h->pgeo.kind == RG_GEOMETRY_CYLINDRICAL)
    RG_CUDA(h, rg::launch_cyl_geometry(gm, at<double>(s.buf.p, s.lay.xarea),
                                       device_geometry ? at<double>(s.buf.p, s.lay.cd_volume) : nullptr,
                                       h->pgeo.origin, h->pgeo.direction, h->pgeo.unit != 0, h->upload_stream));
  // the FP32-mixed path without tracers takes its FP32 geometry straight
  // from the inputs; the FP64 geometry is formed when something needs it
  // (ensure_geom64)
  RG_TRY(geometry_pass(h, s, gm, !h->mixed || tracers_on(h), h->upload_stream));
  RG_CUDA(h, cudaEventRecord(h->ev_uploaded, h->upload_stream));
  // the geometry errors (hs[0]; reconstruction would throw them) and the
  // validation (hs[1])
  DevStatus* hs = static_cast<DevStatus*>(h->host_status.p);
  RG_CUDA(h, cudaMemcpyAsync(hs, h->d_geom_status, 2 * sizeof(DevStatus), cudaMemcpyDeviceToHost, h->upload_stream));
  RG_CUDA(h, cudaStreamSynchronize(h->upload_stream));
  if (hs[1].err_key != ~0ull) {
    // the slot holds an invalid mesh: it is not activated
    s.n = s.g = s.e = s.m = 0;
    return invalid(h, static_cast<int64_t>(hs[1].err_key & rg::kKeyIndexMask), hs[1].err_value);
  }
  if (n_changed) {
    // the cell count changed: the state no longer matches the mesh
    h->have_cells = h->have_ext = false;
  }
  // state buffers sized for this mesh (cells keep their first n records)
  const size_t rec = np;
  if (rec > h->cells_records) {
    DevBuf nb;
    RG_CUDA(h, nb.ensure(32 * rec));
    RG_CUDA(h, cudaStreamSynchronize(h->stream));
    if (h->cells.p && h->have_cells)
      RG_CUDA(h, cudaMemcpy(nb.p, h->cells.p, 32 * static_cast<size_t>(n), cudaMemcpyDeviceToDevice));
    h->cells.release();
    h->cells = nb;
    if (h->mixed) {
      DevBuf nb32;
      RG_CUDA(h, nb32.ensure(16 * rec));
      if (h->cells32.p && h->have_cells)
        RG_CUDA(h, cudaMemcpy(nb32.p, h->cells32.p, 16 * static_cast<size_t>(n), cudaMemcpyDeviceToDevice));
      h->cells32.release();
      h->cells32 = nb32;
    }
    h->cells_records = rec;
  }
  const bool ext_keep = h->ext.bytes >= 32 * static_cast<size_t>(n);
  // the compute stream may still use the state buffers (a step in flight,
  // an rg_get_state_async copy it waits for): wait for it only when one of
  // them is reallocated below
  {
    const size_t e1 = static_cast<size_t>(std::max(e, 1)), nn = static_cast<size_t>(n);
    bool grows = !ext_keep || h->ev.bytes < 16 * e1 || h->slopes.bytes < 64 * nn || h->fluxes.bytes < 32 * e1;
    if (h->heun)
      grows = grows || h->mid_ext.bytes < 32 * nn ||
              (h->mixed ? h->mid_cells32.bytes < 16 * np : h->mid_cells.bytes < 32 * np);
    if (h->mixed)
      grows = grows || h->slopes32.bytes < 32 * nn || h->flux32.bytes < 16 * e1 || h->ev32.bytes < 8 * e1;
    if (grows) RG_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  if (!ext_keep) h->have_ext = false;
  RG_CUDA(h, h->ext.ensure(32 * static_cast<size_t>(n)));
  if (h->ev.bytes < 16 * static_cast<size_t>(e)) h->have_ev = false;
  if (h->ev64_pending) {
    // the FP32-mixed device motion's face velocities belong to the old mesh
    h->ev64_pending = false;
    h->have_ev = false;
  }
  RG_CUDA(h, h->ev.ensure(16 * static_cast<size_t>(std::max(e, 1))));
  RG_CUDA(h, h->slopes.ensure(64 * static_cast<size_t>(n)));
  RG_CUDA(h, h->fluxes.ensure(32 * static_cast<size_t>(std::max(e, 1))));
  if (h->heun) {
    RG_CUDA(h, h->mid_ext.ensure(32 * static_cast<size_t>(n)));
    if (h->mixed)
      RG_CUDA(h, h->mid_cells32.ensure(16 * np));
    else
      RG_CUDA(h, h->mid_cells.ensure(32 * np));
  }
  if (h->mixed) {
    RG_CUDA(h, h->slopes32.ensure(32 * static_cast<size_t>(n)));
    RG_CUDA(h, h->flux32.ensure(16 * static_cast<size_t>(std::max(e, 1))));
    RG_CUDA(h, h->ev32.ensure(8 * static_cast<size_t>(std::max(e, 1))));
  }
  if (h->active >= 0 && active_slot(h)->e != e) h->have_ev = false;
  h->have_fluxes = false;
  s.geom_error = rg_error{};
  if (hs->err_key != ~0ull)
    s.geom_error = rg_error{hs->err_status, 2, static_cast<int64_t>(hs->err_key & rg::kKeyIndexMask), hs->err_value};
  // a new mesh drops the batch table, the captured step and the
  // differentiation buffers
  h->n_problems = 0;
  drop_graph(h);
  adjoint_release(h);
  // later compute work on the stream sees the new slot
  RG_CUDA(h, cudaStreamWaitEvent(h->stream, h->ev_uploaded, 0));
  if (h->active >= 0) RG_CUDA(h, cudaEventRecord(h->slots[h->active].last_use, h->stream));
  h->active = next;
  s.valid = true;
  if (tracers_on(h)) RG_TRY(tracer_buffers(h));
  RG_TRY(lagrangian_buffers(h));
  h->last_upload_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (h->cfg.order == 2 && s.geom_error.status) {
    h->last = s.geom_error;
    return static_cast<rg_status>(s.geom_error.status);
  }
  return RG_OK;
}

rg_status rg_last_upload_ms(const rg_handle* h, double* ms) {
  if (!h || !ms) return RG_ERR_INVALID_ARGUMENT;
  *ms = h->last_upload_ms;
  return RG_OK;
}

rg_status rg_set_cells(rg_handle* h, const double* cells) {
  if (!h || !cells) return RG_ERR_INVALID_ARGUMENT;
  h->dt_next_ready = false;
  if (h->active < 0) return require(h, false, false, false, false);
  RG_CUDA(h, cudaMemcpyAsync(h->cells.p, cells, 32 * static_cast<size_t>(active_slot(h)->n),
                             cudaMemcpyHostToDevice, h->stream));
  if (h->mixed)
    RG_CUDA(h, rg::launch_cells_to32(static_cast<const double*>(h->cells.p), static_cast<float4*>(h->cells32.p),
                                     active_slot(h)->n, h->stream));
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  h->have_cells = true;
  return RG_OK;
}

rg_status rg_get_cells(rg_handle* h, double* cells) {
  if (rg_status st = require(h, true, false, false, false)) return st;
  if (!cells) return RG_ERR_INVALID_ARGUMENT;
  if (h->mixed)
    RG_CUDA(h, rg::launch_cells_to64(static_cast<const float4*>(h->cells32.p), static_cast<double*>(h->cells.p),
                                     active_slot(h)->n, h->stream));
  RG_CUDA(h, cudaMemcpyAsync(cells, h->cells.p, 32 * static_cast<size_t>(active_slot(h)->n),
                             cudaMemcpyDeviceToHost, h->stream));
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  return RG_OK;
}

rg_status rg_get_state_async(rg_handle* h, double* cells, double* ext) {
  if (!h || (!cells && !ext)) return RG_ERR_INVALID_ARGUMENT;
  if (rg_status st = require(h, cells != nullptr, ext != nullptr, false, false)) return st;
  const size_t bytes = 32 * static_cast<size_t>(active_slot(h)->n);
  if (cells && h->mixed)
    RG_CUDA(h, rg::launch_cells_to64(static_cast<const float4*>(h->cells32.p), static_cast<double*>(h->cells.p),
                                     active_slot(h)->n, h->stream));
  RG_CUDA(h, cudaEventRecord(h->ev_state, h->stream));
  RG_CUDA(h, cudaStreamWaitEvent(h->download_stream, h->ev_state, 0));
  if (cells)
    RG_CUDA(h, cudaMemcpyAsync(cells, h->cells.p, bytes, cudaMemcpyDeviceToHost, h->download_stream));
  if (ext) RG_CUDA(h, cudaMemcpyAsync(ext, h->ext.p, bytes, cudaMemcpyDeviceToHost, h->download_stream));
  RG_CUDA(h, cudaEventRecord(h->ev_downloaded, h->download_stream));
  // everything enqueued on the compute stream later waits for the copies
  RG_CUDA(h, cudaStreamWaitEvent(h->stream, h->ev_downloaded, 0));
  h->state_pending = true;
  return RG_OK;
}

rg_status rg_wait_state(rg_handle* h) {
  if (!h) return RG_ERR_INVALID_ARGUMENT;
  if (h->state_pending) RG_CUDA(h, cudaEventSynchronize(h->ev_downloaded));
  h->state_pending = false;
  return RG_OK;
}

rg_status rg_set_extensives(rg_handle* h, const double* ext) {
  if (!h || !ext) return RG_ERR_INVALID_ARGUMENT;
  if (h->active < 0) return require(h, false, false, false, false);
  RG_CUDA(h, cudaMemcpyAsync(h->ext.p, ext, 32 * static_cast<size_t>(active_slot(h)->n),
                             cudaMemcpyHostToDevice, h->stream));
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  h->have_ext = true;
  return RG_OK;
}

rg_status rg_get_extensives(rg_handle* h, double* ext) {
  if (rg_status st = require(h, false, true, false, false)) return st;
  if (!ext) return RG_ERR_INVALID_ARGUMENT;
  RG_CUDA(h, cudaMemcpyAsync(ext, h->ext.p, 32 * static_cast<size_t>(active_slot(h)->n),
                             cudaMemcpyDeviceToHost, h->stream));
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  return RG_OK;
}

rg_status rg_set_edge_velocities(rg_handle* h, const double* ev) {
  if (!h || !ev) return RG_ERR_INVALID_ARGUMENT;
  h->ev64_pending = false;
  h->dt_next_ready = false;
  if (h->active < 0) return require(h, false, false, false, false);
  RG_CUDA(h, cudaMemcpyAsync(h->ev.p, ev, 16 * static_cast<size_t>(active_slot(h)->e),
                             cudaMemcpyHostToDevice, h->stream));
  if (h->mixed)
    RG_CUDA(h, rg::launch_vec2_to32(static_cast<const double*>(h->ev.p), static_cast<float2*>(h->ev32.p),
                                    active_slot(h)->e, h->stream));
  // all faces at rest (Eulerian mesh): the kernels then read no face velocities
  RG_CUDA(h, h->flag_buf.ensure(sizeof(int)));
  RG_CUDA(h, cudaMemsetAsync(h->flag_buf.p, 0, sizeof(int), h->stream));
  RG_CUDA(h, rg::launch_any_nonzero(static_cast<const double*>(h->ev.p), 2LL * active_slot(h)->e,
                                    static_cast<int*>(h->flag_buf.p), h->stream));
  int* hflag = reinterpret_cast<int*>(h->host_status.p);
  RG_CUDA(h, cudaMemcpyAsync(hflag, h->flag_buf.p, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  h->ev_zero = *hflag == 0;
  h->have_ev = true;
  return RG_OK;
}

rg_status rg_set_fluxes(rg_handle* h, const double* fl) {
  if (!h || !fl) return RG_ERR_INVALID_ARGUMENT;
  if (h->active < 0) return require(h, false, false, false, false);
  RG_CUDA(h, cudaMemcpyAsync(h->fluxes.p, fl, 32 * static_cast<size_t>(active_slot(h)->e),
                             cudaMemcpyHostToDevice, h->stream));
  if (h->mixed)
    RG_CUDA(h, rg::launch_flux_to32(static_cast<const double*>(h->fluxes.p), static_cast<float4*>(h->flux32.p),
                                    active_slot(h)->e, h->stream));
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  h->have_fluxes = true;
  return RG_OK;
}

rg_status rg_device_buffers(rg_handle* h, rg_device_view* v) {
  if (!h || !v) return RG_ERR_INVALID_ARGUMENT;
  if (h->active < 0) return require(h, false, false, false, false);
  v->cells = static_cast<double*>(h->cells.p);
  v->extensives = static_cast<double*>(h->ext.p);
  v->edge_velocities = static_cast<double*>(h->ev.p);
  v->fluxes = static_cast<double*>(h->fluxes.p);
  v->stream = h->stream;
  // a caller writing through these pointers provides the state, at any time
  h->have_cells = h->have_ext = h->have_ev = true;
  h->external_state = true;
  h->dt_next_ready = false;
  return RG_OK;
}

rg_status rg_stream(const rg_handle* h, void** stream) {
  if (!h || !stream) return RG_ERR_INVALID_ARGUMENT;
  *stream = h->stream;
  return RG_OK;
}

rg_status rg_init_extensives(rg_handle* h) {
  if (rg_status st = require(h, true, false, false, false)) return st;
  rg::StepArgs a = step_args(h);
  if (h->mixed)
    RG_CUDA(h, rg::launch_cells_to64(static_cast<const float4*>(h->cells32.p), static_cast<double*>(h->cells.p),
                                     active_slot(h)->n, h->stream));
  RG_CUDA(h, rg::launch_init_extensives(a, h->stream));
  if (h->tcfg.n_tracers > 0 && h->have_tr) {
    RG_CUDA(h, rg::launch_tr_init(a, tracer_args(h), h->stream));
    h->have_tr_ext = true;
  }
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  h->have_ext = true;
  return RG_OK;
}

rg_status rg_cfl_dt(rg_handle* h, double* dt) {
  if (rg_status st = require(h, true, false, true, false)) return st;
  if (!dt || h->n_problems > 0) return invalid(h, -1, 0);
  h->last = rg_error{};
  RG_TRY(reset_status(h, h->d_status, h->stream));
  if (h->mixed) {
    RG_CUDA(h, rg::launch_cfl32(mixed_args(h), h->stream, false));
  } else {
    rg::StepArgs a = step_args(h);
    RG_CUDA(h, rg::launch_cfl(a, h->stream, false));
  }
  rg_status st = collect(h, h->d_status, h->stream);
  *dt = h->last_dt;
  return st;
}

rg_status rg_flux(rg_handle* h, double dt, double* fluxes_out) {
  if (rg_status st = require(h, true, false, true, false)) return st;
  if (rg_status st = require_tracers(h, false)) return st;
  h->last = rg_error{};
  if (rg_status st = mesh_error(h)) return st;
  RG_TRY(reset_status(h, h->d_status, h->stream));
  if (h->mixed) {
    rg::MixedArgs a = mixed_args(h);
    a.dt32 = static_cast<float>(dt);
    const bool tr = h->tcfg.n_tracers > 0;
    rg::StepArgs a64 = step_args(h);
    a64.dt_host = dt;
    const rg::TracerArgs ta = tracer_args(h);
    if (h->cfg.order == 2) {
      RG_CUDA(h, rg::launch_ghost_fill32(a, h->stream));
      RG_CUDA(h, rg::launch_slopes32(a, h->stream));
      if (tr) RG_CUDA(h, rg::launch_tr_slopes(a64, ta, h->stream));
    }
    RG_CUDA(h, rg::launch_faces32(a, h->stream, false));
    if (tr) RG_CUDA(h, rg::launch_tr_faces(a64, ta, h->stream, false));
  } else {
    rg::StepArgs a = step_args(h);
    a.dt_host = dt;
    const bool tr = h->tcfg.n_tracers > 0;
    const rg::TracerArgs ta = tracer_args(h);
    if (h->cfg.order == 2) {
      RG_CUDA(h, rg::launch_ghost_fill(a, h->stream));
      RG_CUDA(h, rg::launch_slopes(a, h->stream));
      if (tr) RG_CUDA(h, rg::launch_tr_slopes(a, ta, h->stream));
    }
    RG_CUDA(h, rg::launch_faces(a, h->stream, false));
    if (tr) RG_CUDA(h, rg::launch_tr_faces(a, ta, h->stream, false));
  }
  if (rg_status st = collect(h, h->d_status, h->stream)) return st;
  h->have_fluxes = true;
  if (fluxes_out) {
    if (h->mixed)
      RG_CUDA(h, rg::launch_flux_to64(static_cast<const float4*>(h->flux32.p), static_cast<double*>(h->fluxes.p),
                                      active_slot(h)->e, h->stream));
    RG_CUDA(h, cudaMemcpyAsync(fluxes_out, h->fluxes.p, 32 * static_cast<size_t>(active_slot(h)->e),
                               cudaMemcpyDeviceToHost, h->stream));
    RG_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  return RG_OK;
}

rg_status rg_extensive_update(rg_handle* h, double dt) {
  if (rg_status st = require(h, false, true, false, true)) return st;
  if (rg_status st = require_tracers(h, true)) return st;
  h->last = rg_error{};
  RG_TRY(reset_status(h, h->d_status, h->stream));
  if (h->mixed) {
    rg::MixedArgs a = mixed_args(h);
    a.dt32 = static_cast<float>(dt);
    RG_CUDA(h, rg::launch_update_mixed(a, h->stream, true, true, false));
    if (h->tcfg.n_tracers > 0) {
      rg::StepArgs a64 = step_args(h);
      a64.dt_host = dt;
      RG_CUDA(h, rg::launch_tr_update(a64, tracer_args(h), h->stream, true, true, false));
    }
  } else {
    rg::StepArgs a = step_args(h);
    a.dt_host = dt;
    RG_CUDA(h, rg::launch_update(a, h->stream, true, true, false));
    if (h->tcfg.n_tracers > 0) RG_CUDA(h, rg::launch_tr_update(a, tracer_args(h), h->stream, true, true, false));
  }
  return collect(h, h->d_status, h->stream);
}

rg_status rg_cell_update(rg_handle* h) {
  if (rg_status st = require(h, false, true, false, false)) return st;
  if (rg_status st = require_tracers(h, true)) return st;
  h->last = rg_error{};
  h->dt_next_ready = false;
  RG_TRY(reset_status(h, h->d_status, h->stream));
  if (h->mixed) {
    RG_CUDA(h, rg::launch_update_mixed(mixed_args(h), h->stream, false, false, true));
    if (h->tcfg.n_tracers > 0) {
      // the entropy tracer reads the new cells in FP64
      RG_CUDA(h, rg::launch_cells_to64(static_cast<const float4*>(h->cells32.p), static_cast<double*>(h->cells.p),
                                       active_slot(h)->n, h->stream));
      RG_CUDA(h, rg::launch_tr_update(step_args(h), tracer_args(h), h->stream, false, false, true));
    }
  } else {
    rg::StepArgs a = step_args(h);
    RG_CUDA(h, rg::launch_update(a, h->stream, false, false, true));
    if (h->tcfg.n_tracers > 0) RG_CUDA(h, rg::launch_tr_update(a, tracer_args(h), h->stream, false, false, true));
  }
  rg_status st = collect(h, h->d_status, h->stream);
  if (st == RG_OK) h->have_cells = true;
  return st;
}

rg_status rg_step_async(rg_handle* h) {
  if (rg_status st = require(h, true, true, true, false)) return st;
  if (rg_status st = require_tracers(h, true)) return st;
  if (rg_status st = mesh_error(h)) return st;
  if (h->step_seq == 0) RG_TRY(reset_status(h, h->d_status, h->stream));
  rg_status st = enqueue_step(h, h->step_seq);
  h->step_seq = std::min(h->step_seq + 1, 0x1fff);
  return st;
}

rg_status rg_synchronize(rg_handle* h, double* dt_last) {
  if (!h) return RG_ERR_INVALID_ARGUMENT;
  h->last = rg_error{};
  h->step_seq = 0;
  rg_status st = collect(h, h->d_status, h->stream);
  if (dt_last) *dt_last = h->last_dt;
  return st;
}

rg_status rg_step(rg_handle* h, double* dt_out) {
  if (rg_status st = require(h, true, true, true, false)) return st;
  if (rg_status st = require_tracers(h, true)) return st;
  if (rg_status st = mesh_error(h)) return st;
  h->last = rg_error{};
  RG_TRY(reset_status(h, h->d_status, h->stream));
  if (rg_status st = enqueue_step(h, 0)) return st;
  rg_status st = collect(h, h->d_status, h->stream);
  if (dt_out) *dt_out = h->last_dt;
  return st;
}

rg_status rg_step_timed(rg_handle* h, double* dt_out, float* kernel_ms) {
  if (rg_status st = require(h, true, true, true, false)) return st;
  if (rg_status st = require_tracers(h, true)) return st;
  if (rg_status st = mesh_error(h)) return st;
  if (!kernel_ms) return RG_ERR_INVALID_ARGUMENT;
  h->last = rg_error{};
  RG_TRY(reset_status(h, h->d_status, h->stream));
  if (rg_status st = enqueue_step(h, 0, h->ev_k)) return st;
  rg_status st = collect(h, h->d_status, h->stream);
  for (int k = 0; k < 4; ++k) {
    kernel_ms[k] = 0;
    RG_CUDA(h, cudaEventElapsedTime(&kernel_ms[k], h->ev_k[k], h->ev_k[k + 1]));
  }
  if (dt_out) *dt_out = h->last_dt;
  return st;
}

rg_status rg_run(rg_handle* h, int32_t n_steps, double* dt_out) {
  if (rg_status st = require(h, true, true, true, false)) return st;
  if (rg_status st = require_tracers(h, true)) return st;
  if (n_steps < 0) return RG_ERR_INVALID_ARGUMENT;
  if (rg_status st = mesh_error(h)) return st;
  h->last = rg_error{};
  if (h->step_mode == RG_STEP_PERSISTENT) return run_persistent(h, n_steps, dt_out);
  RG_TRY(reset_status(h, h->d_status, h->stream));
  if (dt_out) RG_CUDA(h, h->host_dts.ensure(sizeof(double) * static_cast<size_t>(std::max(n_steps, 1))));
  double* hd = static_cast<double*>(h->host_dts.p);
  for (int k = 0; k < n_steps; ++k) {
    if (rg_status st = enqueue_step(h, std::min(k, 0x1fff))) return st;
    if (dt_out)
      RG_CUDA(h, cudaMemcpyAsync(hd + k, h->n_problems > 0 ? static_cast<double*>(h->dt_p.p) : &h->d_status->dt,
                                 sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  }
  rg_status st = collect(h, h->d_status, h->stream);
  if (dt_out) std::memcpy(dt_out, hd, sizeof(double) * static_cast<size_t>(n_steps));
  return st;
}

rg_status rg_set_step_mode(rg_handle* h, int32_t mode) {
  if (!h) return RG_ERR_INVALID_ARGUMENT;
  h->last = rg_error{};
  if (mode != RG_STEP_PER_PHASE && mode != RG_STEP_PERSISTENT) return invalid(h, 0, mode);
  if (mode == RG_STEP_PERSISTENT && !persistent_ok(h)) return invalid(h, 1, mode);
  h->step_mode = mode;
  return RG_OK;
}

rg_status rg_grid_barrier_check(rg_handle* h, int32_t missing_blocks) {
  if (!h || missing_blocks < 0) return RG_ERR_INVALID_ARGUMENT;
  h->last = rg_error{};
  RG_CUDA(h, cudaSetDevice(h->cfg.device));
  RG_CUDA(h, h->barrier.ensure(sizeof(rg::GridBarrier)));
  RG_TRY(reset_status(h, h->d_status, h->stream));
  RG_CUDA(h, rg::launch_barrier_check(static_cast<rg::GridBarrier*>(h->barrier.p), missing_blocks, h->d_status,
                                      h->stream));
  return collect(h, h->d_status, h->stream);
}

rg_status rg_set_problems(rg_handle* h, int32_t P, const int32_t* offsets, const double* gamma) {
  if (!h) return RG_ERR_INVALID_ARGUMENT;
  if (h->active < 0) return require(h, false, false, false, false);
  h->last = rg_error{};
  drop_graph(h);
  h->dt_next_ready = false;
  MeshSlot* s = active_slot(h);
  if (P == 0) {
    h->n_problems = 0;
    return RG_OK;
  }
  if (P < 0 || !offsets || !gamma || h->n_rules > 0) return invalid(h, -1, P);
  if (offsets[0] != 0 || offsets[P] != s->n) return invalid(h, -2, offsets[P]);
  for (int p = 0; p < P; ++p) {
    if (offsets[p + 1] <= offsets[p]) return invalid(h, p, offsets[p + 1]);
    if (!(gamma[p] > 1.0)) return invalid(h, p, gamma[p]);
  }
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  RG_CUDA(h, h->cell_problem.ensure(4 * (static_cast<size_t>(s->n) + s->g)));
  RG_CUDA(h, h->problem_offsets.ensure(4 * (static_cast<size_t>(P) + 1)));
  RG_CUDA(h, h->gamma_p.ensure(8 * static_cast<size_t>(P)));
  RG_CUDA(h, h->gamma32_p.ensure(4 * static_cast<size_t>(P)));
  RG_CUDA(h, h->inv_gm1_32_p.ensure(4 * static_cast<size_t>(P)));
  RG_CUDA(h, h->dtmin_p.ensure(8 * static_cast<size_t>(P)));
  RG_CUDA(h, h->time_p.ensure(8 * static_cast<size_t>(P)));
  RG_CUDA(h, h->dt_p.ensure(8 * static_cast<size_t>(P)));
  std::vector<float> g32(static_cast<size_t>(P)), igm(static_cast<size_t>(P));
  std::vector<unsigned long long> inf(static_cast<size_t>(P), rg::kInfBits);
  for (int p = 0; p < P; ++p) {
    g32[static_cast<size_t>(p)] = static_cast<float>(gamma[p]);
    igm[static_cast<size_t>(p)] = static_cast<float>(1.0 / (gamma[p] - 1.0));
  }
  RG_CUDA(h, cudaMemcpy(h->problem_offsets.p, offsets, 4 * (static_cast<size_t>(P) + 1), cudaMemcpyHostToDevice));
  RG_CUDA(h, cudaMemcpy(h->gamma_p.p, gamma, 8 * static_cast<size_t>(P), cudaMemcpyHostToDevice));
  RG_CUDA(h, cudaMemcpy(h->gamma32_p.p, g32.data(), 4 * static_cast<size_t>(P), cudaMemcpyHostToDevice));
  RG_CUDA(h, cudaMemcpy(h->inv_gm1_32_p.p, igm.data(), 4 * static_cast<size_t>(P), cudaMemcpyHostToDevice));
  RG_CUDA(h, cudaMemcpy(h->dtmin_p.p, inf.data(), 8 * static_cast<size_t>(P), cudaMemcpyHostToDevice));
  RG_CUDA(h, cudaMemset(h->time_p.p, 0, 8 * static_cast<size_t>(P)));
  RG_CUDA(h, cudaMemset(h->dt_p.p, 0, 8 * static_cast<size_t>(P)));
  RG_TRY(reset_status(h, h->d_geom_status, h->stream));
  RG_CUDA(h, rg::launch_problems(s->mesh, static_cast<const int*>(h->problem_offsets.p), P,
                                 static_cast<int*>(h->cell_problem.p), h->d_geom_status, h->stream));
  DevStatus* hs = static_cast<DevStatus*>(h->host_status.p);
  RG_CUDA(h, cudaMemcpyAsync(hs, h->d_geom_status, sizeof(DevStatus), cudaMemcpyDeviceToHost, h->stream));
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  if (hs->err_key != ~0ull) {
    h->n_problems = 0;
    return invalid(h, static_cast<int64_t>(hs->err_key & rg::kKeyIndexMask), hs->err_value);
  }
  h->n_problems = P;
  return RG_OK;
}

rg_status rg_get_problem_times(rg_handle* h, double* time_out, double* dt_out) {
  if (!h) return RG_ERR_INVALID_ARGUMENT;
  if (h->n_problems <= 0) return invalid(h, -1, 0);
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  if (time_out)
    RG_CUDA(h, cudaMemcpy(time_out, h->time_p.p, 8 * static_cast<size_t>(h->n_problems), cudaMemcpyDeviceToHost));
  if (dt_out)
    RG_CUDA(h, cudaMemcpy(dt_out, h->dt_p.p, 8 * static_cast<size_t>(h->n_problems), cudaMemcpyDeviceToHost));
  return RG_OK;
}

rg_status rg_run_graph(rg_handle* h, int32_t n_steps) {
  if (rg_status st = require(h, true, true, true, false)) return st;
  if (rg_status st = require_tracers(h, true)) return st;
  if (n_steps < 0) return RG_ERR_INVALID_ARGUMENT;
  if (rg_status st = mesh_error(h)) return st;
  h->last = rg_error{};
  if (n_steps == 0) return RG_OK;
  if (h->step_mode == RG_STEP_PERSISTENT) return run_persistent(h, n_steps, nullptr);
  RG_TRY(reset_status(h, h->d_status, h->stream));
  if (fusable(h) && !h->dt_next_ready) {
    // one step with its own CFL pass; the captured step is the fused form,
    // which takes the dt the previous step's update computed
    RG_TRY(enqueue_step(h, 0));
    if (--n_steps == 0) {
      h->have_fluxes = false;
      return collect(h, h->d_status, h->stream);
    }
  }
  if (!h->graph_exec) {
    RG_CUDA(h, cudaStreamSynchronize(h->stream));
    RG_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    const rg_status st = enqueue_step(h, 0);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(h->stream, &g);
    if (st != RG_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    if (ce != cudaSuccess) return cuda_fail(h, ce);
    h->graph = g;
    RG_CUDA(h, cudaGraphInstantiate(&h->graph_exec, h->graph, 0));
  }
  for (int k = 0; k < n_steps; ++k) RG_CUDA(h, cudaGraphLaunch(h->graph_exec, h->stream));
  h->have_fluxes = false;
  return collect(h, h->d_status, h->stream);
}

}  // extern "C"
