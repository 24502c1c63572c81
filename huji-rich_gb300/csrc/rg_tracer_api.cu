// rg_tracer_api.cu -- C ABI of tracers and stickers (include/rich_gb300.h,
// "Tracers and stickers"): configuration, state transfer and the handle's
// tracer buffers.  The kernels are in rg_tracers.cu; the hydro kernels read
// the sticker masks (rg_fp64.cu).
//
// The reference keeps tracers and stickers inside every ComputationalCell
// (computational_cell_2d.hpp:19-36) and names them through
// TracerStickerNames (hdsim2d.hpp:86-101); here they are flat cell-major
// arrays and bit masks, and the names' sorted positions are the indices.
#include <cuda_runtime.h>

#include <cstring>

#include "rg_handle.cuh"

using namespace rgh;

namespace rgh {

bool tracers_on(const rg_handle* h) {
  return h->tcfg.n_tracers > 0 || h->tcfg.n_stickers > 0 || h->tcfg.skip_sticker >= 0 ||
         h->tcfg.frozen_sticker >= 0;
}

void tracer_release(rg_handle* h) {
  for (DevBuf* b : {&h->tr, &h->tr_ext, &h->tr_slopes, &h->tr_flux, &h->mflux, &h->tr_side, &h->shock, &h->stickers,
                    &h->mid_tr, &h->mid_tr_ext})
    b->release();
  h->have_tr = h->have_tr_ext = false;
  h->tr_n = h->tr_e = -1;
}

rg_status tracer_buffers(rg_handle* h) {
  MeshSlot* s = active_slot(h);
  if (!s) return RG_OK;
  const size_t n = static_cast<size_t>(s->n), e = static_cast<size_t>(s->e > 0 ? s->e : 1);
  const size_t nt = static_cast<size_t>(h->tcfg.n_tracers > 0 ? h->tcfg.n_tracers : 1);
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  if (s->n != h->tr_n) {
    // a new cell count: the tracer state no longer matches, stickers start clear
    h->have_tr = h->have_tr_ext = false;
    h->stickers.release();
    RG_CUDA(h, h->stickers.ensure(4 * n));
    RG_CUDA(h, cudaMemset(h->stickers.p, 0, 4 * n));
  }
  RG_CUDA(h, h->tr.ensure(8 * n * nt));
  RG_CUDA(h, h->tr_ext.ensure(8 * n * nt));
  RG_CUDA(h, h->tr_slopes.ensure(16 * n * nt));
  RG_CUDA(h, h->tr_flux.ensure(8 * e * nt));
  RG_CUDA(h, h->mflux.ensure(8 * e));
  RG_CUDA(h, h->tr_side.ensure(e));
  RG_CUDA(h, h->shock.ensure(n));
  if (h->heun) {
    RG_CUDA(h, h->mid_tr.ensure(8 * n * nt));
    RG_CUDA(h, h->mid_tr_ext.ensure(8 * n * nt));
  }
  h->tr_n = s->n;
  h->tr_e = s->e;
  drop_graph(h);
  return RG_OK;
}

rg::TracerArgs tracer_args(rg_handle* h) {
  rg::TracerArgs t{};
  t.nt = h->tcfg.n_tracers;
  t.limited = h->tcfg.limited_mask;
  t.entropy = h->tcfg.entropy_tracer;
  t.tr = static_cast<double*>(h->tr.p);
  t.tr_ext = static_cast<double*>(h->tr_ext.p);
  t.tr_slopes = static_cast<double*>(h->tr_slopes.p);
  t.tr_flux = static_cast<double*>(h->tr_flux.p);
  return t;
}

rg_status require_tracers(rg_handle* h, bool ext) {
  if (h->tcfg.n_tracers == 0) return RG_OK;
  if (!h->have_tr || (ext && !h->have_tr_ext)) {
    h->last = rg_error{RG_ERR_NOT_READY, 0, -2, 0};
    return RG_ERR_NOT_READY;
  }
  return RG_OK;
}

}  // namespace rgh

namespace {

// host <-> device copy of one cell-major tracer array (n_cells * n_tracers)
rg_status copy_tracers(rg_handle* h, DevBuf& d, void* host, bool to_device, size_t per_row) {
  MeshSlot* s = active_slot(h);
  const size_t bytes = 8 * static_cast<size_t>(s->n) * per_row;
  if (bytes == 0) return RG_OK;
  RG_CUDA(h, cudaMemcpyAsync(to_device ? d.p : host, to_device ? host : d.p, bytes,
                             to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, h->stream));
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  return RG_OK;
}

rg_status ready(rg_handle* h, const void* p) {
  if (!h || !p) return RG_ERR_INVALID_ARGUMENT;
  if (h->active < 0) return require(h, false, false, false, false);
  if (h->tcfg.n_tracers == 0) return invalid(h, -1, 0);
  return RG_OK;
}

}  // namespace

extern "C" {

rg_status rg_set_tracer_config(rg_handle* h, const rg_tracer_config* cfg) {
  if (!h) return RG_ERR_INVALID_ARGUMENT;
  h->last = rg_error{};
  const rg_tracer_config off{0, 0, 0u, -1, -1, -1};
  const rg_tracer_config c = cfg ? *cfg : off;
  if (c.n_tracers < 0 || c.n_tracers > RG_MAX_TRACERS) return invalid(h, 0, c.n_tracers);
  if (c.n_stickers < 0 || c.n_stickers > 32) return invalid(h, 6, c.n_stickers);
  if (c.n_tracers < 32 && (c.limited_mask >> c.n_tracers) != 0) return invalid(h, 1, c.limited_mask);
  if (c.entropy_tracer < -1 || c.entropy_tracer >= c.n_tracers) return invalid(h, 2, c.entropy_tracer);
  if (c.skip_sticker < -1 || c.skip_sticker > 31) return invalid(h, 3, c.skip_sticker);
  if (c.frozen_sticker < -1 || c.frozen_sticker > 31) return invalid(h, 4, c.frozen_sticker);
  const bool on = c.n_tracers > 0 || c.n_stickers > 0 || c.skip_sticker >= 0 || c.frozen_sticker >= 0;
  // the FP32-mixed path runs its tracer passes with hdsim::TimeAdvance (fused
  // or through the plugin calls), not in the fused TimeAdvance2Heun step
  if (on && h->mixed && h->heun) return invalid(h, 5, 0);
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  const bool nt_changed = c.n_tracers != h->tcfg.n_tracers;
  h->tcfg = c;
  drop_graph(h);
  h->dt_next_ready = false;
  if (!on) {
    tracer_release(h);
    return RG_OK;
  }
  if (nt_changed) h->have_tr = h->have_tr_ext = false;
  RG_TRY(tracer_buffers(h));
  // the tracer passes read the FP64 geometry
  return ensure_geom64(h);
}

rg_status rg_set_tracers(rg_handle* h, const double* tracers) {
  if (rg_status st = ready(h, tracers)) return st;
  RG_TRY(copy_tracers(h, h->tr, const_cast<double*>(tracers), true, h->tcfg.n_tracers));
  h->have_tr = true;
  return RG_OK;
}

rg_status rg_get_tracers(rg_handle* h, double* tracers) {
  if (rg_status st = ready(h, tracers)) return st;
  if (rg_status st = require_tracers(h, false)) return st;
  return copy_tracers(h, h->tr, tracers, false, h->tcfg.n_tracers);
}

rg_status rg_set_extensive_tracers(rg_handle* h, const double* tracers) {
  if (rg_status st = ready(h, tracers)) return st;
  RG_TRY(copy_tracers(h, h->tr_ext, const_cast<double*>(tracers), true, h->tcfg.n_tracers));
  h->have_tr_ext = true;
  return RG_OK;
}

rg_status rg_get_extensive_tracers(rg_handle* h, double* tracers) {
  if (rg_status st = ready(h, tracers)) return st;
  if (!h->have_tr_ext) return require_tracers(h, true);
  return copy_tracers(h, h->tr_ext, tracers, false, h->tcfg.n_tracers);
}

rg_status rg_set_stickers(rg_handle* h, const uint32_t* stickers) {
  if (!h || !stickers) return RG_ERR_INVALID_ARGUMENT;
  if (h->active < 0) return require(h, false, false, false, false);
  if (!tracers_on(h)) return invalid(h, -1, 0);
  RG_CUDA(h, cudaMemcpyAsync(h->stickers.p, stickers, 4 * static_cast<size_t>(active_slot(h)->n),
                             cudaMemcpyHostToDevice, h->stream));
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  return RG_OK;
}

rg_status rg_set_tracer_fluxes(rg_handle* h, const double* in) {
  if (rg_status st = ready(h, in)) return st;
  const size_t bytes = 8 * static_cast<size_t>(active_slot(h)->e) * h->tcfg.n_tracers;
  if (bytes) {
    RG_CUDA(h, cudaMemcpyAsync(h->tr_flux.p, in, bytes, cudaMemcpyHostToDevice, h->stream));
    RG_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  return RG_OK;
}

rg_status rg_get_tracer_fluxes(rg_handle* h, double* out) {
  if (rg_status st = ready(h, out)) return st;
  if (!h->have_fluxes) return require(h, false, false, false, true);
  const size_t bytes = 8 * static_cast<size_t>(active_slot(h)->e) * h->tcfg.n_tracers;
  if (bytes) {
    RG_CUDA(h, cudaMemcpyAsync(out, h->tr_flux.p, bytes, cudaMemcpyDeviceToHost, h->stream));
    RG_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  return RG_OK;
}

rg_status rg_get_tracer_slopes(rg_handle* h, double* out) {
  if (rg_status st = ready(h, out)) return st;
  if (h->cfg.order != 2) return invalid(h, -2, h->cfg.order);
  if (!h->have_fluxes) return require(h, false, false, false, true);
  return copy_tracers(h, h->tr_slopes, out, false, 2 * static_cast<size_t>(h->tcfg.n_tracers));
}

}  // extern "C"
