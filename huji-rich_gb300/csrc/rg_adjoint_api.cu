// rg_adjoint_api.cu -- the differentiation entry points of the C ABI:
// rg_step_fwd / rg_step_bwd (adjoint pair with checkpointing) and
// rg_step_tlm (tangent-linear run).
//
// Forward: the plain FP64 kernels of rg_fp64.cu with the fixed dt (ghost
// fill, slopes, dt*area-scaled fluxes, update), W and U copied to a
// checkpoint every `every` steps.
// Backward: per checkpoint interval, last first: the interval is recomputed
// from its checkpoint into per-step buffers (W_k with ghost records, U_k, the
// slopes and the limiter trace of k_record_slopes, which yields the same
// slopes as the plain path), then the reverse steps run from the interval's
// last step to its first.  Memory: (n_steps/every) checkpoints of 64 bytes
// per cell plus `every` recomputed steps of about 240 bytes per cell.
// The reverse adjacency (which face sides and CSR entries read each cell)
// is built once per mesh on the host, in ascending order, so every reverse
// gather is deterministic.
// FP32-mixed handles differentiate the FP32-mixed step: the forward and the
// recomputation run the FP32-mixed kernels, the recomputation records the
// limiter trace of the FP32 slopes (k_slopes32_trace), and the reverse runs
// the face and cell kernels in FP32 with the FP64 transposed gather and cell
// update (adj_launch_reverse32).  Checkpoints hold the FP32 primitives.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <utility>
#include <vector>

#include "rg_adjoint.cuh"
#include "rg_handle.cuh"

using namespace rgh;

struct rg_adjoint_state {
  int n = 0, g = 0, e = 0, m = 0;  // mesh the adjacency was built for
  bool adjacency = false;
  DevBuf side_off, sides, target_off, targets;
  // forward record
  bool have_forward = false;
  int n_steps = 0, every = 0, n_ckpt = 0;
  double dt = 0;
  DevBuf ckpt_cells, ckpt_ext, final_ext;
  // recomputed interval
  DevBuf seg_cells, seg_ext, seg_slopes, seg_trace;
  // reverse sweep and tangent work arrays
  DevBuf ubar0, ubar1, side_bar, self_bar, entry_bar, io;
  DevBuf dcells, dslopes, dflux, dext;
  // FP32-mixed recomputation: the interval's running FP32 primitives and extensives
  DevBuf w_cells32, w_ext;
  void release() {
    for (DevBuf* b : {&side_off, &sides, &target_off, &targets, &ckpt_cells, &ckpt_ext, &final_ext, &seg_cells,
                      &seg_ext, &seg_slopes, &seg_trace, &ubar0, &ubar1, &side_bar, &self_bar, &entry_bar, &io,
                      &dcells, &dslopes, &dflux, &dext, &w_cells32, &w_ext})
      b->release();
    adjacency = have_forward = false;
  }
};

namespace rgh {

void adjoint_release(rg_handle* h) {
  if (!h || !h->adj) return;
  h->adj->release();
  delete h->adj;
  h->adj = nullptr;
}

}  // namespace rgh

namespace {

template <class T>
T* ptr(DevBuf& b, size_t elem_offset = 0) {
  return static_cast<T*>(b.p) + elem_offset;
}

rg_status check_config(rg_handle* h, bool allow_mixed = true) {
  if (h->cfg.order != 2 || h->cfg.ghost_kind != RG_GHOST_PERIODIC || (h->mixed && !allow_mixed) || h->heun ||
      h->n_problems > 0 ||
      tracers_on(h) || active_slot(h)->lay.own_xarea || h->n_rules > 0)
    return invalid(h, -10, h->cfg.order);
  // the reverse kernels read the FP64 geometry (rounded to FP32 for an
  // FP32-mixed handle, as its forward kernels then use it)
  return ensure_geom64(h);
}

rg::AdjArgs adj_args(rg_handle* h) {
  MeshSlot* s = active_slot(h);
  rg_adjoint_state* A = h->adj;
  rg::AdjArgs a{};
  a.mesh = s->mesh;
  a.geom = s->geom;
  a.gamma = h->cfg.gamma;
  a.dt = A->dt;
  a.delta_v = h->cfg.delta_v;
  a.theta = h->cfg.theta;
  a.delta_p = h->cfg.delta_p;
  a.slf = h->cfg.slope_limiter;
  a.status = h->d_status;
  a.side_bar = ptr<double>(A->side_bar);
  a.self_bar = ptr<double>(A->self_bar);
  a.entry_bar = ptr<double>(A->entry_bar);
  a.side_off = ptr<int>(A->side_off);
  a.sides = ptr<int>(A->sides);
  a.target_off = ptr<int>(A->target_off);
  a.targets = ptr<int>(A->targets);
  return a;
}

// Counting sort of keys 0..n-1 that keeps ascending item order per key.
void bucket(int n, const std::vector<int>& key, std::vector<int>& off, std::vector<int>& items) {
  off.assign(static_cast<size_t>(n) + 1, 0);
  for (int k : key) ++off[static_cast<size_t>(k) + 1];
  for (int i = 0; i < n; ++i) off[static_cast<size_t>(i) + 1] += off[static_cast<size_t>(i)];
  items.resize(key.size());
  std::vector<int> fill(off.begin(), off.end() - 1);
  for (size_t t = 0; t < key.size(); ++t) items[static_cast<size_t>(fill[static_cast<size_t>(key[t])]++)] = static_cast<int>(t);
}

// Reverse adjacency of the active mesh and the check that it is one the
// adjoint covers (no self-mirror neighbour, no boundary-slope cell).
rg_status ensure_adjacency(rg_handle* h) {
  MeshSlot* s = active_slot(h);
  if (!h->adj) {
    h->adj = new (std::nothrow) rg_adjoint_state();
    if (!h->adj) return RG_ERR_OUT_OF_MEMORY;
  }
  rg_adjoint_state* A = h->adj;
  if (A->adjacency && A->n == s->n && A->g == s->g && A->e == s->e && A->m == s->m) return RG_OK;
  A->adjacency = false;
  A->have_forward = false;
  const int n = s->n, g = s->g, e = s->e, m = s->m;
  std::vector<int2> fc(static_cast<size_t>(e));
  std::vector<int> gsrc(static_cast<size_t>(g));
  std::vector<uint32_t> nbr(static_cast<size_t>(m));
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  if (e) RG_CUDA(h, cudaMemcpy(fc.data(), s->mesh.face_cells, 8 * static_cast<size_t>(e), cudaMemcpyDeviceToHost));
  if (g) RG_CUDA(h, cudaMemcpy(gsrc.data(), s->mesh.ghost_source, 4 * static_cast<size_t>(g), cudaMemcpyDeviceToHost));
  if (m) RG_CUDA(h, cudaMemcpy(nbr.data(), s->geom.nbr, 4 * static_cast<size_t>(m), cudaMemcpyDeviceToHost));
  auto source = [&](int p) { return p < n ? p : gsrc[static_cast<size_t>(p - n)]; };
  std::vector<int> key(2 * static_cast<size_t>(e)), off, items;
  for (int f = 0; f < e; ++f) {
    key[2 * static_cast<size_t>(f)] = source(fc[static_cast<size_t>(f)].x);
    key[2 * static_cast<size_t>(f) + 1] = source(fc[static_cast<size_t>(f)].y);
  }
  bucket(n, key, off, items);
  RG_CUDA(h, A->side_off.ensure(4 * off.size()));
  RG_CUDA(h, A->sides.ensure(4 * std::max<size_t>(items.size(), 1)));
  RG_CUDA(h, cudaMemcpy(A->side_off.p, off.data(), 4 * off.size(), cudaMemcpyHostToDevice));
  if (!items.empty()) RG_CUDA(h, cudaMemcpy(A->sides.p, items.data(), 4 * items.size(), cudaMemcpyHostToDevice));
  key.resize(static_cast<size_t>(m));
  for (int t = 0; t < m; ++t) key[static_cast<size_t>(t)] = source(static_cast<int>(nbr[static_cast<size_t>(t)] & rg::kNbrIdMask));
  bucket(n, key, off, items);
  RG_CUDA(h, A->target_off.ensure(4 * off.size()));
  RG_CUDA(h, A->targets.ensure(4 * std::max<size_t>(items.size(), 1)));
  RG_CUDA(h, cudaMemcpy(A->target_off.p, off.data(), 4 * off.size(), cudaMemcpyHostToDevice));
  if (!items.empty()) RG_CUDA(h, cudaMemcpy(A->targets.p, items.data(), 4 * items.size(), cudaMemcpyHostToDevice));
  // work arrays of the reverse sweep
  const size_t ne = std::max(e, 1), nm = std::max(m, 1);
  RG_CUDA(h, A->ubar0.ensure(32 * static_cast<size_t>(n)));
  RG_CUDA(h, A->ubar1.ensure(32 * static_cast<size_t>(n)));
  RG_CUDA(h, A->io.ensure(32 * static_cast<size_t>(n)));
  RG_CUDA(h, A->side_bar.ensure(64 * ne));
  RG_CUDA(h, A->self_bar.ensure(32 * static_cast<size_t>(n)));
  RG_CUDA(h, A->entry_bar.ensure(32 * nm));
  RG_CUDA(h, A->final_ext.ensure(32 * static_cast<size_t>(n)));
  // the mesh must be one the adjoint covers
  RG_TRY(reset_status(h, h->d_status, h->stream));
  RG_CUDA(h, rg::adj_launch_check(adj_args(h), h->stream));
  if (collect(h, h->d_status, h->stream) != RG_OK) {
    h->last.status = RG_ERR_INVALID_ARGUMENT;
    return RG_ERR_INVALID_ARGUMENT;
  }
  A->n = n;
  A->g = g;
  A->e = e;
  A->m = m;
  A->adjacency = true;
  return RG_OK;
}

// The plain FP64 step with a fixed dt, from a.cells / a.ext into
// a.cells_out / a.ext_out (nullptr: in place).
rg_status enqueue_plain_step(rg_handle* h, const rg::StepArgs& a, bool faces_and_update = true) {
  RG_CUDA(h, rg::launch_ghost_fill(a, h->stream));
  RG_CUDA(h, rg::launch_slopes(a, h->stream));
  if (faces_and_update) {
    RG_CUDA(h, rg::launch_faces(a, h->stream, true));
    RG_CUDA(h, rg::launch_update(a, h->stream, false, true, true));
  }
  return RG_OK;
}

rg_status check_run(rg_handle* h, int32_t n_steps, double dt, bool allow_mixed = true) {
  if (rg_status st = require(h, true, false, false, false)) return st;
  if (rg_status st = check_config(h, allow_mixed)) return st;
  if (n_steps < 1 || !(dt > 0)) return invalid(h, -11, dt);
  if (rg_status st = mesh_error(h)) return st;
  return ensure_adjacency(h);
}

// One FP32-mixed step with a fixed dt on the FP32 primitives and FP64
// extensives of `m` (in place).
rg_status enqueue_mixed_step(rg_handle* h, const rg::MixedArgs& m) {
  RG_CUDA(h, rg::launch_slopes32(m, h->stream));
  RG_CUDA(h, rg::launch_faces32(m, h->stream, true));
  RG_CUDA(h, rg::launch_update_mixed(m, h->stream, false, true, true));
  return RG_OK;
}

rg::MixedArgs mixed_fixed_dt(rg_handle* h, double dt) {
  rg::MixedArgs m = mixed_args(h);
  m.dt32 = static_cast<float>(dt);
  m.dt32_from_device = 0;
  return m;
}

}  // namespace

extern "C" {

rg_status rg_step_fwd(rg_handle* h, int32_t n_steps, double dt, int32_t every) {
  if (!h) return RG_ERR_INVALID_ARGUMENT;
  h->last = rg_error{};
  if (rg_status st = check_run(h, n_steps, dt)) return st;
  if (every < 1) return invalid(h, -12, every);
  rg_adjoint_state* A = h->adj;
  A->have_forward = false;
  h->dt_next_ready = false;
  MeshSlot* s = active_slot(h);
  const size_t n = static_cast<size_t>(s->n), np = n + static_cast<size_t>(s->g);
  const int n_ckpt = (n_steps + every - 1) / every;
  RG_CUDA(h, A->ckpt_cells.ensure(32 * n * static_cast<size_t>(n_ckpt)));
  RG_CUDA(h, A->ckpt_ext.ensure(32 * n * static_cast<size_t>(n_ckpt)));
  const size_t seg = static_cast<size_t>(std::min(every, n_steps));
  RG_CUDA(h, A->seg_cells.ensure(32 * np * seg));
  RG_CUDA(h, A->seg_ext.ensure(32 * n * seg));
  RG_CUDA(h, A->seg_slopes.ensure(64 * n * seg));
  RG_CUDA(h, A->seg_trace.ensure(sizeof(rg::SlopeTrace) * n * seg));
  RG_TRY(reset_status(h, h->d_status, h->stream));
  rg::StepArgs a = step_args(h);
  a.dt_host = dt;
  if (h->mixed) {
    // U_0 from the FP32 primitives the mixed steps start from
    RG_CUDA(h, rg::launch_cells_to64(static_cast<const float4*>(h->cells32.p), static_cast<double*>(h->cells.p),
                                     s->n, h->stream));
    RG_CUDA(h, rg::launch_init_extensives(a, h->stream));
    const rg::MixedArgs mx = mixed_fixed_dt(h, dt);
    for (int k = 0; k < n_steps; ++k) {
      if (k % every == 0) {
        const size_t c = static_cast<size_t>(k / every);
        RG_CUDA(h, cudaMemcpyAsync(ptr<double>(A->ckpt_cells, 4 * n * c), h->cells32.p, 16 * n,
                                   cudaMemcpyDeviceToDevice, h->stream));
        RG_CUDA(h, cudaMemcpyAsync(ptr<double>(A->ckpt_ext, 4 * n * c), h->ext.p, 32 * n, cudaMemcpyDeviceToDevice,
                                   h->stream));
      }
      rg::MixedArgs mk = mx;
      mk.step = std::min(k, 0x1fff);
      RG_TRY(enqueue_mixed_step(h, mk));
    }
  } else {
    RG_CUDA(h, rg::launch_init_extensives(a, h->stream));
  }
  for (int k = 0; k < (h->mixed ? 0 : n_steps); ++k) {
    if (k % every == 0) {
      const size_t c = static_cast<size_t>(k / every);
      RG_CUDA(h, cudaMemcpyAsync(ptr<double>(A->ckpt_cells, 4 * n * c), h->cells.p, 32 * n, cudaMemcpyDeviceToDevice,
                                 h->stream));
      RG_CUDA(h, cudaMemcpyAsync(ptr<double>(A->ckpt_ext, 4 * n * c), h->ext.p, 32 * n, cudaMemcpyDeviceToDevice,
                                 h->stream));
    }
    a.step = std::min(k, 0x1fff);
    RG_TRY(enqueue_plain_step(h, a));
  }
  RG_CUDA(h, cudaMemcpyAsync(A->final_ext.p, h->ext.p, 32 * n, cudaMemcpyDeviceToDevice, h->stream));
  h->have_ext = true;
  h->have_fluxes = false;
  rg_status st = collect(h, h->d_status, h->stream);
  if (st != RG_OK) return st;
  A->n_steps = n_steps;
  A->every = every;
  A->n_ckpt = n_ckpt;
  A->dt = dt;
  A->have_forward = true;
  return RG_OK;
}

rg_status rg_step_bwd(rg_handle* h, const double* cells_bar, double* cells0_bar) {
  if (!h || !cells_bar || !cells0_bar) return RG_ERR_INVALID_ARGUMENT;
  h->last = rg_error{};
  if (h->active < 0 || !h->adj || !h->adj->have_forward) {
    h->last = rg_error{RG_ERR_NOT_READY, 0, -1, 0};
    return RG_ERR_NOT_READY;
  }
  rg_adjoint_state* A = h->adj;
  MeshSlot* s = active_slot(h);
  const size_t n = static_cast<size_t>(s->n), np = n + static_cast<size_t>(s->g);
  RG_TRY(reset_status(h, h->d_status, h->stream));
  RG_CUDA(h, cudaMemcpyAsync(A->io.p, cells_bar, 32 * n, cudaMemcpyHostToDevice, h->stream));
  rg::AdjArgs base = adj_args(h);
  base.ext = ptr<double>(A->final_ext);
  double* cur = ptr<double>(A->ubar0);
  double* nxt = ptr<double>(A->ubar1);
  RG_CUDA(h, rg::adj_launch_seed(base, ptr<double>(A->io), cur, h->stream));
  rg::StepArgs a = step_args(h);
  a.dt_host = A->dt;
  if (h->mixed) {
    RG_CUDA(h, A->w_cells32.ensure(16 * np));
    RG_CUDA(h, A->w_ext.ensure(32 * n));
  }
  for (int c = A->n_ckpt - 1; c >= 0 && h->mixed; --c) {
    // FP32-mixed: recompute the interval with the mixed kernels, recording
    // each step's state (widened), extensives, FP32 slopes and their trace
    const int start = c * A->every;
    const int len = std::min(A->every, A->n_steps - start);
    RG_CUDA(h, cudaMemcpyAsync(A->w_cells32.p, ptr<double>(A->ckpt_cells, 4 * n * static_cast<size_t>(c)), 16 * n,
                               cudaMemcpyDeviceToDevice, h->stream));
    RG_CUDA(h, cudaMemcpyAsync(A->w_ext.p, ptr<double>(A->ckpt_ext, 4 * n * static_cast<size_t>(c)), 32 * n,
                               cudaMemcpyDeviceToDevice, h->stream));
    rg::MixedArgs mx = mixed_fixed_dt(h, A->dt);
    mx.cells32 = static_cast<float4*>(A->w_cells32.p);
    mx.ext = ptr<double>(A->w_ext);
    for (int j = 0; j < len; ++j) {
      const size_t J = static_cast<size_t>(j);
      RG_CUDA(h, cudaMemcpyAsync(ptr<double>(A->seg_ext, 4 * n * J), A->w_ext.p, 32 * n, cudaMemcpyDeviceToDevice,
                                 h->stream));
      RG_CUDA(h, rg::launch_cells_to64(mx.cells32, ptr<double>(A->seg_cells, 4 * np * J), s->n, h->stream));
      RG_CUDA(h, rg::launch_slopes32_trace(mx, ptr<double>(A->seg_slopes, 8 * n * J),
                                           ptr<rg::SlopeTrace>(A->seg_trace, n * J), h->stream));
      if (j + 1 < len) {
        // the rest of the step: the trace kernel has left the FP32 slopes
        rg::MixedArgs mj = mx;
        mj.step = std::min(start + j, 0x1fff);
        RG_CUDA(h, rg::launch_faces32(mj, h->stream, true));
        RG_CUDA(h, rg::launch_update_mixed(mj, h->stream, false, true, true));
      }
    }
    for (int j = len - 1; j >= 0; --j) {
      const size_t J = static_cast<size_t>(j);
      rg::AdjArgs r = base;
      r.cells = ptr<double>(A->seg_cells, 4 * np * J);
      r.ext = ptr<double>(A->seg_ext, 4 * n * J);
      r.slopes = ptr<double>(A->seg_slopes, 8 * n * J);
      r.trace = ptr<rg::SlopeTrace>(A->seg_trace, n * J);
      const bool first = start + j == 0;
      RG_CUDA(h, rg::adj_launch_reverse32(r, cur, nxt, first ? ptr<double>(A->io) : nullptr, h->stream));
      std::swap(cur, nxt);
    }
  }
  for (int c = h->mixed ? -1 : A->n_ckpt - 1; c >= 0; --c) {
    const int start = c * A->every;
    const int len = std::min(A->every, A->n_steps - start);
    RG_CUDA(h, cudaMemcpyAsync(A->seg_cells.p, ptr<double>(A->ckpt_cells, 4 * n * static_cast<size_t>(c)), 32 * n,
                               cudaMemcpyDeviceToDevice, h->stream));
    RG_CUDA(h, cudaMemcpyAsync(A->seg_ext.p, ptr<double>(A->ckpt_ext, 4 * n * static_cast<size_t>(c)), 32 * n,
                               cudaMemcpyDeviceToDevice, h->stream));
    // recompute the interval: W_j, U_j, slopes and trace of every step in it
    for (int j = 0; j < len; ++j) {
      const size_t J = static_cast<size_t>(j);
      rg::StepArgs aj = a;
      aj.step = std::min(start + j, 0x1fff);
      aj.cells = ptr<double>(A->seg_cells, 4 * np * J);
      aj.ext = ptr<double>(A->seg_ext, 4 * n * J);
      aj.slopes = ptr<double>(A->seg_slopes, 8 * n * J);
      aj.cells_out = ptr<double>(A->seg_cells, 4 * np * (J + 1));
      aj.ext_out = ptr<double>(A->seg_ext, 4 * n * (J + 1));
      RG_CUDA(h, rg::launch_ghost_fill(aj, h->stream));
      rg::AdjArgs r = base;
      r.cells = aj.cells;
      r.slopes = aj.slopes;
      r.trace = ptr<rg::SlopeTrace>(A->seg_trace, n * J);
      RG_CUDA(h, rg::adj_launch_record_slopes(r, h->stream));
      if (j + 1 < len) {
        RG_CUDA(h, rg::launch_faces(aj, h->stream, true));
        RG_CUDA(h, rg::launch_update(aj, h->stream, false, true, true));
      }
    }
    // reverse steps
    for (int j = len - 1; j >= 0; --j) {
      const size_t J = static_cast<size_t>(j);
      rg::AdjArgs r = base;
      r.cells = ptr<double>(A->seg_cells, 4 * np * J);
      r.ext = ptr<double>(A->seg_ext, 4 * n * J);
      r.slopes = ptr<double>(A->seg_slopes, 8 * n * J);
      r.trace = ptr<rg::SlopeTrace>(A->seg_trace, n * J);
      const bool first = start + j == 0;
      RG_CUDA(h, rg::adj_launch_reverse(r, cur, nxt, first ? ptr<double>(A->io) : nullptr, h->stream));
      std::swap(cur, nxt);
    }
  }
  RG_CUDA(h, cudaMemcpyAsync(cells0_bar, A->io.p, 32 * n, cudaMemcpyDeviceToHost, h->stream));
  return collect(h, h->d_status, h->stream);
}

rg_status rg_step_tlm(rg_handle* h, int32_t n_steps, double dt, const double* dcells0, double* dcells) {
  if (!h || !dcells0 || !dcells) return RG_ERR_INVALID_ARGUMENT;
  h->last = rg_error{};
  if (rg_status st = check_run(h, n_steps, dt, false)) return st;  // the tangent-linear model is FP64
  rg_adjoint_state* A = h->adj;
  A->have_forward = false;
  h->dt_next_ready = false;
  MeshSlot* s = active_slot(h);
  const size_t n = static_cast<size_t>(s->n), ne = static_cast<size_t>(std::max(s->e, 1));
  RG_CUDA(h, A->dcells.ensure(32 * n));
  RG_CUDA(h, A->dslopes.ensure(64 * n));
  RG_CUDA(h, A->dflux.ensure(32 * ne));
  RG_CUDA(h, A->dext.ensure(32 * n));
  RG_TRY(reset_status(h, h->d_status, h->stream));
  RG_CUDA(h, cudaMemcpyAsync(A->dcells.p, dcells0, 32 * n, cudaMemcpyHostToDevice, h->stream));
  A->dt = dt;
  rg::AdjArgs t = adj_args(h);
  t.cells = static_cast<const double*>(h->cells.p);
  t.dcells = ptr<double>(A->dcells);
  t.ext_rw = static_cast<double*>(h->ext.p);
  t.dext = ptr<double>(A->dext);
  t.slopes = static_cast<double*>(h->slopes.p);
  t.dslopes = ptr<double>(A->dslopes);
  t.flux = static_cast<double*>(h->fluxes.p);
  t.dflux = ptr<double>(A->dflux);
  t.cells_out = static_cast<double*>(h->cells.p);
  t.dcells_out = ptr<double>(A->dcells);
  RG_CUDA(h, rg::tl_launch_init(t, h->stream));
  for (int k = 0; k < n_steps; ++k) RG_CUDA(h, rg::tl_launch_step(t, h->stream));
  RG_CUDA(h, cudaMemcpyAsync(dcells, A->dcells.p, 32 * n, cudaMemcpyDeviceToHost, h->stream));
  h->have_ext = true;
  h->have_fluxes = false;
  return collect(h, h->d_status, h->stream);
}

}  // extern "C"
