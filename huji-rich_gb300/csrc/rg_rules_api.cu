// rg_rules_api.cu -- C ABI of the condition/action flux schemes
// (include/rich_gb300.h, "Condition/action flux schemes"): the rule table
// of ConditionActionSequence / ConditionActionSequence2
// (condition_action_sequence.cpp, condition_action_sequence_2.cpp) and
// LagrangianExtensiveUpdater (LagrangianExtensiveUpdater.cpp) with its
// LagrangianFlux's per-face data.  The kernels are in rg_fp64.cu
// (k_faces_cas, the update kernel's Lagrangian scaling) and rg_hllc.cuh
// (LagrangianHLLC).
#include <cuda_runtime.h>

#include "rg_handle.cuh"

using namespace rgh;

namespace rgh {

rg_status lagrangian_buffers(rg_handle* h) {
  MeshSlot* s = active_slot(h);
  if (!s || !h->lag_rule) return RG_OK;
  const size_t e = static_cast<size_t>(s->e > 0 ? s->e : 1);
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  const bool fresh = h->lag_ws.bytes < 8 * e;
  RG_CUDA(h, h->lag_ws.ensure(8 * e));
  RG_CUDA(h, h->lag_ev.ensure(8 * e));
  if (fresh) {
    // LagrangianFlux::Reset: every face starts at 0
    RG_CUDA(h, cudaMemset(h->lag_ws.p, 0, 8 * e));
    RG_CUDA(h, cudaMemset(h->lag_ev.p, 0, 8 * e));
  }
  return RG_OK;
}

}  // namespace rgh

extern "C" {

rg_status rg_set_flux_rules(rg_handle* h, int32_t n_rules, const rg_flux_rule* rules) {
  if (!h || n_rules < 0 || (n_rules > 0 && !rules)) return RG_ERR_INVALID_ARGUMENT;
  if (n_rules > RG_MAX_FLUX_RULES) return invalid(h, -1, n_rules);
  if (n_rules > 0 && (h->mixed || h->n_problems > 0)) return invalid(h, -2, 0);
  for (int k = 0; k < n_rules; ++k) {
    const rg_flux_rule& r = rules[k];
    const bool ok = (r.sequence == 0 || r.sequence == 1) && r.condition >= 0 && r.condition <= 2 &&
                    (r.condition != RG_COND_SPECIAL_EDGE || (r.sticker >= 0 && r.sticker < 32)) &&
                    (r.sequence == 0 ? (r.action >= 0 && r.action <= 2) : (r.action >= 3 && r.action <= 6)) &&
                    (r.sequence == 0 || h->cfg.order == 2) && (r.massflux & ~3) == 0;
    if (!ok) return invalid(h, k, r.action);
    if (r.condition == RG_COND_SPECIAL_EDGE && !tracers_on(h)) return invalid(h, k, -1);  // no stickers kept
  }
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  h->n_rules = n_rules;
  h->lag_rule = false;
  for (int k = 0; k < n_rules; ++k) {
    h->rules[k] = rules[k];
    h->lag_rule = h->lag_rule || rules[k].action == RG_ACT_LAGRANGIAN;
  }
  RG_TRY(lagrangian_buffers(h));
  drop_graph(h);
  h->dt_next_ready = false;
  return RG_OK;
}

rg_status rg_set_lagrangian_updater(rg_handle* h, int32_t on) {
  if (!h) return RG_ERR_INVALID_ARGUMENT;
  if (on && (h->mixed || h->n_problems > 0)) return invalid(h, 0, on);
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  h->lag_update = on != 0;
  drop_graph(h);
  return RG_OK;
}

rg_status rg_get_lagrangian_faces(rg_handle* h, double* ws, double* edge_vel) {
  if (rg_status st = require(h, false, false, false, false)) return st;
  if (!h->lag_rule || !h->lag_ws.p) return invalid(h, -1, 0);
  const size_t bytes = 8 * static_cast<size_t>(active_slot(h)->e);
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  if (ws) RG_CUDA(h, cudaMemcpy(ws, h->lag_ws.p, bytes, cudaMemcpyDeviceToHost));
  if (edge_vel) RG_CUDA(h, cudaMemcpy(edge_vel, h->lag_ev.p, bytes, cudaMemcpyDeviceToHost));
  return RG_OK;
}

rg_status rg_set_lagrangian_faces(rg_handle* h, const double* ws, const double* edge_vel) {
  if (rg_status st = require(h, false, false, false, false)) return st;
  if (!h->lag_rule || !h->lag_ws.p || !ws || !edge_vel) return invalid(h, -1, 0);
  const size_t bytes = 8 * static_cast<size_t>(active_slot(h)->e);
  RG_CUDA(h, cudaStreamSynchronize(h->stream));
  RG_CUDA(h, cudaMemcpy(h->lag_ws.p, ws, bytes, cudaMemcpyHostToDevice));
  RG_CUDA(h, cudaMemcpy(h->lag_ev.p, edge_vel, bytes, cudaMemcpyHostToDevice));
  return RG_OK;
}

}  // extern "C"
