// rg_tune.cu -- launch shapes of the per-step kernels and the autotuner
// (rg_autotune, rg_set_launch_shapes, rg_get_launch_shapes).
//
// Candidates per kernel: 64, 128, 256 or 512 threads per block, times one
// thread per item or a persistent grid of 2, 4 or 8 blocks per SM, times the
// kernel's builds (the slopes kernels and the FP32-mixed update kernel also
// have register-capped builds for blocks of up to 256 threads; the FP32-mixed
// slopes kernel a build with its neighbour loops unrolled by two and one
// that loads the neighbour data up front; the FP32-mixed face kernel one
// or two threads per face).  Each
// candidate runs `reps` launches on the handle's stream, on the uploaded mesh
// and the current state, each timed alone with CUDA events after a write of
// a buffer larger than L2 (a kernel of a step finds most of its inputs in
// HBM, not in a warm L2); the mean is compared.  The update kernel writes to
// scratch buffers, and the per-problem dt / time arrays of a batch are saved
// and restored, so the state is unchanged.
#include <cuda_runtime.h>

#include <cstring>

#include "rg_handle.cuh"

using namespace rgh;

namespace {

constexpr int kBlocks[] = {64, 128, 256, 512};
constexpr size_t kFlushBytes = size_t(256) << 20;  // > 129 MB of L2
constexpr int kPerSm[] = {0, 2, 4, 8};

rg::LaunchShape* slot(rg::StepShapes& s, int k) {
  switch (k) {
    case RG_KERNEL_CFL: return &s.cfl;
    case RG_KERNEL_SLOPES: return &s.slopes;
    case RG_KERNEL_FACES: return &s.faces;
    default: return &s.update;
  }
}

rg::StepShapes& path_shapes(rg_handle* h) { return h->mixed ? h->shapes32 : h->shapes64; }

void to_c(const rg::StepShapes& s, rg_launch_shapes* out) {
  rg::StepShapes c = s;
  for (int k = 0; k < 4; ++k) {
    out->block[k] = slot(c, k)->block;
    out->max_blocks[k] = slot(c, k)->max_blocks;
    out->variant[k] = slot(c, k)->variant;
  }
}

// One launch of kernel k of the handle's path with shape `sh`.  Scratch
// outputs for the update: ext_scr (4n doubles), cells_scr (n+g records).
rg_status launch_one(rg_handle* h, int k, const rg::LaunchShape& sh, void* ext_scr, void* cells_scr) {
  const bool o2 = h->cfg.order == 2;
  if (h->mixed) {
    rg::MixedArgs a = mixed_args(h);
    *slot(a.shapes, k) = sh;
    a.dt32_from_device = 1;
    switch (k) {
      case RG_KERNEL_CFL: RG_CUDA(h, rg::launch_cfl32(a, h->stream, o2)); break;
      case RG_KERNEL_SLOPES: if (o2) RG_CUDA(h, rg::launch_slopes32(a, h->stream)); break;
      case RG_KERNEL_FACES: RG_CUDA(h, rg::launch_faces32(a, h->stream, true)); break;
      default:
        a.ext_out = static_cast<double*>(ext_scr);
        a.cells32_out = static_cast<float4*>(cells_scr);
        RG_CUDA(h, rg::launch_update_mixed(a, h->stream, false, true, true));
    }
  } else {
    rg::StepArgs a = step_args(h);
    *slot(a.shapes, k) = sh;
    a.dt_from_device = 1;
    switch (k) {
      case RG_KERNEL_CFL: RG_CUDA(h, rg::launch_cfl(a, h->stream, o2)); break;
      case RG_KERNEL_SLOPES: if (o2) RG_CUDA(h, rg::launch_slopes(a, h->stream)); break;
      case RG_KERNEL_FACES: RG_CUDA(h, rg::launch_faces(a, h->stream, true)); break;
      default:
        a.ext_out = static_cast<double*>(ext_scr);
        a.cells_out = static_cast<double*>(cells_scr);
        RG_CUDA(h, rg::launch_update(a, h->stream, false, true, true));
    }
  }
  return RG_OK;
}

// Builds of kernel k on the handle's path: mixed slopes 0-4; mixed update 0,
// 2, 3 (register-capped); mixed faces 0, 1 (two threads per face); FP64
// slopes 0, 2, 3 (register-capped); otherwise 0.
bool has_build(const rg_handle* h, int k, int v) {
  if (v == 0) return true;
  if (k == RG_KERNEL_SLOPES) return h->mixed ? v >= 1 && v <= 4 : v == 2 || v == 3;
  if (k == RG_KERNEL_UPDATE) return h->mixed && (v == 2 || v == 3);
  if (k == RG_KERNEL_FACES) return h->mixed && v == 1;
  return false;
}
constexpr int kMaxVariant = 4;
bool capped(int k, int v) { return (k == RG_KERNEL_SLOPES || k == RG_KERNEL_UPDATE) && (v == 2 || v == 3); }

rg_status check_shapes(rg_handle* h, const rg_launch_shapes* s) {
  for (int k = 0; k < 4; ++k) {
    const int b = s->block[k], v = s->variant[k];
    if (b < 32 || b > rg::kMaxBlock || b % 32 != 0 || s->max_blocks[k] < 0) return invalid(h, k, b);
    if (v < 0 || !has_build(h, k, v) || (capped(k, v) && b > rg::kCappedBlock)) return invalid(h, k, v);
  }
  return RG_OK;
}

}  // namespace

extern "C" {

rg_status rg_set_launch_shapes(rg_handle* h, const rg_launch_shapes* s) {
  if (!h || !s) return RG_ERR_INVALID_ARGUMENT;
  h->last = rg_error{};
  if (rg_status st = check_shapes(h, s)) return st;
  rg::StepShapes& dst = path_shapes(h);
  for (int k = 0; k < 4; ++k) *slot(dst, k) = rg::LaunchShape{s->block[k], s->max_blocks[k], s->variant[k]};
  drop_graph(h);
  return RG_OK;
}

rg_status rg_get_launch_shapes(const rg_handle* h, rg_launch_shapes* s) {
  if (!h || !s) return RG_ERR_INVALID_ARGUMENT;
  std::memset(s, 0, sizeof *s);
  to_c(h->mixed ? h->shapes32 : h->shapes64, s);
  return RG_OK;
}

rg_status rg_autotune(rg_handle* h, int32_t reps, rg_launch_shapes* chosen) {
  if (rg_status st = require(h, true, true, true, false)) return st;
  if (reps < 1) return invalid(h, -1, reps);
  if (rg_status st = mesh_error(h)) return st;
  h->last = rg_error{};
  MeshSlot* s = active_slot(h);
  int dev = 0, sms = 0;
  RG_CUDA(h, cudaGetDevice(&dev));
  RG_CUDA(h, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const size_t n = static_cast<size_t>(s->n), np = n + static_cast<size_t>(s->g);
  DevBuf ext_scr, cells_scr, saved, flush;
  RG_CUDA(h, flush.ensure(kFlushBytes));
  RG_CUDA(h, ext_scr.ensure(32 * n));
  RG_CUDA(h, cells_scr.ensure(32 * np));
  const size_t P = static_cast<size_t>(h->n_problems);
  if (P) {
    RG_CUDA(h, saved.ensure(24 * P));
    char* b = static_cast<char*>(saved.p);
    RG_CUDA(h, cudaMemcpyAsync(b, h->dtmin_p.p, 8 * P, cudaMemcpyDeviceToDevice, h->stream));
    RG_CUDA(h, cudaMemcpyAsync(b + 8 * P, h->time_p.p, 8 * P, cudaMemcpyDeviceToDevice, h->stream));
    RG_CUDA(h, cudaMemcpyAsync(b + 16 * P, h->dt_p.p, 8 * P, cudaMemcpyDeviceToDevice, h->stream));
  }
  RG_TRY(reset_status(h, h->d_status, h->stream));
  cudaEvent_t e0 = h->ev_k[0], e1 = h->ev_k[1];
  rg::StepShapes& cur = path_shapes(h);
  rg_launch_shapes out{};
  // inputs of every kernel first: ghosts and dt (CFL), slopes, fluxes
  for (int k = 0; k < 3; ++k) RG_TRY(launch_one(h, k, *slot(cur, k), ext_scr.p, cells_scr.p));
  for (int k = 0; k < 4; ++k) {
    float best = 0;
    rg::LaunchShape best_shape = *slot(cur, k);
    for (int v = 0; v <= kMaxVariant; ++v)
    for (int b : kBlocks) {
      if (!has_build(h, k, v) || (capped(k, v) && b > rg::kCappedBlock)) continue;
      for (int per_sm : kPerSm) {
        const rg::LaunchShape sh{b, per_sm * sms, v};
        RG_TRY(launch_one(h, k, sh, ext_scr.p, cells_scr.p));  // warm
        float ms = 0;
        for (int r = 0; r < reps; ++r) {
          RG_CUDA(h, cudaMemsetAsync(flush.p, r & 0xff, kFlushBytes, h->stream));
          RG_CUDA(h, cudaEventRecord(e0, h->stream));
          RG_TRY(launch_one(h, k, sh, ext_scr.p, cells_scr.p));
          RG_CUDA(h, cudaEventRecord(e1, h->stream));
          RG_CUDA(h, cudaEventSynchronize(e1));
          float one = 0;
          RG_CUDA(h, cudaEventElapsedTime(&one, e0, e1));
          ms += one;
        }
        ms /= static_cast<float>(reps);
        if (best == 0 || ms < best) {
          best = ms;
          best_shape = sh;
        }
      }
    }
    *slot(cur, k) = best_shape;
    out.ms[k] = best;
  }
  if (P) {
    char* b = static_cast<char*>(saved.p);
    RG_CUDA(h, cudaMemcpyAsync(h->dtmin_p.p, b, 8 * P, cudaMemcpyDeviceToDevice, h->stream));
    RG_CUDA(h, cudaMemcpyAsync(h->time_p.p, b + 8 * P, 8 * P, cudaMemcpyDeviceToDevice, h->stream));
    RG_CUDA(h, cudaMemcpyAsync(h->dt_p.p, b + 16 * P, 8 * P, cudaMemcpyDeviceToDevice, h->stream));
  }
  rg_status st = collect(h, h->d_status, h->stream);
  ext_scr.release();
  cells_scr.release();
  saved.release();
  flush.release();
  h->have_fluxes = false;  // the flux buffer holds scaled fluxes of the tuning runs
  drop_graph(h);
  to_c(cur, &out);
  if (chosen) *chosen = out;
  return st;
}

}  // extern "C"
