// rg_3d_api.cu -- C ABI of the 3D first-order path (rg3_* in
// include/rich_gb300.h): a handle owning the packed 3D mesh (validated on the
// device before use), the cell / extensive state and the face fluxes, all on
// one stream.  Host records of 5 doubles are moved to and from the device's
// 48-byte records with pitched copies.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "rg_3d.cuh"

using rg::DevStatus;

namespace {

struct Buf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t want) {
    if (want <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    const cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) bytes = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};

}  // namespace

struct rg3_handle {
  rg_config cfg{};
  cudaStream_t stream = nullptr;
  int n = 0, e = 0, m = 0;
  bool have_mesh = false, have_cells = false, have_ext = false, have_fluxes = false;
  Buf face_cells, normal, area, volume, width, cell_off, cell_faces, nhat, fsign;
  Buf cells, ext, fluxes, fvel, status_buf;
  bool fvel_set = false;
  // FP32-mixed path (rg_config.precision == RG_FP32_MIXED)
  bool mixed = false;
  Buf nhat32, area32, width32, cells32, vz32, flux32, fen32, fvel32;
  DevStatus* d_status = nullptr;
  DevStatus* h_status = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  rg_error last{};
};

namespace {

rg_status fail(rg3_handle* h, cudaError_t e) {
  if (h) h->last = rg_error{RG_ERR_CUDA, 0, static_cast<int64_t>(e), 0.0};
  cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? RG_ERR_OUT_OF_MEMORY : RG_ERR_CUDA;
}

#define RG3_CUDA(h, call)                         \
  do {                                            \
    const cudaError_t e_ = (call);                \
    if (e_ != cudaSuccess) return fail((h), e_);  \
  } while (0)

rg_status not_ready(rg3_handle* h) {
  h->last = rg_error{RG_ERR_NOT_READY, 0, -1, 0};
  return RG_ERR_NOT_READY;
}

rg_status reset(rg3_handle* h) {
  RG3_CUDA(h, cudaMemsetAsync(&h->d_status->err_key, 0xff, sizeof(unsigned long long), h->stream));
  RG3_CUDA(h, cudaMemsetAsync(&h->d_status->err_status, 0, 2 * sizeof(int), h->stream));
  return RG_OK;
}

rg_status collect(rg3_handle* h, double* dt = nullptr) {
  RG3_CUDA(h, cudaMemcpyAsync(h->h_status, h->d_status, sizeof(DevStatus), cudaMemcpyDeviceToHost, h->stream));
  RG3_CUDA(h, cudaStreamSynchronize(h->stream));
  RG3_CUDA(h, cudaGetLastError());
  if (dt) *dt = h->h_status->dt;
  if (h->h_status->err_key != ~0ull) {
    const unsigned long long key = h->h_status->err_key;
    h->last = rg_error{h->h_status->err_status, static_cast<int32_t>((key >> rg::kKeyPhaseShift) & 0xf),
                       static_cast<int64_t>(key & rg::kKeyIndexMask), h->h_status->err_value};
    if (h->last.status == 0) h->last.status = RG_ERR_CUDA;
    return static_cast<rg_status>(h->last.status);
  }
  return RG_OK;
}

rg::Step3Args args(rg3_handle* h) {
  rg::Step3Args a{};
  a.mesh.n = h->n;
  a.mesh.e = h->e;
  a.mesh.m = h->m;
  a.mesh.face_cells = static_cast<const int2*>(h->face_cells.p);
  a.mesh.normal = static_cast<const double*>(h->normal.p);
  a.mesh.area = static_cast<const double*>(h->area.p);
  a.mesh.volume = static_cast<const double*>(h->volume.p);
  a.mesh.width = static_cast<const double*>(h->width.p);
  a.mesh.cell_off = static_cast<const int*>(h->cell_off.p);
  a.mesh.cell_faces = static_cast<const int*>(h->cell_faces.p);
  a.nhat = static_cast<const rg::dbl4*>(h->nhat.p);
  a.fsign = static_cast<const int*>(h->fsign.p);
  a.gamma = h->cfg.gamma;
  a.cfl = h->cfg.cfl;
  a.cells = static_cast<double*>(h->cells.p);
  a.ext = static_cast<double*>(h->ext.p);
  a.fluxes = static_cast<double*>(h->fluxes.p);
  a.fvel = h->fvel_set ? static_cast<const double*>(h->fvel.p) : nullptr;
  a.status = h->d_status;
  return a;
}

rg::Mixed3Args margs(rg3_handle* h) {
  const rg::Step3Args b = args(h);
  rg::Mixed3Args a{};
  a.mesh = b.mesh;
  a.fsign = b.fsign;
  a.nhat32 = static_cast<const float4*>(h->nhat32.p);
  a.area32 = static_cast<const float*>(h->area32.p);
  a.width32 = static_cast<const float*>(h->width32.p);
  a.gamma = static_cast<float>(h->cfg.gamma);
  a.cfl = h->cfg.cfl;
  a.cells32 = static_cast<float4*>(h->cells32.p);
  a.vz32 = static_cast<float*>(h->vz32.p);
  a.ext = static_cast<double*>(h->ext.p);
  a.flux32 = static_cast<float4*>(h->flux32.p);
  a.fen32 = static_cast<float*>(h->fen32.p);
  a.fvel = h->fvel_set ? static_cast<const float*>(h->fvel32.p) : nullptr;
  a.status = h->d_status;
  return a;
}

// the FP64 cell records from the FP32 ones (mixed path, before they are read)
rg_status sync_cells64(rg3_handle* h) {
  if (h->mixed)
    RG3_CUDA(h, rg::launch3m_cells_to64(static_cast<const float4*>(h->cells32.p), static_cast<const float*>(h->vz32.p),
                                        static_cast<double*>(h->cells.p), h->n, h->stream));
  return RG_OK;
}

// 5-double host records <-> 6-double device records
rg_status put5(rg3_handle* h, Buf& dst, const double* src, int rows) {
  RG3_CUDA(h, cudaMemcpy2DAsync(dst.p, 48, src, 40, 40, static_cast<size_t>(rows), cudaMemcpyHostToDevice,
                                h->stream));
  RG3_CUDA(h, cudaStreamSynchronize(h->stream));
  return RG_OK;
}
rg_status get5(rg3_handle* h, double* dst, const Buf& src, int rows) {
  RG3_CUDA(h, cudaMemcpy2DAsync(dst, 40, src.p, 48, 40, static_cast<size_t>(rows), cudaMemcpyDeviceToHost,
                                h->stream));
  RG3_CUDA(h, cudaStreamSynchronize(h->stream));
  return RG_OK;
}

rg_status enqueue_step(rg3_handle* h, int step, bool timed = false) {
  if (timed) RG3_CUDA(h, cudaEventRecord(h->ev[0], h->stream));
  if (h->mixed) {
    rg::Mixed3Args a = margs(h);
    a.dt_from_device = 1;
    a.step = step;
    RG3_CUDA(h, rg::launch3m_cfl(a, h->stream));
    if (timed) RG3_CUDA(h, cudaEventRecord(h->ev[1], h->stream));
    RG3_CUDA(h, rg::launch3m_faces(a, true, h->stream));
    if (timed) RG3_CUDA(h, cudaEventRecord(h->ev[2], h->stream));
    RG3_CUDA(h, rg::launch3m_update(a, false, true, true, h->stream));
  } else {
    rg::Step3Args a = args(h);
    a.dt_from_device = 1;
    a.step = step;
    RG3_CUDA(h, rg::launch3_cfl(a, h->stream));
    if (timed) RG3_CUDA(h, cudaEventRecord(h->ev[1], h->stream));
    RG3_CUDA(h, rg::launch3_faces(a, true, h->stream));
    if (timed) RG3_CUDA(h, cudaEventRecord(h->ev[2], h->stream));
    RG3_CUDA(h, rg::launch3_update(a, false, true, true, h->stream));
  }
  if (timed) RG3_CUDA(h, cudaEventRecord(h->ev[3], h->stream));
  h->have_fluxes = false;
  return RG_OK;
}

}  // namespace

extern "C" {

rg_status rg3_create(const rg_config* cfg, rg3_handle** out) {
  if (!cfg || !out) return RG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (!(cfg->gamma > 1.0) || !(cfg->cfl > 0.0)) return RG_ERR_INVALID_ARGUMENT;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || cfg->device < 0 || cfg->device >= ndev) {
    cudaGetLastError();
    return RG_ERR_CUDA;
  }
  if (cfg->precision != RG_FP64 && cfg->precision != RG_FP32_MIXED) return RG_ERR_INVALID_ARGUMENT;
  rg3_handle* h = new (std::nothrow) rg3_handle();
  if (!h) return RG_ERR_OUT_OF_MEMORY;
  h->cfg = *cfg;
  h->mixed = cfg->precision == RG_FP32_MIXED;
  cudaError_t e;
  if ((e = cudaSetDevice(cfg->device)) != cudaSuccess || (e = cudaStreamCreateWithFlags(&h->stream,
                                                                                         cudaStreamNonBlocking)) !=
                                                             cudaSuccess ||
      (e = h->status_buf.ensure(sizeof(DevStatus))) != cudaSuccess ||
      (e = cudaMallocHost(&h->h_status, sizeof(DevStatus))) != cudaSuccess ||
      (e = cudaEventCreate(&h->ev[0])) != cudaSuccess || (e = cudaEventCreate(&h->ev[1])) != cudaSuccess ||
      (e = cudaEventCreate(&h->ev[2])) != cudaSuccess || (e = cudaEventCreate(&h->ev[3])) != cudaSuccess) {
    rg3_destroy(h);
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? RG_ERR_OUT_OF_MEMORY : RG_ERR_CUDA;
  }
  h->d_status = static_cast<DevStatus*>(h->status_buf.p);
  DevStatus init{};
  init.err_key = ~0ull;
  init.dt_min_bits = rg::kInfBits;
  if ((e = cudaMemcpy(h->d_status, &init, sizeof init, cudaMemcpyHostToDevice)) != cudaSuccess) {
    rg3_destroy(h);
    return RG_ERR_CUDA;
  }
  *out = h;
  return RG_OK;
}

rg_status rg3_destroy(rg3_handle* h) {
  if (!h) return RG_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (Buf* b : {&h->face_cells, &h->normal, &h->area, &h->volume, &h->width, &h->cell_off, &h->cell_faces,
                 &h->nhat, &h->fsign, &h->cells, &h->ext, &h->fluxes, &h->fvel, &h->status_buf, &h->nhat32,
                 &h->area32, &h->width32, &h->cells32, &h->vz32, &h->flux32, &h->fen32, &h->fvel32})
    b->release();
  if (h->h_status) cudaFreeHost(h->h_status);
  for (cudaEvent_t& v : h->ev)
    if (v) cudaEventDestroy(v);
  if (h->stream) cudaStreamDestroy(h->stream);
  cudaGetLastError();
  delete h;
  return RG_OK;
}

rg_status rg3_last_error(const rg3_handle* h, rg_error* err) {
  if (!h || !err) return RG_ERR_INVALID_ARGUMENT;
  *err = h->last;
  return RG_OK;
}

rg_status rg3_upload_mesh(rg3_handle* h, const rg_mesh3d_view* v) {
  if (!h) return RG_ERR_INVALID_ARGUMENT;
  h->last = rg_error{};
  auto bad = [h](int64_t idx) {
    h->last = rg_error{RG_ERR_INVALID_ARGUMENT, 0, idx, 0};
    return RG_ERR_INVALID_ARGUMENT;
  };
  if (!v || v->n_cells <= 0 || v->n_faces <= 0) return bad(-1);
  if (!v->face_cells || !v->face_normal || !v->face_area || !v->volume || !v->width || !v->cell_face_offset ||
      !v->cell_faces)
    return bad(-3);
  const int n = v->n_cells, e = v->n_faces, m = v->cell_face_offset[n];
  if (v->cell_face_offset[0] != 0 || m < 0 || m > 2 * e) return bad(-4);
  RG3_CUDA(h, cudaSetDevice(h->cfg.device));
  RG3_CUDA(h, cudaStreamSynchronize(h->stream));
  const size_t N = static_cast<size_t>(n), E = static_cast<size_t>(e), M = static_cast<size_t>(std::max(m, 1));
  RG3_CUDA(h, h->face_cells.ensure(8 * E));
  RG3_CUDA(h, h->normal.ensure(24 * E));
  RG3_CUDA(h, h->area.ensure(8 * E));
  RG3_CUDA(h, h->volume.ensure(8 * N));
  RG3_CUDA(h, h->width.ensure(8 * N));
  RG3_CUDA(h, h->cell_off.ensure(4 * (N + 1)));
  RG3_CUDA(h, h->cell_faces.ensure(4 * M));
  RG3_CUDA(h, h->nhat.ensure(32 * E));
  RG3_CUDA(h, h->fsign.ensure(4 * M));
  RG3_CUDA(h, h->fluxes.ensure(48 * E));
  RG3_CUDA(h, h->fvel.ensure(24 * E));
  if (n != h->n) h->have_cells = h->have_ext = false;
  RG3_CUDA(h, h->cells.ensure(48 * N));
  RG3_CUDA(h, h->ext.ensure(48 * N));
  RG3_CUDA(h, cudaMemcpyAsync(h->face_cells.p, v->face_cells, 8 * E, cudaMemcpyHostToDevice, h->stream));
  RG3_CUDA(h, cudaMemcpyAsync(h->normal.p, v->face_normal, 24 * E, cudaMemcpyHostToDevice, h->stream));
  RG3_CUDA(h, cudaMemcpyAsync(h->area.p, v->face_area, 8 * E, cudaMemcpyHostToDevice, h->stream));
  RG3_CUDA(h, cudaMemcpyAsync(h->volume.p, v->volume, 8 * N, cudaMemcpyHostToDevice, h->stream));
  RG3_CUDA(h, cudaMemcpyAsync(h->width.p, v->width, 8 * N, cudaMemcpyHostToDevice, h->stream));
  RG3_CUDA(h, cudaMemcpyAsync(h->cell_off.p, v->cell_face_offset, 4 * (N + 1), cudaMemcpyHostToDevice, h->stream));
  if (m > 0)
    RG3_CUDA(h, cudaMemcpyAsync(h->cell_faces.p, v->cell_faces, 4 * static_cast<size_t>(m), cudaMemcpyHostToDevice,
                                h->stream));
  h->n = n;
  h->e = e;
  h->m = m;
  h->fvel_set = false;
  h->have_fluxes = false;
  rg::Step3Args a = args(h);
  if (rg_status st = reset(h)) return st;
  RG3_CUDA(h, rg::launch3_validate(a.mesh, h->d_status, h->stream));
  if (collect(h) != RG_OK) {
    h->have_mesh = false;
    h->last.status = RG_ERR_INVALID_ARGUMENT;
    return RG_ERR_INVALID_ARGUMENT;
  }
  RG3_CUDA(h, rg::launch3_geometry(a.mesh, static_cast<rg::dbl4*>(h->nhat.p), static_cast<int*>(h->fsign.p),
                                   h->stream));
  if (h->mixed) {
    RG3_CUDA(h, h->nhat32.ensure(16 * E));
    RG3_CUDA(h, h->area32.ensure(4 * E));
    RG3_CUDA(h, h->width32.ensure(4 * N));
    RG3_CUDA(h, h->cells32.ensure(16 * N));
    RG3_CUDA(h, h->vz32.ensure(4 * N));
    RG3_CUDA(h, h->flux32.ensure(16 * E));
    RG3_CUDA(h, h->fen32.ensure(4 * E));
    RG3_CUDA(h, h->fvel32.ensure(12 * E));
    RG3_CUDA(h, rg::launch3m_geometry(a.mesh, static_cast<const rg::dbl4*>(h->nhat.p),
                                      static_cast<float4*>(h->nhat32.p), static_cast<float*>(h->area32.p),
                                      static_cast<float*>(h->width32.p), h->stream));
  }
  RG3_CUDA(h, cudaStreamSynchronize(h->stream));
  h->have_mesh = true;
  return RG_OK;
}

rg_status rg3_set_cells(rg3_handle* h, const double* cells) {
  if (!h || !cells) return RG_ERR_INVALID_ARGUMENT;
  if (!h->have_mesh) return not_ready(h);
  if (rg_status st = put5(h, h->cells, cells, h->n)) return st;
  if (h->mixed) {
    RG3_CUDA(h, rg::launch3m_cells_to32(static_cast<const double*>(h->cells.p), static_cast<float4*>(h->cells32.p),
                                        static_cast<float*>(h->vz32.p), h->n, h->stream));
    RG3_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  h->have_cells = true;
  return RG_OK;
}

rg_status rg3_get_cells(rg3_handle* h, double* cells) {
  if (!h || !cells) return RG_ERR_INVALID_ARGUMENT;
  if (!h->have_cells) return not_ready(h);
  if (rg_status st = sync_cells64(h)) return st;
  return get5(h, cells, h->cells, h->n);
}

rg_status rg3_set_extensives(rg3_handle* h, const double* ext) {
  if (!h || !ext) return RG_ERR_INVALID_ARGUMENT;
  if (!h->have_mesh) return not_ready(h);
  if (rg_status st = put5(h, h->ext, ext, h->n)) return st;
  h->have_ext = true;
  return RG_OK;
}

rg_status rg3_get_extensives(rg3_handle* h, double* ext) {
  if (!h || !ext) return RG_ERR_INVALID_ARGUMENT;
  if (!h->have_ext) return not_ready(h);
  return get5(h, ext, h->ext, h->n);
}

rg_status rg3_set_face_velocities(rg3_handle* h, const double* fv) {
  if (!h) return RG_ERR_INVALID_ARGUMENT;
  if (!h->have_mesh) return not_ready(h);
  h->fvel_set = fv != nullptr;
  if (fv) {
    RG3_CUDA(h, cudaMemcpyAsync(h->fvel.p, fv, 24 * static_cast<size_t>(h->e), cudaMemcpyHostToDevice, h->stream));
    if (h->mixed)
      RG3_CUDA(h, rg::launch3m_d2f(static_cast<const double*>(h->fvel.p), static_cast<float*>(h->fvel32.p), 3 * h->e,
                                   h->stream));
    RG3_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  return RG_OK;
}

rg_status rg3_init_extensives(rg3_handle* h) {
  if (!h) return RG_ERR_INVALID_ARGUMENT;
  if (!h->have_cells) return not_ready(h);
  if (rg_status st = sync_cells64(h)) return st;
  RG3_CUDA(h, rg::launch3_init_extensives(args(h), h->stream));
  RG3_CUDA(h, cudaStreamSynchronize(h->stream));
  h->have_ext = true;
  return RG_OK;
}

rg_status rg3_cfl_dt(rg3_handle* h, double* dt) {
  if (!h || !dt) return RG_ERR_INVALID_ARGUMENT;
  if (!h->have_cells) return not_ready(h);
  h->last = rg_error{};
  if (rg_status st = reset(h)) return st;
  if (h->mixed)
    RG3_CUDA(h, rg::launch3m_cfl(margs(h), h->stream));
  else
    RG3_CUDA(h, rg::launch3_cfl(args(h), h->stream));
  return collect(h, dt);
}

rg_status rg3_flux(rg3_handle* h, double* fluxes_out) {
  if (!h) return RG_ERR_INVALID_ARGUMENT;
  if (!h->have_cells) return not_ready(h);
  h->last = rg_error{};
  if (rg_status st = reset(h)) return st;
  if (h->mixed)
    RG3_CUDA(h, rg::launch3m_faces(margs(h), false, h->stream));
  else
    RG3_CUDA(h, rg::launch3_faces(args(h), false, h->stream));
  if (rg_status st = collect(h)) return st;
  h->have_fluxes = true;
  if (!fluxes_out) return RG_OK;
  if (h->mixed)
    RG3_CUDA(h, rg::launch3m_flux_to64(static_cast<const float4*>(h->flux32.p), static_cast<const float*>(h->fen32.p),
                                       static_cast<double*>(h->fluxes.p), h->e, h->stream));
  return get5(h, fluxes_out, h->fluxes, h->e);
}

rg_status rg3_extensive_update(rg3_handle* h, double dt) {
  if (!h) return RG_ERR_INVALID_ARGUMENT;
  if (!h->have_ext || !h->have_fluxes) return not_ready(h);
  h->last = rg_error{};
  if (rg_status st = reset(h)) return st;
  if (h->mixed) {
    rg::Mixed3Args a = margs(h);
    a.dt32 = static_cast<float>(dt);
    RG3_CUDA(h, rg::launch3m_update(a, true, true, false, h->stream));
  } else {
    rg::Step3Args a = args(h);
    a.dt_host = dt;
    RG3_CUDA(h, rg::launch3_update(a, true, true, false, h->stream));
  }
  return collect(h);
}

rg_status rg3_cell_update(rg3_handle* h) {
  if (!h) return RG_ERR_INVALID_ARGUMENT;
  if (!h->have_ext) return not_ready(h);
  h->last = rg_error{};
  if (rg_status st = reset(h)) return st;
  if (h->mixed)
    RG3_CUDA(h, rg::launch3m_update(margs(h), false, false, true, h->stream));
  else
    RG3_CUDA(h, rg::launch3_update(args(h), false, false, true, h->stream));
  const rg_status st = collect(h);
  if (st == RG_OK) h->have_cells = true;
  return st;
}

rg_status rg3_step(rg3_handle* h, double* dt_out) {
  if (!h) return RG_ERR_INVALID_ARGUMENT;
  if (!h->have_cells || !h->have_ext) return not_ready(h);
  h->last = rg_error{};
  if (rg_status st = reset(h)) return st;
  if (rg_status st = enqueue_step(h, 0)) return st;
  return collect(h, dt_out);
}

rg_status rg3_step_timed(rg3_handle* h, double* dt_out, float* kernel_ms) {
  if (!h || !kernel_ms) return RG_ERR_INVALID_ARGUMENT;
  if (!h->have_cells || !h->have_ext) return not_ready(h);
  h->last = rg_error{};
  if (rg_status st = reset(h)) return st;
  if (rg_status st = enqueue_step(h, 0, true)) return st;
  const rg_status st = collect(h, dt_out);
  for (int k = 0; k < 3; ++k) {
    kernel_ms[k] = 0;
    RG3_CUDA(h, cudaEventElapsedTime(&kernel_ms[k], h->ev[k], h->ev[k + 1]));
  }
  return st;
}

rg_status rg3_run(rg3_handle* h, int32_t n_steps, double* dts) {
  if (!h || n_steps < 0) return RG_ERR_INVALID_ARGUMENT;
  if (!h->have_cells || !h->have_ext) return not_ready(h);
  h->last = rg_error{};
  if (rg_status st = reset(h)) return st;
  std::vector<double> hd;
  double* pinned = nullptr;
  if (dts && n_steps > 0) RG3_CUDA(h, cudaMallocHost(&pinned, sizeof(double) * static_cast<size_t>(n_steps)));
  rg_status st = RG_OK;
  for (int k = 0; k < n_steps && st == RG_OK; ++k) {
    st = enqueue_step(h, std::min(k, 0x1fff));
    if (st == RG_OK && pinned) {
      const cudaError_t ce = cudaMemcpyAsync(pinned + k, &h->d_status->dt, sizeof(double), cudaMemcpyDeviceToHost,
                                             h->stream);
      if (ce != cudaSuccess) st = fail(h, ce);
    }
  }
  if (st == RG_OK) st = collect(h);
  if (pinned) {
    cudaStreamSynchronize(h->stream);
    if (dts) std::memcpy(dts, pinned, sizeof(double) * static_cast<size_t>(n_steps));
    cudaFreeHost(pinned);
  }
  return st;
}

}  // extern "C"
