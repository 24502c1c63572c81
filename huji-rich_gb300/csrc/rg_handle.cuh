// rg_handle.cuh -- the handle behind the C ABI and the host helpers shared
// by the translation units that drive it (rg_capi.cu: mesh, state, plugin
// operations, batch; rg_adjoint_api.cu: differentiation).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "rg_internal.cuh"
#include "rg_mixed.cuh"

namespace rgh {


constexpr size_t kAlign = 256;
inline size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t want) {
    if (want <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) bytes = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};

struct HostBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t want) {
    if (want <= bytes) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaHostAlloc(&p, want, cudaHostAllocDefault);
    if (e == cudaSuccess) bytes = want;
    return e;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
  }
};

// Offsets of every array of one mesh slot inside one allocation.  The input
// arrays come first and form one contiguous block, mirrored byte for byte by
// the pinned staging buffer so that one copy moves the whole mesh.
struct SlotLayout {
  size_t points, cms, volume, cd_volume, ghost_source, ghost_face, face_cells, face_vertices, cell_off,
      cell_faces, input_end;
  size_t area, nrm, nabs, par, dm0, dm1, dab, rij, cij, xarea, width, minv, cflags, nbr, hr, ghost_real,
      ghost_unit, cell_order;
  size_t nrm32, nabs32, par32, area32, xarea32, dm0_32, dm1_32, width32, minv32, ent32, fsign32, gunit32, icdv32,
      frec32, total;
  bool own_xarea = false;  // a non-slab PhysicalGeometry: CacheData areas differ from the edge lengths
  void compute(int n, int g, int e, int m, bool mixed, bool cyl = false) {
    own_xarea = cyl;
    const size_t np = static_cast<size_t>(n) + g;
    size_t o = 0;
    auto take = [&o](size_t bytes) {
      const size_t at = o;
      o = align_up(o + bytes);
      return at;
    };
    points = take(16 * np);
    cms = take(16 * np);
    volume = take(8 * static_cast<size_t>(n));
    cd_volume = take(8 * static_cast<size_t>(n));
    ghost_source = take(4 * static_cast<size_t>(g));
    ghost_face = take(4 * static_cast<size_t>(g));
    face_cells = take(8 * static_cast<size_t>(e));
    face_vertices = take(32 * static_cast<size_t>(e));
    cell_off = take(4 * (static_cast<size_t>(n) + 1));
    cell_faces = take(4 * static_cast<size_t>(m));
    input_end = o;
    area = take(8 * static_cast<size_t>(e));
    nrm = take(16 * static_cast<size_t>(e));
    nabs = take(8 * static_cast<size_t>(e));
    par = take(16 * static_cast<size_t>(e));
    dm0 = take(16 * static_cast<size_t>(e));
    dm1 = take(16 * static_cast<size_t>(e));
    dab = take(8 * static_cast<size_t>(e));
    rij = take(16 * static_cast<size_t>(e));
    cij = take(16 * static_cast<size_t>(e));
    xarea = take(cyl ? 8 * static_cast<size_t>(e) : 0);
    width = take(8 * static_cast<size_t>(n));
    minv = take(32 * static_cast<size_t>(n));
    cflags = take(4 * static_cast<size_t>(n));
    nbr = take(4 * static_cast<size_t>(m));
    hr = take(16 * static_cast<size_t>(m));
    ghost_real = take(4 * static_cast<size_t>(g));
    ghost_unit = take(16 * static_cast<size_t>(g));
    cell_order = take(4 * static_cast<size_t>(n));
    const size_t k = mixed ? 1 : 0;  // FP32 copies only for the mixed path
    nrm32 = take(k * 8 * static_cast<size_t>(e));
    nabs32 = take(k * 4 * static_cast<size_t>(e));
    par32 = take(k * 8 * static_cast<size_t>(e));
    area32 = take(k * 4 * static_cast<size_t>(e));
    xarea32 = take(cyl ? k * 4 * static_cast<size_t>(e) : 0);
    dm0_32 = take(k * 8 * static_cast<size_t>(e));
    dm1_32 = take(k * 8 * static_cast<size_t>(e));
    width32 = take(k * 4 * static_cast<size_t>(n));
    minv32 = take(k * 16 * static_cast<size_t>(n));
    ent32 = take(k * 16 * static_cast<size_t>(m));
    fsign32 = take(k * 4 * static_cast<size_t>(m));
    gunit32 = take(k * 8 * static_cast<size_t>(g));
    icdv32 = take(k * 4 * static_cast<size_t>(n));
    frec32 = take(k * 32 * static_cast<size_t>(e));
    total = o;
  }
};

struct MeshSlot {
  int n = 0, g = 0, e = 0, m = 0;
  bool valid = false;
  DevBuf buf;
  SlotLayout lay;
  rg::MeshDev mesh{};
  rg::GeomDev geom{};
  rg::MixedGeom g32{};
  rg_error geom_error{};  // reconstruction failure found by the geometry pass
  // the FP64 per-face / per-cell geometry is formed (an FP32-mixed handle
  // without tracers uploads only its FP32 geometry: ensure_geom64)
  bool geom64 = true;
  cudaEvent_t last_use = nullptr;
};

template <class T>
T* at(void* base, size_t off) {
  return reinterpret_cast<T*>(static_cast<char*>(base) + off);
}


}  // namespace rgh

struct rg_adjoint_state;  // rg_adjoint_api.cu

struct rg_handle {
  rg_config cfg{};
  cudaStream_t stream = nullptr;
  cudaStream_t upload_stream = nullptr;
  cudaEvent_t ev_uploaded = nullptr;  // the upload stream's work for the newest mesh slot
  // rg_get_state_async: its copies run on download_stream after ev_state
  // (recorded on stream); stream waits for ev_downloaded before later work
  cudaStream_t download_stream = nullptr;
  cudaEvent_t ev_state = nullptr, ev_downloaded = nullptr;
  bool state_pending = false;
  cudaEvent_t ev_k[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  rgh::MeshSlot slots[2];
  int active = -1;
  // state
  rgh::DevBuf cells, ext, ev, slopes, fluxes, status_buf;
  // FP32-mixed path: FP32 primitives (n + g records), slopes, face fluxes, edge velocities
  rgh::DevBuf cells32, slopes32, flux32, ev32;
  bool mixed = false;
  // Heun mid stage: extensives and cells after the first flux pass
  rgh::DevBuf mid_ext, mid_cells, mid_cells32;
  bool heun = false;
  // batch of independent problems (n_problems == 0: one problem)
  int n_problems = 0;
  rgh::DevBuf cell_problem, problem_offsets, gamma_p, gamma32_p, inv_gm1_32_p, dtmin_p, time_p, dt_p;
  // RG_STEP_PERSISTENT: rg_run / rg_run_graph of a batch in one cooperative
  // launch (its grid barrier and problem 0's dt per step)
  int step_mode = 0;
  rgh::DevBuf barrier, dt_trace;
  // CUDA graph of one fused step
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  size_t cells_records = 0;
  bool have_cells = false, have_ext = false, have_ev = false, have_fluxes = false;
  rgh::HostBuf staging, host_status, host_dts;
  rg::DevStatus* d_status = nullptr;
  rg::DevStatus* d_geom_status = nullptr;
  rg::DevStatus* d_valid_status = nullptr;  // index validation of an upload (follows d_geom_status)
  rg_error last{};
  double last_upload_ms = 0;
  double last_dt = 0;
  int step_seq = 0;
  // launch shapes of the per-step kernels (rg_autotune / rg_set_launch_shapes)
  rg::StepShapes shapes64, shapes32;
  // Fused steps: the update kernel of a fused step also computes the next
  // step's SimpleCFL dt (status->dt_next) from the cells it writes and the
  // current face velocities, so the next fused step needs no CFL pass.  Any
  // change of the cells, face velocities or mesh clears dt_next_ready; a
  // caller with the device pointers (rg_device_buffers) may write them at
  // any time, so fusing stops for that handle.
  bool dt_next_ready = false;
  bool external_state = false;
  // every face velocity last set is +-0 (checked on the device when set)
  bool ev_zero = false;
  // FP32-mixed device motion wrote only the FP32 face velocities: the FP64
  // ones are formed from the point velocities when read back
  bool ev64_pending = false;
  rgh::DevBuf flag_buf;
  // differentiation: checkpoints, recomputation buffers, reverse adjacency
  rg_adjoint_state* adj = nullptr;
  // tracers and stickers (rg_set_tracer_config): cell tracers, extensive
  // tracers, tracer slopes and fluxes, each face's unscaled mass flux, each
  // cell's shock decision and sticker mask; sized for tr_n cells, tr_e faces
  rg_tracer_config tcfg{0, 0, 0u, -1, -1, -1};
  // condition/action flux rules (rg_set_flux_rules)
  int n_rules = 0;
  rg_flux_rule rules[RG_MAX_FLUX_RULES];
  // LagrangianFlux's ws_ / edge_vel_ per face (sized when a rule uses it) and
  // LagrangianExtensiveUpdater (rg_set_lagrangian_updater)
  rgh::DevBuf lag_ws, lag_ev;
  bool lag_rule = false, lag_update = false;
  rgh::DevBuf tr, tr_ext, tr_slopes, tr_flux, mflux, tr_side, shock, stickers;
  rgh::DevBuf mid_tr, mid_tr_ext;  // TimeAdvance2Heun's mid tracers (n*nt each)
  bool have_tr = false, have_tr_ext = false;
  int tr_n = -1, tr_e = -1;
  // device-side point motion (rg_set_point_motion), the outer boundary's box
  // (rg_set_outer_box) and the point velocities of the last motion call
  rg_point_motion motion{RG_MOTION_EULERIAN, RG_EDGES_STATIONARY_BOX, 0.15, 0.02, 0, 0};
  // PhysicalGeometry (rg_set_physical_geometry), applied at each upload
  rg_physical_geometry pgeo{RG_GEOMETRY_SLAB, {0, 0}, {0, 1}, 0};
  double box[4] = {0, 0, 0, 0};
  bool have_box = false;
  rgh::DevBuf pv;
};


namespace rgh {

rg_status cuda_fail(rg_handle* h, cudaError_t e);
rg_status invalid(rg_handle* h, int64_t index, double value);
rg_status reset_status(rg_handle* h, rg::DevStatus* st, cudaStream_t s);
rg_status collect(rg_handle* h, rg::DevStatus* st, cudaStream_t s);
MeshSlot* active_slot(rg_handle* h);
rg::StepArgs step_args(rg_handle* h);
rg::MixedArgs mixed_args(rg_handle* h);
void drop_graph(rg_handle* h);
rg_status require(rg_handle* h, bool cells, bool ext, bool ev, bool fluxes);
rg_status mesh_error(rg_handle* h);
// forms the active slot's FP64 geometry where an FP32-mixed upload left it out
rg_status ensure_geom64(rg_handle* h);
// frees the differentiation buffers (rg_destroy; a new mesh drops them too)
void adjoint_release(rg_handle* h);
// tracers or stickers configured (rg_tracer_api.cu)
bool tracers_on(const rg_handle* h);
// sizes the tracer buffers for the active mesh; a new cell count clears the
// tracer state and the stickers
rg_status tracer_buffers(rg_handle* h);
// sizes LagrangianFlux's per-face buffers for the active mesh (a rule uses it)
rg_status lagrangian_buffers(rg_handle* h);
rg::TracerArgs tracer_args(rg_handle* h);
// NOT_READY unless the tracer state a step needs is set
rg_status require_tracers(rg_handle* h, bool ext);
void tracer_release(rg_handle* h);

}  // namespace rgh

#define RG_CUDA(h, call)                                  \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return rgh::cuda_fail(h, e_);  \
  } while (0)
#define RG_TRY(call)                  \
  do {                                \
    rg_status s_ = (call);            \
    if (s_ != RG_OK) return s_;       \
  } while (0)
