// rg_mixed.cuh -- arguments and launchers of the FP32-mixed kernels
// (rg_mixed.cu).  FP32 copies of the geometry live next to the FP64
// geometry of each mesh slot; the neighbour words, cell flags and ghost
// sources are shared with the FP64 path.
#pragma once
#include "rg_internal.cuh"

namespace rg {

struct MixedGeom {
  const float2* nrm;
  const float* nabs;
  const float2* par;
  const float* area;
  const float* xarea;  // CacheData::areas (SlabSymmetry: area)
  const float2* dm0;
  const float2* dm1;
  const float* width;
  const float4* minv;
  // per CSR entry (cell i, face k): {hr.x, hr.y, dm.x, dm.y} with hr the LGI
  // stencil vector (0.5 r_ij, or the CM offset of a boundary-slope cell) and
  // dm = face centroid - CM of cell i; one 16-byte record read in order
  const float4* ent;
  // per CSR entry: face index, bit 31 set when the cell is the face's first
  // neighbour (the flux enters with a minus sign)
  const int* fsign;
  const float2* ghost_unit;
  const float* inv_cd_volume;
};

struct MixedGeomArgs {
  int n, g, e, m;
  GeomDev g64;  // source (FP64 geometry of the same slot)
  const double* cd_volume;
  float2* nrm;
  float* nabs;
  float2* par;
  float* area;
  float* xarea;  // == area for SlabSymmetry
  float2* dm0;
  float2* dm1;
  float* width;
  float4* minv;
  float4* ent;
  int* fsign;
  const int* cell_faces;
  float2* ghost_unit;
  float* inv_cd_volume;
  const unsigned long long* invalid;  // MeshDev::invalid of the upload
  // launch_geom32_direct's per-face record, two float4 per face, from its
  // face pass to its cell pass: {r_ij.x, r_ij.y, first, second} (the two
  // neighbours' indices as bit patterns) and {dm0.x, dm0.y, dm1.x, dm1.y}
  float4* frec;
};

struct MixedArgs {
  MeshDev mesh;
  GeomDev geom;   // FP64 geometry: neighbour words, cell flags, ghost sources
  MixedGeom g32;
  float gamma;
  float inv_gm1;  // 1/(gamma-1)
  double cfl;
  int order, ghost_kind, slf;
  float delta_v, theta, delta_p;
  float4* cells32;   // n + g records (ghost states at the end), read by every pass
  float4* cells32_out;    // where the update writes cells (nullptr: cells32)
  double* ext_out;        // where the update writes extensives (nullptr: ext)
  const double* ext_avg;  // Heun: extensives = 0.5*(gathered + ext_avg)
  float4* slopes32;  // 2 per cell
  float4* flux32;    // per face, unscaled or dt*area scaled
  const float2* ev32;
  double* ext;       // FP64 extensives
  DevStatus* status;
  float dt32;            // dt given by the caller (split API)
  int dt32_from_device;  // 1: dt from status->dt (fused step)
  int step;
  int cfl_next;          // the update also computes the next step's dt (status->dt_next)
  int ev_zero;          // every face velocity is +-0: kernels read none
  int take_next_dt;      // the slopes kernel first moves status->dt_next to status->dt
  int batch_keep_dt;     // batch: the update leaves the per-problem dt, time and minimum
                         // as they are (TimeAdvance2Heun's first half)
  // batch of independent problems (cell_problem == nullptr: one problem)
  const int* cell_problem;
  const float* gamma_p;     // per problem
  const float* inv_gm1_p;   // per problem 1/(gamma-1)
  unsigned long long* dtmin_p;
  double* time_p;
  double* dt_p;
  int n_problems;
  // stickers and the FP64 tracer passes (as StepArgs): the skip_key and
  // SkipUpdate bits, each cell's shock decision and each face's unscaled
  // mass flux for the tracer kernels (nullptr / 0: none)
  const uint32_t* stickers;
  uint32_t skip_mask;
  uint32_t frozen_mask;
  unsigned char* shock;
  double* mflux;
  StepShapes shapes;  // launch shapes (host side; the kernels ignore it)
};

cudaError_t launch_geom32(const MixedGeomArgs& a, cudaStream_t s);
// The FP32-mixed path's geometry without the FP64 geometry pass: the face
// geometry (vertex differences, areas, centroid offsets, |x1 - x0|) in FP64
// rounded once, the normal as the exact perpendicular of the FP64 vertex
// difference, and the reconstruction stencil (the naive slope's matrix, its
// inverse, 0.5 r_ij) in FP32.  Also writes the FP64 values the FP64 motion
// kernels read (|x1 - x0| per face, sqrt(V/pi) per cell, bit-equal to the
// FP64 pass) and the neighbour words; the ghost pass (launch_geom_ghosts)
// runs first.
cudaError_t launch_geom32_direct(const GeomArgs& ga, const MixedGeomArgs& a, cudaStream_t s);
cudaError_t launch_cells_to32(const double* c64, float4* c32, int n, cudaStream_t s);
cudaError_t launch_cells_to64(const float4* c32, double* c64, int n, cudaStream_t s);
cudaError_t launch_vec2_to32(const double* v64, float2* v32, int n, cudaStream_t s);
cudaError_t launch_flux_to64(const float4* f32, double* f64, int n, cudaStream_t s);
cudaError_t launch_flux_to32(const double* f64, float4* f32, int n, cudaStream_t s);
cudaError_t launch_cfl32(const MixedArgs& a, cudaStream_t s, bool fill_ghosts);
// the FP32 slopes with the adjoint's limiter trace, slopes widened to FP64
// (periodic meshes; rg_adjoint.cuh's SlopeTrace)
struct SlopeTrace;
cudaError_t launch_slopes32_trace(const MixedArgs& a, double* slopes64, SlopeTrace* trace, cudaStream_t s);
cudaError_t launch_ghost_fill32(const MixedArgs& a, cudaStream_t s);
cudaError_t launch_slopes32(const MixedArgs& a, cudaStream_t s);
cudaError_t launch_faces32(const MixedArgs& a, cudaStream_t s, bool scaled);
cudaError_t launch_update_mixed(const MixedArgs& a, cudaStream_t s, bool from_unscaled, bool extensive, bool cells);
// n_steps batch steps (hdsim::TimeAdvance, second order) in one cooperative
// launch with grid barriers between the phases; missing > 0 makes the first
// barrier expect that many blocks more than run (its wait then runs out:
// RG_ERR_TIMEOUT).  dt_trace (n_steps, or null) receives problem 0's dts.
constexpr int kPersistBlock = 256;
cudaError_t launch_run32_persistent(const MixedArgs& a, int n_steps, int step0, GridBarrier* gb, int missing,
                                   double* dt_trace, cudaStream_t s, int* grid_out);
// grid_sync once, in a cooperative launch of two blocks per SM
cudaError_t launch_barrier_check(GridBarrier* gb, int missing, DevStatus* st, cudaStream_t s);

}  // namespace rg
