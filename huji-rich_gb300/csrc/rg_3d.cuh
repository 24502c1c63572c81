// rg_3d.cuh -- device layout of the 3D first-order path (rg_3d.cu,
// rg_3d_api.cu): HDSim3D's step (hdsim_3d.cpp:133-145) with
// FirstOrderHydroFlux, update_extensive, DefaultCellUpdater and
// CourantFriedrichsLewy on a packed 3D tessellation (rg_mesh3d_view).
//
// Layout in HBM: cells and extensives as 48-byte records (three 16-byte
// loads): cells {density, pressure, vx, vy, vz, -}, extensives and face
// fluxes {mass, px, py, pz, energy, -} (Conserved3D order).  Per face:
// neighbour pair (-1 outside), unit normal (computed once per upload as
// FirstOrderHydroFlux's normalize does), area.  Per cell: volume, width and
// the ascending face list, each entry with bit 31 set when the cell is the
// face's first neighbour.
#pragma once
#include "rg_internal.cuh"

namespace rg {

struct Mesh3Dev {
  int n, e, m;           // cells, faces, CSR entries
  const int2* face_cells;
  const double* normal;  // 3 per face, as given (Tessellation3D::Normal)
  const double* area;
  const double* volume;
  const double* width;
  const int* cell_off;
  const int* cell_faces;
};

struct Step3Args {
  Mesh3Dev mesh;
  const dbl4* nhat;       // unit normals (x, y, z, 0)
  const int* fsign;       // per CSR entry: face | bit 31 when the cell is the face's first neighbour
  double gamma, cfl;
  double* cells;          // 6 per cell
  double* ext;            // 6 per cell
  double* fluxes;         // 6 per face
  const double* fvel;     // 3 per face, or nullptr (faces at rest)
  DevStatus* status;
  double dt_host;
  int dt_from_device;
  int step;
};

// FP32-mixed 3D path (rg_3d_mixed.cu): FP32 primitives, unit normals,
// areas and widths, Hllc and CFL in FP32; FP64 extensives, volumes, the
// float-float accumulation of each cell's FP32 face fluxes and the
// internal-energy conversion.
struct Mixed3Args {
  Mesh3Dev mesh;              // FP64 mesh (face pairs, CSR, volumes)
  const int* fsign;
  const float4* nhat32;       // unit normal (x, y, z, 0)
  const float* area32;
  const float* width32;
  float gamma;
  double cfl;
  float4* cells32;            // {density, pressure, vx, vy}
  float* vz32;                // vz
  double* ext;                // 6 per cell, FP64
  float4* flux32;             // {mass, px, py, pz} per face
  float* fen32;               // energy flux per face
  const float* fvel;          // 3 per face, or nullptr
  DevStatus* status;
  float dt32;                 // dt given by the caller (split API)
  int dt_from_device;
  int step;
};

cudaError_t launch3m_geometry(const Mesh3Dev& m, const dbl4* nhat, float4* nhat32, float* area32, float* width32,
                              cudaStream_t s);
cudaError_t launch3m_cells_to32(const double* c64, float4* c32, float* vz32, int n, cudaStream_t s);
cudaError_t launch3m_cells_to64(const float4* c32, const float* vz32, double* c64, int n, cudaStream_t s);
cudaError_t launch3m_flux_to64(const float4* f32, const float* fen32, double* f64, int e, cudaStream_t s);
cudaError_t launch3m_d2f(const double* a, float* b, int n, cudaStream_t s);
cudaError_t launch3m_cfl(const Mixed3Args& a, cudaStream_t s);
cudaError_t launch3m_faces(const Mixed3Args& a, bool scaled, cudaStream_t s);
cudaError_t launch3m_update(const Mixed3Args& a, bool from_unscaled, bool do_ext, bool do_cells, cudaStream_t s);

cudaError_t launch3_validate(const Mesh3Dev& m, DevStatus* st, cudaStream_t s);
cudaError_t launch3_geometry(const Mesh3Dev& m, dbl4* nhat, int* fsign, cudaStream_t s);
cudaError_t launch3_init_extensives(const Step3Args& a, cudaStream_t s);
cudaError_t launch3_cfl(const Step3Args& a, cudaStream_t s);
// scaled: fluxes times dt*area (the fused step); otherwise the reference's
// unscaled FirstOrderHydroFlux output
cudaError_t launch3_faces(const Step3Args& a, bool scaled, cudaStream_t s);
// from_unscaled: the fluxes are unscaled and dt comes from the args
cudaError_t launch3_update(const Step3Args& a, bool from_unscaled, bool do_ext, bool do_cells, cudaStream_t s);

}  // namespace rg
