// rg_motion.cuh -- device-side geometry and point motion of the 2D path
// (rg_motion.cu, C ABI in rg_motion_api.cu).
#pragma once
#include "rg_internal.cuh"

namespace rg {

struct MotionArgs {
  int kind;        // rg_motion_kind
  int edges;       // rg_edge_velocity_kind
  int cold;        // RoundCells cold form (velocity correction in ApplyFix)
  int fix;         // RoundCells CorrectPointsOverShoot (outer boundary not periodic)
  double chi, eta; // RoundCells parameters
  dbl4 box;        // outer boundary (left, right, down, up)
  double2* pv;     // n point velocities
  double2* ev;     // e edge velocities
};

// volume, real and ghost CMs and cd_volume of a mesh from its points and face
// vertices (box = left, right, down, up; used for rigid-wall ghost CMs)
cudaError_t launch_device_geometry(const MeshDev& m, const int* order, double2* cms, double* volume, double* cd_volume,
                                   int ghost_kind, const double* box, cudaStream_t s);
// CylindricalSymmetry's CacheData face areas and (cd_volume != nullptr) cell volumes
cudaError_t launch_cyl_geometry(const MeshDev& m, double* xarea, double* cd_volume, const double* origin,
                                const double* direction, bool unit, cudaStream_t s);
cudaError_t launch_point_velocities(const StepArgs& a, const MotionArgs& mo, cudaStream_t s);
cudaError_t launch_apply_fix(const StepArgs& a, const MotionArgs& mo, cudaStream_t s);
cudaError_t launch_edge_velocities(const StepArgs& a, const MotionArgs& mo, cudaStream_t s);
// FP32-mixed handles: the face velocities into their FP32 copy only
cudaError_t launch_edge_velocities32(const StepArgs& a, const MotionArgs& mo, float2* ev32, cudaStream_t s);

}  // namespace rg
