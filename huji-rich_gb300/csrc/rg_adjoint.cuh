// rg_adjoint.cuh -- data layout of the differentiated step (tangent-linear
// and adjoint kernels, rg_adjoint.cu and rg_adjoint_rev.cu).
//
// The differentiated map is hdsim::TimeAdvance (hdsim2d.cpp:149-241) on a
// fixed periodic mesh with a fixed dt, LinearGaussImproved + Hllc +
// SimpleExtensiveUpdater + SimpleCellUpdater:
//     U_0 = I(W_0),  U_{k+1} = U_k + G(W_k),  W_{k+1} = C(U_{k+1})
// with W the cells {density, pressure, vx, vy}, U the extensives {mass,
// energy, px, py}, I hdsim's init_extensives, C SimpleCellUpdater and G the
// dt*area-scaled flux gather of one step.
#pragma once
#include "rg_internal.cuh"

namespace rg {

// What the reverse slope kernel needs from the forward limiter of one cell
// (LinearGaussImproved.cpp:174-399), per component q in {d, p, vx, vy}:
//   naive[q], naive[4+q]  the unlimited Green-Gauss slope (x, y)
//   psi[q]                the limiter factor applied to it
//   dphi[q]               centroid difference of the active candidate
//   code[q]               bits 0-7 active CSR entry (0xff: psi = 1),
//                         bits 8-9 kind (0 max, 1 min, 2 shocked, 3 shocked
//                         and clamped to 0), bits 16-23 the entry whose
//                         neighbour gave the numerator, plus one (0: the
//                         numerator is identically zero)
struct __align__(16) SlopeTrace {
  double naive[8];
  double psi[4];
  double dphi[4];
  int code[4];
};
constexpr int kTraceNone = 0xff;

struct AdjArgs {
  MeshDev mesh;
  GeomDev geom;
  double gamma, dt, delta_v, theta, delta_p;
  int slf;
  const double* cells;   // W_k: 4 doubles per point (only real records are read)
  const double* ext;     // U_k: 4*n
  double* slopes;        // 8*n (forward: written; reverse: read)
  SlopeTrace* trace;     // n
  DevStatus* status;
  // tangent-linear forward: tangents beside the values
  const double* dcells;  // 4*n
  double* dslopes;       // 8*n
  double* flux;          // 4*e dt*area scaled fluxes
  double* dflux;         // 4*e
  double* ext_rw;        // 4*n extensives updated in place
  double* dext;          // 4*n
  double* cells_out;     // 4*n
  double* dcells_out;    // 4*n
  // reverse sweep work arrays
  double* side_bar;      // 8*e: adjoint of each face's two reconstructed states
  double* self_bar;      // 4*n: a cell's own share of its state adjoint
  double* entry_bar;     // 4*m: per CSR entry, the share of that neighbour's source
  // reverse adjacency (ascending, built once per mesh)
  const int* side_off;   // n+1
  const int* sides;      // 2*e: side s = 2*face + (0 first, 1 second) whose source is the cell
  const int* target_off;  // n+1
  const int* targets;    // m: CSR entries whose neighbour's source is the cell
};

// rg_adjoint.cu (plain FP64: the values equal the production path bit for bit)
cudaError_t adj_launch_record_slopes(const AdjArgs& a, cudaStream_t s);
cudaError_t tl_launch_init(const AdjArgs& a, cudaStream_t s);
cudaError_t tl_launch_step(const AdjArgs& a, cudaStream_t s);

// rg_adjoint_rev.cu
cudaError_t adj_launch_check(const AdjArgs& a, cudaStream_t s);
cudaError_t adj_launch_seed(const AdjArgs& a, const double* wbar, double* ubar, cudaStream_t s);
// One reverse step: from U-bar_{k+1} (ubar_in) to U-bar_k (ubar_out), or,
// for the first step (grad != nullptr), to the gradient with respect to W_0.
cudaError_t adj_launch_reverse(const AdjArgs& a, const double* ubar_in, double* ubar_out, double* grad,
                               cudaStream_t s);
// the transposed cell update and gather alone (shared by both precisions)
cudaError_t adj_launch_update(const AdjArgs& a, const double* ubar_in, double* ubar_out, double* grad,
                              cudaStream_t s);
// rg_adjoint_rev32.cu: the same reverse step with the face and cell kernels in FP32
cudaError_t adj_launch_reverse32(const AdjArgs& a, const double* ubar_in, double* ubar_out, double* grad,
                                 cudaStream_t s);

}  // namespace rg
