// rg_internal.cuh -- device-side data layout shared by the kernels and the
// C-ABI host code of the GB300 hydro hot path.
//
// Layout in HBM (all arrays owned by one rg_handle):
//   points  double2[np]   mesh points, real cells then ghosts (np = n + g)
//   cms     double2[np]   cell centres of mass
//   cells   dbl4-like  double[4*np]: {density, pressure, vx, vy}; entries
//                         n..np-1 hold ghost states (filled per step)
//   ext     double[4*n]   {mass, energy, px, py}
//   faces   int2[e]       (first, second) point ids
//   face geometry (per upload): area, normal n, |n|, parallel p, mid - cm of
//                         each side
//   CSR     cell -> faces, ascending face ids, plus per entry the
//           neighbour id (with side / mirror flags) and a geometry pair
// Everything that depends only on the mesh is computed once per upload by
// the geometry kernels; the per-step kernels only do state-dependent work.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "rg_convert.cuh"
#include "rich_gb300.h"

namespace rg {

// 32-byte aligned record of four doubles (one cell, face-vertex pair or 2x2 matrix)
struct __align__(32) dbl4 {
  double x, y, z, w;
};
__host__ __device__ inline dbl4 make_dbl4(double x, double y, double z, double w) { return dbl4{x, y, z, w}; }

constexpr int kMaxNaiveNeighbours = 20;  // LinearGaussImproved.cpp:73
constexpr double kPi = 3.14159265358979323846;  // M_PI (VoronoiMesh.cpp:412)

// neighbour word of a CSR entry: low 30 bits point id, bit 30 self-mirror
// face (GetOriginalIndex(first) == GetOriginalIndex(second)), bit 31 the cell
// is the face's first neighbour (its flux enters with a minus sign).
constexpr uint32_t kNbrIdMask = 0x3fffffffu;
constexpr uint32_t kNbrMirror = 0x40000000u;
constexpr uint32_t kNbrFirst = 0x80000000u;

// per-cell geometry flags
constexpr int kCellBoundarySlope = 1;  // LinearGaussImproved.cpp:454-464

struct MeshDev {
  int n, g, e, m;           // cells, ghosts, faces, CSR entries
  const double2* points;    // np
  const double2* cms;       // np
  const double* volume;     // n (Tessellation::GetVolume)
  const double* cd_volume;  // n (CacheData::volumes)
  const int* ghost_source;  // g
  const int* ghost_face;    // g
  const int2* face_cells;   // e
  const dbl4* face_vertices;  // e
  const int* cell_off;      // n+1
  const int* cell_faces;    // m
  // the upload's geometry pass runs behind the index validation without
  // waiting for its result on the host: its kernels return at once when this
  // error key of the validation is set (nullptr: no check)
  const unsigned long long* invalid;
};
__device__ __forceinline__ bool mesh_rejected(const MeshDev& m) { return m.invalid && *m.invalid != ~0ull; }

struct GeomDev {
  // per face
  const double* area;    // |first - second| (= GetLength = calcArea)
  const double2* nrm;    // flux-frame normal (order 1: x1-x0; order 2: calc_parallel_normal)
  const double* nabs;    // abs(nrm)
  const double2* par;    // Parallel(edge) = second - first
  const double2* dm0;    // CalcCentroid(edge) - cm[first]
  const double2* dm1;    // CalcCentroid(edge) - cm[second]
  const double* dab;     // |x_second - x_first|
  const double* xarea;   // CacheData::areas of the PhysicalGeometry (SlabSymmetry: area)
  // per cell
  const double* width;   // sqrt(volume/pi)
  const dbl4* minv;   // naive-slope inverse matrix, or (SxSy, Sx2, Sy2, den) for boundary cells
  const int* cflags;
  // per CSR entry
  const uint32_t* nbr;
  const double2* hr;     // naive: 0.5*r_ij; boundary: cm[other] - cm[cell]
  // per ghost
  const int* ghost_real;      // cell whose state the ghost copies / reflects
  const double2* ghost_unit;  // rigid wall: unit normal (x_ghost - x_real)/|.|
  // the cell each thread of the FP64 slopes and update kernels takes: within
  // every tile of kOrderTile cells, the cells ordered by (boundary-slope
  // flag, neighbour count), ties by index (null: thread i takes cell i)
  const int* cell_order;
};
constexpr int kOrderTile = 256;

// Device status word.  The error kept is the one with the smallest
// (phase, index) key, which is the one the reference throws first: its
// passes run in phase order and each loops in ascending cell / face order.
struct DevStatus {
  unsigned long long err_key;  // ~0ull = none
  double err_value;
  int err_status;
  int lock;
  unsigned long long dt_min_bits;  // CFL min-reduction (positive doubles order as integers)
  double dt;                       // cfl * min, written by the last CFL block
  unsigned int blocks_done;        // CFL blocks finished (reset by the last one)
  int lock_timeouts;
  double dt_next;                  // next step's dt, computed by the update of this one
  float dt32, dt_next32;           // the same rounded to FP32 (FP32-mixed face kernels)
};
constexpr unsigned long long kInfBits = 0x7ff0000000000000ull;

// key = step (bits 50..62) | phase (46..49) | index (0..45): within a run of
// several steps the earliest step's failure wins, as it would on the host.
constexpr int kKeyPhaseShift = 46;
constexpr int kKeyStepShift = 50;
constexpr unsigned long long kKeyIndexMask = (1ull << kKeyPhaseShift) - 1;
__host__ __device__ inline unsigned long long err_key(int step, int phase, long long index) {
  return (static_cast<unsigned long long>(step & 0x1fff) << kKeyStepShift) |
         (static_cast<unsigned long long>(phase & 0xf) << kKeyPhaseShift) |
         (static_cast<unsigned long long>(index) & kKeyIndexMask);
}

#ifdef __CUDACC__
// Records an error; keeps the smallest key.  The lock wait is bounded: if it
// times out the key is still min-reduced and the value may be stale.
// the real cell a point stands for (a ghost: the cell it copies)
__device__ __forceinline__ int orig_of(const MeshDev& m, int p) {
  return p < m.n ? p : m.ghost_source[p - m.n];
}

__device__ inline void record_error(DevStatus* st, int step, int status, int phase, long long index,
                                    double value) {
  const unsigned long long key = err_key(step, phase, index);
  if (key >= atomicAdd(&st->err_key, 0ull)) return;
  bool done = false;
  for (int it = 0; it < (1 << 16) && !done; ++it) {
    if (atomicCAS(&st->lock, 0, 1) == 0) {
      __threadfence();
      if (key < st->err_key) {
        st->err_key = key;
        st->err_value = value;
        st->err_status = status;
      }
      __threadfence();
      atomicExch(&st->lock, 0);
      done = true;
    }
  }
  if (!done) {
    atomicAdd(&st->lock_timeouts, 1);
    atomicMin(&st->err_key, key);
  }
}

// std::min / std::max semantics
__device__ __forceinline__ double smin(double a, double b) { return b < a ? b : a; }
__device__ __forceinline__ double smax(double a, double b) { return a < b ? b : a; }

constexpr int kMaxBlockWarps = 16;  // kMaxBlock / 32

// Grid-wide minimum of non-negative doubles given as bit patterns (one value
// per thread; every thread of the grid calls this once), then *out =
// cfl * minimum, written by the last block to finish: SimpleCFL's
// `cfl * min` (simple_cfl.cpp:58-71).  Leaves the reduction words reset.
__device__ inline void grid_min_times(DevStatus* st, unsigned long long bits, double cfl, double* out,
                                      float* out32 = nullptr) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long ob = __shfl_xor_sync(0xffffffffu, bits, o);
    bits = ob < bits ? ob : bits;
  }
  __shared__ unsigned long long wmin[kMaxBlockWarps];
  __shared__ bool last;
  if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = bits;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long bm = wmin[0];
    for (int w = 1; w < static_cast<int>(blockDim.x >> 5); ++w) bm = wmin[w] < bm ? wmin[w] : bm;
    atomicMin(&st->dt_min_bits, bm);
    __threadfence();
    last = atomicAdd(&st->blocks_done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    // every block's atomicMin is visible here (threadfence before its ticket)
    __threadfence();
    const unsigned long long mb = atomicAdd(&st->dt_min_bits, 0ull);
    *out = cfl * __longlong_as_double(static_cast<long long>(mb));
    if (out32) *out32 = static_cast<float>(*out);
    st->dt_min_bits = kInfBits;  // ready for the next reduction
    st->blocks_done = 0;
  }
}
#endif

// Launch shape of a per-item kernel (cells, faces): `block` threads per block
// (a multiple of 32, at most kMaxBlock); max_blocks == 0 launches one thread
// per item, max_blocks > 0 at most that many blocks striding over the items
// (a persistent grid, typically a multiple of the SM count).  Results do not
// depend on the shape: every item is computed by one thread from the same
// inputs, and the only cross-item reductions are minima.
constexpr int kMaxBlock = 512;
// variant: 0 the kernel's plain build (blocks of up to kMaxBlock threads);
// the FP32-mixed slopes kernel also has 1, its neighbour loops unrolled by
// two, 2 and 3, register-capped builds for blocks of up to 256 threads
// with 5 or 6 blocks resident per SM (more warps in flight against fewer
// registers per thread), and 4, which loads the neighbour words, stencil
// records and states of cells with up to 8 neighbours before any arithmetic;
// the FP32-mixed update kernel has register-capped builds 2 and 3 too, and the
// FP64 slopes kernel register-capped builds 2 and 3 for 3 and 4 resident
// blocks.
struct LaunchShape {
  int block;
  int max_blocks;
  int variant;
};
constexpr LaunchShape kDefaultShape{256, 0, 0};
constexpr int kCappedBlock = 256;
inline int grid_of(const LaunchShape& s, int items) {
  const int need = items > 0 ? (items + s.block - 1) / s.block : 1;
  return s.max_blocks > 0 && need > s.max_blocks ? s.max_blocks : need;
}
// per-step kernels of one path (FP64 or FP32-mixed)
struct StepShapes {
  LaunchShape cfl = kDefaultShape, slopes = kDefaultShape, faces = kDefaultShape, update = kDefaultShape;
};

// Kernel launchers (rg_fp64.cu)
// tracer source of a condition/action face: the first or the second
// neighbour, its own cell's tracers or LinearGaussImproved's face value
constexpr unsigned char kTrSideFirst = 1, kTrSideSecond = 2, kTrSideFace = 4;

struct StepArgs {
  MeshDev mesh;
  GeomDev geom;
  double gamma, cfl;
  int order, ghost_kind, slf;
  double delta_v, theta, delta_p;
  double* cells;        // 4*np (ghost entries at the end), read by every pass
  double* ext;          // 4*n, read by the update
  double* ext_out;      // where the update writes extensives (nullptr: ext)
  double* cells_out;    // where the update writes cells (nullptr: cells)
  const double* ext_avg;  // Heun: extensives = 0.5*(gathered + ext_avg) before the cell update
  const double* ev;     // 2*e edge velocities
  double* slopes;       // 8*n
  double* fluxes;       // 4*e (unscaled or dt*area scaled)
  DevStatus* status;
  double dt_host;       // dt given by the caller (split API)
  int dt_from_device;   // 1: dt = cfl * min from status->dt_min_bits
  int step;             // step number within an rg_run (error ordering)
  int cfl_next;         // the update also computes the next step's SimpleCFL dt (status->dt_next)
  int ev_zero;          // every face velocity is +-0: kernels read none
  int take_next_dt;     // the slopes kernel first moves status->dt_next to status->dt
  int batch_keep_dt;    // batch: the update leaves the per-problem dt, time and minimum
                        // as they are (TimeAdvance2Heun's first half)
  // batch of independent problems (cell_problem == nullptr: one problem)
  const int* cell_problem;        // n + g: problem of every point
  const double* gamma_p;          // per problem
  unsigned long long* dtmin_p;    // per problem CFL minimum (bit pattern), reset by the update
  double* time_p;                 // per problem simulated time
  double* dt_p;                   // per problem last dt
  int n_problems;
  // stickers (ComputationalCell::stickers as one bit mask per cell)
  const uint32_t* stickers;       // n
  uint32_t skip_mask;             // LinearGaussImproved's skip_key bit (0: none)
  uint32_t frozen_mask;           // HasSticker + SkipUpdate bit (0: none)
  // tracer passes: the faces kernel keeps each face's unscaled mass flux and
  // the slopes kernel each cell's shock decision
  double* mflux;                  // e, or nullptr
  // e, or nullptr: for the condition/action fluxes, where face e's tracer
  // flux takes its tracers (kTrSide* bits), written beside mflux
  unsigned char* tr_side;
  unsigned char* shock;           // n, or nullptr
  // condition/action flux rules (0: Simple/ModularFluxCalculator)
  int n_rules;
  int rules[RG_MAX_FLUX_RULES][6];  // sequence, condition, sticker, action, ratchet_in, massflux bits
  // LagrangianFlux's per-face outputs (nullptr: no LagrangianFlux rule) and
  // whether the extensive update applies LagrangianExtensiveUpdater's scaling
  double* lag_ws;                 // e
  double* lag_ev;                 // e
  int lag_update;
  StepShapes shapes;  // launch shapes (host side; the kernels ignore it)
};

// Tracers (ComputationalCell::tracers, Extensive::tracers), cell-major.
constexpr int kMaxTracers = RG_MAX_TRACERS;
struct TracerArgs {
  int nt;
  uint32_t limited;       // bit j: tracer j in LinearGaussImproved's calc_tracers
  int entropy;            // the "Entropy" tracer, -1: none
  double* tr;             // n*nt
  double* tr_ext;         // n*nt
  double* tr_slopes;      // n*2*nt (x derivatives, then y)
  double* tr_flux;        // e*nt (unscaled or dt*area scaled, as the hydro fluxes)
  // TimeAdvance2Heun: the update writes the cell and extensive tracers to
  // tr_out / tr_ext_out (nullptr: in place) and averages the extensive
  // tracers with tr_ext_avg (average_extensive) when set
  double* tr_out;         // n*nt
  double* tr_ext_out;     // n*nt
  const double* tr_ext_avg;  // n*nt
};

#ifdef __CUDACC__
// Warp-aggregated atomicMin on per-problem minima: one atomic per warp when
// the warp's cells belong to one problem (the common case: problems are
// contiguous), one per lane otherwise.  Inactive lanes pass problem -1.
__device__ __forceinline__ void problem_min(unsigned long long* mins, int problem, unsigned long long bits) {
  const int p0 = __shfl_sync(0xffffffffu, problem, 0);
  if (__all_sync(0xffffffffu, problem == p0 || problem < 0)) {
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long ob = __shfl_xor_sync(0xffffffffu, bits, o);
      bits = ob < bits ? ob : bits;
    }
    if ((threadIdx.x & 31) == 0 && p0 >= 0) atomicMin(&mins[p0], bits);
  } else if (problem >= 0) {
    atomicMin(&mins[problem], bits);
  }
}
#endif

// Grid barrier of a cooperative launch (every block resident): an arrival
// counter and a generation word, zeroed before the launch.
struct GridBarrier {
  unsigned int count;
  unsigned int gen;
};
// waits of one barrier: __nanosleep(500) each, about 1 s in all
constexpr unsigned int kBarrierSpins = 1u << 21;

#ifdef __CUDACC__
// All blocks of the grid meet here (expected: the blocks that arrive, the
// grid's size).  The last to arrive resets the counter and advances the
// generation; the others wait for the generation to move, at most
// kBarrierSpins sleeps, after which the block records RG_ERR_TIMEOUT (phase
// 7, the block) and the barrier returns false: the caller returns, so the
// launch ends with the error instead of waiting on.  gen is the block's copy
// of the generation (thread 0's is the one used); ok is a __shared__ word.
__device__ inline bool grid_sync(GridBarrier* gb, unsigned int& gen, unsigned int expected, int& ok, DevStatus* st,
                                 int step) {
  __syncthreads();
  if (threadIdx.x == 0) {
    int good = 1;
    __threadfence();
    const unsigned int arrived = atomicAdd(&gb->count, 1u) + 1u;
    if (arrived == expected) {
      atomicExch(&gb->count, 0u);
      __threadfence();
      atomicAdd(&gb->gen, 1u);
    } else {
      unsigned int spins = 0;
      while (*reinterpret_cast<volatile unsigned int*>(&gb->gen) == gen) {
        if (++spins > kBarrierSpins) {
          good = 0;
          record_error(st, step, RG_ERR_TIMEOUT, 7, blockIdx.x, static_cast<double>(arrived));
          break;
        }
        __nanosleep(500);
      }
    }
    __threadfence();
    gen += 1u;
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}
#endif

struct GeomArgs {
  MeshDev mesh;
  int order;
  double* area;
  double2* nrm;
  double* nabs;
  double2* par;
  double2* dm0;
  double2* dm1;
  double* dab;
  double2* rij;  // calc_naive_slope's r_ij as the first cell sees it (the second sees -r_ij)
  double2* cij;  // calc_naive_slope's c_ij (the same for both cells)
  double* width;
  dbl4* minv;
  int* cflags;
  uint32_t* nbr;
  double2* hr;
  int* ghost_real;
  double2* ghost_unit;
  int* cell_order;
  int ghost_kind;
  DevStatus* status;
};

cudaError_t launch_any_nonzero(const double* v, long long n, int* flag, cudaStream_t s);
cudaError_t launch_validate(const MeshDev& m, DevStatus* st, cudaStream_t s);
cudaError_t launch_problems(const MeshDev& m, const int* offsets, int P, int* cell_problem, DevStatus* st,
                            cudaStream_t s);
cudaError_t launch_cell_order(const MeshDev& m, int* order, int* cflags, cudaStream_t s);
cudaError_t launch_geometry(const GeomArgs& a, cudaStream_t s);
cudaError_t launch_geom_ghosts(const GeomArgs& a, cudaStream_t s);  // the ghost part of launch_geometry
cudaError_t launch_cfl(const StepArgs& a, cudaStream_t s, bool fill_ghosts);
cudaError_t launch_ghost_fill(const StepArgs& a, cudaStream_t s);
cudaError_t launch_slopes(const StepArgs& a, cudaStream_t s);
cudaError_t launch_faces(const StepArgs& a, cudaStream_t s, bool scaled);
cudaError_t launch_update(const StepArgs& a, cudaStream_t s, bool from_unscaled, bool extensive, bool cells);
cudaError_t launch_init_extensives(const StepArgs& a, cudaStream_t s);
// Tracer passes (rg_tracers.cu), each after its hydro pass
cudaError_t launch_tr_slopes(const StepArgs& a, const TracerArgs& t, cudaStream_t s);
cudaError_t launch_tr_faces(const StepArgs& a, const TracerArgs& t, cudaStream_t s, bool scaled);
cudaError_t launch_tr_update(const StepArgs& a, const TracerArgs& t, cudaStream_t s, bool from_unscaled,
                             bool extensive, bool cells);
cudaError_t launch_tr_init(const StepArgs& a, const TracerArgs& t, cudaStream_t s);

}  // namespace rg
