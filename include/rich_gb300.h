/*
 * rich_gb300.h -- C ABI of the GB300 (sm_103a) hydro hot path of RICH.
 *
 * The library replaces, on one GPU, the per-step work that RICH's hdsim does
 * through five plugin interfaces:
 *
 *   FluxCalculator        source/newtonian/two_dimensional/flux_calculator_2d.hpp:35-44
 *     SimpleFluxCalculator   simple_flux_calculator.cpp:216-244  (order 1)
 *     ModularFluxCalculator  modular_flux_calculator.cpp:39-71   (order 2)
 *   SpatialReconstruction spatial_reconstruction.hpp:37-42
 *     LinearGaussImproved    interpolations/LinearGaussImproved.cpp:536-635
 *   RiemannSolver         source/newtonian/common/riemann_solver.hpp:22-23
 *     Hllc (massflux=true)   source/newtonian/common/hllc.cpp:97-154
 *   ExtensiveUpdater      extensive_updater.hpp:34-43
 *     SimpleExtensiveUpdater simple_extensive_updater.cpp:11-35
 *   CellUpdater           cell_updater_2d.hpp:34-41
 *     SimpleCellUpdater      simple_cell_updater.cpp:85-106
 *   TimeStepFunction      time_step_function.hpp:29-35
 *     SimpleCFL              simple_cfl.cpp:58-71
 *   EquationOfState       source/newtonian/common/equation_of_state.hpp:20-85
 *     IdealGas               source/newtonian/common/ideal_gas.cpp:13-44
 *
 * Conventions
 *  - Every function returns rg_status and never throws.  Physical failures
 *    that the reference reports by throwing UniversalError are returned as
 *    the matching RG_ERR_* code; rg_last_error() gives the cell or face index
 *    and the offending value, as the reference's AddEntry diagnostics do.
 *  - Host arrays passed in are borrowed for the duration of the call only.
 *    Device memory is owned by the handle.
 *  - A handle is not thread-safe (like the reference's const plugins, which
 *    mutate mutable caches); use one handle per simulation.
 *  - Cell records are 4 doubles {density, pressure, velocity.x, velocity.y}
 *    (ComputationalCell order); extensive records are 4 doubles
 *    {mass, energy, momentum.x, momentum.y} (Extensive order); face fluxes
 *    use the extensive layout.
 */
#ifndef RICH_GB300_H
#define RICH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum rg_status {
  RG_OK = 0,
  RG_ERR_INVALID_ARGUMENT = 1,
  RG_ERR_CUDA = 2,
  RG_ERR_NOT_READY = 3,          /* call order violated (e.g. flux before mesh) */
  RG_ERR_OUT_OF_MEMORY = 4,
  /* physical failures, same conditions as the reference's UniversalError */
  RG_ERR_NEGATIVE_DENSITY = 10,  /* simple_cell_updater.cpp:33-34 "Negative density" */
  RG_ERR_NEGATIVE_ENERGY = 11,   /* ideal_gas.cpp:20-21 "Negative thermal energy" */
  RG_ERR_HLLC_NAN = 12,          /* hllc.cpp:102-103 "Hllc::Solved entered with nan" */
  RG_ERR_HLLC_WAVE_SPEEDS = 13,  /* hllc.cpp:142-148 "Invalid wave speeds in hllc solver" */
  RG_ERR_SINGULAR_MATRIX = 14,   /* LinearGaussImproved.cpp:111-119 "Singular matrix" */
  RG_ERR_TOO_MANY_NEIGHBORS = 15, /* LinearGaussImproved.cpp:73-79 "Cell has too many neighbors" */
  RG_ERR_TIMEOUT = 16             /* a device-side wait gave up (the persistent batch run's grid
                                     barrier, rg_set_step_mode); the launch ended, the context
                                     stays usable */
} rg_status;

/* First failure of the last call.  index is a cell index for density,
 * energy, slope errors and a face (edge) index for HLLC errors; value is the
 * offending quantity (density, thermal energy, determinant, ...). */
typedef struct rg_error {
  int32_t status;
  int32_t phase;   /* 1 cfl, 2 slopes, 3 faces, 4 extensive update, 5 cell update, 6 geometry */
  int64_t index;
  double value;
} rg_error;

/* LinearGaussImproved's GhostPointGenerator (its `ghost_` member). */
typedef enum rg_ghost_kind {
  RG_GHOST_RIGID_WALL = 0, /* RigidWallGenerator.cpp:17-54 */
  RG_GHOST_PERIODIC = 1    /* PeriodicGhostGenerator.cpp:3-24 */
} rg_ghost_kind;

/* Which hdsim time advance rg_step / rg_run perform (fixed mesh). */
typedef enum rg_time_integrator {
  RG_TIME_ADVANCE = 0,      /* hdsim::TimeAdvance (hdsim2d.cpp:149-241): one flux pass */
  RG_TIME_ADVANCE_HEUN = 1  /* hdsim::TimeAdvance2Heun (hdsim2d.cpp:323-449): two flux passes,
                               averaged extensives */
} rg_time_integrator;

typedef enum rg_precision {
  RG_FP64 = 0,      /* plain FP64: every operation in the reference's order */
  RG_FP32_MIXED = 1 /* reconstruction + HLLC in FP32; geometry, volumes,
                       extensive accumulation and e = E/m - v^2/2 in FP64 */
} rg_precision;

typedef struct rg_config {
  double gamma;          /* IdealGas adiabatic index (ideal_gas.cpp:5-6) */
  double cfl;            /* SimpleCFL cfl number (simple_cfl.cpp:8) */
  int32_t order;         /* 1: SimpleFluxCalculator; 2: ModularFluxCalculator(LinearGaussImproved, Hllc) */
  int32_t ghost_kind;    /* rg_ghost_kind, used by order 2 */
  int32_t slope_limiter; /* LinearGaussImproved slf (LinearGaussImproved.hpp:31-40), default 1 */
  int32_t precision;     /* rg_precision */
  double delta_v;        /* LinearGaussImproved shockratio_, default 0.2 */
  double theta;          /* LinearGaussImproved diffusecoeff_, default 0.5 */
  double delta_p;        /* LinearGaussImproved pressure_ratio_, default 0.7 */
  int32_t device;        /* CUDA device ordinal */
  int32_t time_integrator; /* rg_time_integrator: the step rg_step / rg_run take */
} rg_config;

/* Fills *cfg with the reference's constructor defaults: Hllc(), SimpleCFL(0.3),
 * LinearGaussImproved(eos, ghost) defaults, IdealGas(5/3), order 2, FP64. */
void rg_default_config(rg_config* cfg);

/*
 * A tessellation packed into flat arrays (what a Tessellation + CacheData
 * give the hot path).  Point ids: real cells are 0..n_cells-1; ghost
 * (mirror / periodic) points are n_cells..n_cells+n_ghosts-1.  The adapter
 * in huji-rich_gb300/host/rich_pack.hpp builds this from a VoronoiMesh.
 *
 *   point_xy      (n_cells+n_ghosts)*2  Tessellation::GetMeshPoint
 *   cm_xy         (n_cells+n_ghosts)*2  Tessellation::GetCellCM (ghost CMs are
 *                                       the reflected / shifted ones, VoronoiMesh.cpp:355-398)
 *   volume        n_cells   Tessellation::GetVolume (mesh-point fan, VoronoiMesh.cpp:420-434)
 *   cd_volume     n_cells   CacheData::volumes = SlabSymmetry::calcVolume (physical_geometry.cpp:13-21)
 *   ghost_source  n_ghosts  Tessellation::GetOriginalIndex of each ghost
 *   ghost_face    n_ghosts  first face (ascending) touching the ghost, -1 if none
 *                           (the entry RigidWallGenerator's flat_map keeps)
 *   face_cells    n_faces*2 Edge::neighbors (first, second) as point ids
 *   face_vertices n_faces*4 Edge::vertices (first.x, first.y, second.x, second.y)
 *   cell_face_offset n_cells+1, cell_faces: Tessellation::GetCellEdges, which
 *                 VoronoiMesh::build_v fills in ascending face order
 */
typedef struct rg_mesh_view {
  int32_t n_cells;
  int32_t n_ghosts;
  int32_t n_faces;
  int32_t reserved;
  const double* point_xy;
  const double* cm_xy;
  const double* volume;
  const double* cd_volume;
  const int32_t* ghost_source;
  const int32_t* ghost_face;
  const int32_t* face_cells;
  const double* face_vertices;
  const int32_t* cell_face_offset;
  const int32_t* cell_faces;
} rg_mesh_view;

/*
 * A 3D tessellation packed for the first-order 3D path (HDSim3D with
 * FirstOrderHydroFlux, hdsim_3d.cpp:63-76 update_extensive,
 * DefaultCellUpdater, CourantFriedrichsLewy).  Faces with a neighbour outside
 * the domain (CubeGrid's boundary faces, Tessellation3D::BoundaryFace) carry
 * -1 for it and are rigid walls.
 *
 *   face_cells       n_faces*2  Face::neighbors (first, second), -1 outside
 *   face_normal      n_faces*3  Tessellation3D::Normal (normalised by the library)
 *   face_area        n_faces    Face::GetArea
 *   volume, width    n_cells    Tessellation3D::GetVolume, GetWidth
 *   cell_face_offset n_cells+1, cell_faces: Tessellation3D::GetCellFaces,
 *                    ascending face ids
 */
typedef struct rg_mesh3d_view {
  int32_t n_cells;
  int32_t n_faces;
  const int32_t* face_cells;
  const double* face_normal;
  const double* face_area;
  const double* volume;
  const double* width;
  const int32_t* cell_face_offset;
  const int32_t* cell_faces;
} rg_mesh3d_view;

/* Device addresses of the handle's state, for callers that keep data on the
 * GPU (all valid until the next rg_upload_mesh or rg_destroy). */
typedef struct rg_device_view {
  double* cells;           /* n_cells*4 */
  double* extensives;      /* n_cells*4 */
  double* edge_velocities; /* n_faces*2 */
  double* fluxes;          /* n_faces*4, last rg_flux result (unscaled) */
  void* stream;            /* cudaStream_t all kernels of the handle run on */
} rg_device_view;

/* Upload flags */
#define RG_MESH_STATIC 1u /* mesh will not change: later uploads may be skipped by the caller */
/* cm_xy, volume and cd_volume are computed on the device from the points and
 * face vertices (and may be NULL): Tessellation::GetVolume
 * (VoronoiMesh.cpp:420-434), CalcCellCM (:436-451) with the ghosts' shifted
 * (periodic) or reflected (rigid walls, the box of rg_set_outer_box) CMs
 * (:316-330, 355-398), SlabSymmetry::calcVolume (physical_geometry.cpp:13-21).
 * Bit-identical to the reference's values. */
#define RG_MESH_DEVICE_GEOMETRY 2u

typedef struct rg_handle rg_handle;

/* Lifecycle ---------------------------------------------------------------- */
rg_status rg_create(const rg_config* cfg, rg_handle** out);
rg_status rg_destroy(rg_handle* h);
const char* rg_status_string(rg_status s);
rg_status rg_last_error(const rg_handle* h, rg_error* err);

/* Mesh --------------------------------------------------------------------- */
/* Copies the mesh to the device through pinned staging buffers on the upload
 * stream and computes all geometry-only terms there (face normals, lengths,
 * widths, gradient matrices).  Returns RG_ERR_SINGULAR_MATRIX /
 * RG_ERR_TOO_MANY_NEIGHBORS only when the reconstruction would throw for it
 * (order 2); the error is also returned by the next rg_flux, which is where
 * the reference throws it. */
rg_status rg_upload_mesh(rg_handle* h, const rg_mesh_view* mesh, uint32_t flags);
/* Milliseconds the last upload took (host->device copies + geometry pass). */
rg_status rg_last_upload_ms(const rg_handle* h, double* ms);

/* State -------------------------------------------------------------------- */
rg_status rg_set_cells(rg_handle* h, const double* cells);
rg_status rg_get_cells(rg_handle* h, double* cells);
rg_status rg_set_extensives(rg_handle* h, const double* extensives);
/* No counterpart in the reference.  rg_get_cells / rg_get_extensives
 * without waiting: copies the cells and the extensives (either may be NULL)
 * into the caller's host arrays on the handle's download stream once the
 * work enqueued so far has finished, and returns at once.  The copies run
 * beside a following rg_upload_mesh (its own stream; the host link is full
 * duplex), and every computation enqueued on the handle afterwards waits for
 * them on the device.  The arrays must not be read or freed before
 * rg_wait_state returns; they should be pinned host memory (pageable memory
 * is copied before the call returns). */
rg_status rg_get_state_async(rg_handle* h, double* cells, double* extensives);
/* Waits for the copies of the last rg_get_state_async. */
rg_status rg_wait_state(rg_handle* h);
rg_status rg_get_extensives(rg_handle* h, double* extensives);
rg_status rg_set_edge_velocities(rg_handle* h, const double* edge_velocities);
rg_status rg_device_buffers(rg_handle* h, rg_device_view* view);
/* hdsim's init_extensives (hdsim2d.cpp:41-67): extensives from cells and cd_volume. */
rg_status rg_init_extensives(rg_handle* h);

/* The five plugin operations ---------------------------------------------- */
/* SimpleCFL::operator() on the current cells and edge velocities. */
rg_status rg_cfl_dt(rg_handle* h, double* dt);
/* FluxCalculator::operator(): per-face fluxes (unscaled, as the reference
 * returns them).  fluxes_out (n_faces*4, host) may be NULL to keep them on
 * the device only. */
rg_status rg_flux(rg_handle* h, double dt, double* fluxes_out);
/* Upload caller-provided fluxes (n_faces*4) in place of the last rg_flux. */
rg_status rg_set_fluxes(rg_handle* h, const double* fluxes);
/* SimpleExtensiveUpdater::operator(): extensives += gathered dt*area*flux,
 * in ascending face order per cell (no atomics). */
rg_status rg_extensive_update(rg_handle* h, double dt);
/* SimpleCellUpdater::operator(): cells from extensives and cd_volume. */
rg_status rg_cell_update(rg_handle* h);

/* hdsim::TimeAdvance's hot path fused on the device (hdsim2d.cpp:149-241 with
 * a fixed mesh): dt = SimpleCFL, fluxes, extensive update, cell update; or,
 * with time_integrator = RG_TIME_ADVANCE_HEUN, hdsim::TimeAdvance2Heun
 * (hdsim2d.cpp:323-449): fluxes on the cells, mid extensives and cells,
 * fluxes on the mid cells, extensives averaged.  dt never leaves the device
 * between the passes; *dt_out receives it. */
rg_status rg_step(rg_handle* h, double* dt_out);
/* n_steps rg_step calls without a host synchronisation between them; errors
 * are checked once at the end.  dt_out (n_steps, host) may be NULL. */
rg_status rg_run(rg_handle* h, int32_t n_steps, double* dt_out);
/* rg_step with CUDA events between its kernels (the work is identical):
 * kernel_ms[0..3] = CFL (with the ghost fill), LinearGaussImproved slopes
 * (0 for order 1), face fluxes, gather + cell update.  For the Heun step:
 * CFL, first pass (slopes + faces + update), second pass (ghost fill +
 * slopes + faces), final update. */
rg_status rg_step_timed(rg_handle* h, double* dt_out, float* kernel_ms);
/* Enqueues one fused step on the handle's stream and returns at once; its
 * failures surface at the next rg_synchronize. */
rg_status rg_step_async(rg_handle* h);
/* Waits for the handle's stream; returns the first failure of the enqueued
 * steps and the dt of the last one (dt_last may be NULL). */
rg_status rg_synchronize(rg_handle* h, double* dt_last);

/* Batches of independent problems ----------------------------------------- */
/* No counterpart in the reference (its hdsim runs one problem; this is the
 * batched form of the path).  Declares the uploaded mesh a batch: problem p
 * owns the real cells [problem_cell_offset[p], problem_cell_offset[p+1]) and
 * the ghosts and faces that touch them (a face joining two problems is
 * rejected).  Each problem has its own IdealGas index gamma[p] and, in
 * rg_step / rg_run / rg_run_graph, its own SimpleCFL dt and simulated time;
 * every problem advances one step per step.  n_problems = 0 returns to one
 * problem.  Call after rg_upload_mesh (an upload drops the table).  Only the
 * fused steps and the state transfers are available in batch mode (rg_cfl_dt
 * returns RG_ERR_INVALID_ARGUMENT); the steps are TimeAdvance or
 * TimeAdvance2Heun (cfg.time_integrator), with tracers and stickers on the
 * FP64 path; condition/action flux rules and differentiation are
 * single-problem only. */
rg_status rg_set_problems(rg_handle* h, int32_t n_problems, const int32_t* problem_cell_offset,
                          const double* gamma);
/* Per-problem simulated time (sum of its dts since rg_set_problems) and last
 * dt (n_problems doubles each; either may be NULL). */
rg_status rg_get_problem_times(rg_handle* h, double* time_out, double* dt_last_out);

/* n_steps fused steps replayed from a CUDA graph of one step (captured on
 * first use and after every upload or configuration change), one host
 * synchronisation at the end.  Same results as rg_run; a failure is reported
 * with step 0 in its key. */
rg_status rg_run_graph(rg_handle* h, int32_t n_steps);

/* How rg_run / rg_run_graph run a batch (no reference counterpart).
 * RG_STEP_PER_PHASE (default): one launch per phase of each step.
 * RG_STEP_PERSISTENT: the whole run in one cooperative launch, every block
 * resident, the phases of each step (CFL, slopes, faces, each problem's dt
 * and time, update) separated by a grid barrier; results bit-identical to
 * RG_STEP_PER_PHASE, and rg_run's dt_out is problem 0's dt per step.  Taken
 * by a batch (rg_set_problems) on the FP32-mixed path, second order,
 * hdsim::TimeAdvance, without tracers, stickers or flux rules; anything else
 * returns RG_ERR_INVALID_ARGUMENT, here or at the run.  A barrier wait that
 * runs out (about 1 s) ends the launch with RG_ERR_TIMEOUT. */
typedef enum { RG_STEP_PER_PHASE = 0, RG_STEP_PERSISTENT = 1 } rg_step_mode;
rg_status rg_set_step_mode(rg_handle* h, int32_t mode);
/* Runs the persistent form's grid barrier once on its own, in a cooperative
 * launch, expecting missing_blocks more blocks than it launches: RG_OK for 0,
 * RG_ERR_TIMEOUT (after the barrier's bounded wait) otherwise.  For testing
 * the timeout path; the handle stays usable. */
rg_status rg_grid_barrier_check(rg_handle* h, int32_t missing_blocks);

/* The CUDA stream (cudaStream_t) all kernels of the handle run on, for
 * callers that order their own work with the handle's (no reference
 * counterpart).  Unlike rg_device_buffers it hands out no state pointers. */
rg_status rg_stream(const rg_handle* h, void** stream);

/* Launch shapes and the autotuner ------------------------------------------ */
/* No counterpart in the reference.  The per-step kernels (rg_kernel order:
 * CFL, slopes, face fluxes, gather+update) of the handle's current path
 * (rg_config.precision; batch or single problem) each run with a launch
 * shape: threads per block (a multiple of 32, 32..512) and max_blocks (0: one
 * thread per cell or face; > 0: a persistent grid of at most that many blocks
 * striding over the items).  Results are identical for every shape. */
typedef enum { RG_KERNEL_CFL = 0, RG_KERNEL_SLOPES = 1, RG_KERNEL_FACES = 2, RG_KERNEL_UPDATE = 3 } rg_kernel;
typedef struct {
  int32_t block[4];
  int32_t max_blocks[4];
  int32_t variant[4]; /* build: 0; the FP32-mixed slopes kernel also has 1 (loops unrolled
                         by two), 2, 3 (register-capped: blocks of at most 256 threads,
                         5 or 6 resident per SM) and 4 (up to 8 neighbours loaded up front);
                         the FP32-mixed update kernel 2 and 3 (register-capped); the
                         FP32-mixed face kernel 1 (two threads per face, second order); the
                         FP64 slopes kernel 2 and 3 (register-capped: blocks of at most
                         256 threads, 3 or 4 resident per SM) */
  float ms[4];        /* rg_autotune: mean time per launch of the chosen shape (ms) */
} rg_launch_shapes;
/* Times every candidate shape of each per-step kernel on the uploaded mesh
 * and the current state (reps launches each; the state is left unchanged)
 * and keeps the fastest.  Needs the cells, extensives and edge velocities. */
rg_status rg_autotune(rg_handle* h, int32_t reps, rg_launch_shapes* chosen);
rg_status rg_set_launch_shapes(rg_handle* h, const rg_launch_shapes* shapes);
rg_status rg_get_launch_shapes(const rg_handle* h, rg_launch_shapes* shapes);

/* Point motion on the device ---------------------------------------------- */
/* hdsim::TimeAdvance's first half (hdsim2d.cpp:149-195) on the device: the
 * PointMotion's point velocities, the EdgeVelocityCalculator's face
 * velocities, SimpleCFL on them, PointMotion::ApplyFix with that dt, the face
 * velocities again, the fluxes and the extensive update.  The host then moves
 * the points (MoveMeshPoints), rebuilds the tessellation, uploads it (with
 * RG_MESH_DEVICE_GEOMETRY only points, topology and face vertices cross the
 * bus) and calls rg_cell_update, which uses the new mesh's volumes as
 * hdsim's cell update does. */
typedef enum rg_motion_kind {
  RG_MOTION_EULERIAN = 0,    /* eulerian.cpp: points at rest */
  RG_MOTION_LAGRANGIAN = 1,  /* lagrangian.cpp:3-13: the cell velocity */
  RG_MOTION_ROUND_CELLS = 2  /* RoundCells(Lagrangian) (round_cells.cpp) */
} rg_motion_kind;
typedef enum rg_edge_velocity_kind {
  RG_EDGES_STATIONARY_BOX = 0, /* stationary_box.cpp:20-40: 0 on a point's face with its own copy */
  RG_EDGES_PERIODIC = 1        /* periodic_edge_velocities.cpp:5-21 */
} rg_edge_velocity_kind;
typedef struct rg_point_motion {
  int32_t kind;              /* rg_motion_kind */
  int32_t edges;             /* rg_edge_velocity_kind */
  double chi, eta;           /* RoundCells chi, eta (defaults 0.15, 0.02) */
  int32_t cold;              /* RoundCells cold switch */
  int32_t correct_overshoot; /* RoundCells' outer boundary is not periodic: CorrectPointsOverShoot
                                with the box of rg_set_outer_box */
} rg_point_motion;
/* the OuterBoundary's box (GetGridBoundary Left, Right, Down, Up) */
rg_status rg_set_outer_box(rg_handle* h, double left, double right, double down, double up);
rg_status rg_set_point_motion(rg_handle* h, const rg_point_motion* pm);
/* PointMotion::operator() and the face velocities from it (the handle's edge
 * velocities); point_velocities_out (n_cells*2) may be NULL */
rg_status rg_point_velocities(rg_handle* h, double* point_velocities_out);
/* PointMotion::ApplyFix with dt on the current point velocities, then the face
 * velocities again */
rg_status rg_apply_fix(rg_handle* h, double dt, double* point_velocities_out);
/* The handle's face velocities (n_faces*2).  On an FP32-mixed handle the
 * device motion forms only their FP32 copy, which the FP32 passes read; this
 * call forms the FP64 ones from the same point velocities first.  After a
 * new mesh is uploaded, face velocities of the old mesh's motion are gone
 * (RG_ERR_NOT_READY until the next motion or rg_set_edge_velocities). */
rg_status rg_get_edge_velocities(rg_handle* h, double* edge_velocities_out);
/* the mesh geometry in use (computed on the device or uploaded); cd_area:
 * CacheData's face areas (n_faces) of the PhysicalGeometry.  Any pointer may
 * be NULL.  On an FP32-mixed handle without tracers the upload forms only
 * the FP32 face geometry; asking for cd_area forms the FP64 geometry (once
 * per mesh) and rounds the FP32 copies from it. */
rg_status rg_get_geometry(rg_handle* h, double* volume, double* cm_xy, double* cd_volume, double* cd_area);

/* PhysicalGeometry (physical_geometry.hpp): SlabSymmetry (the default) or
 * CylindricalSymmetry about the axis through origin along direction
 * (physical_geometry.cpp:62-110).  It sets CacheData's face areas, by which
 * SimpleExtensiveUpdater scales the fluxes, and, with RG_MESH_DEVICE_GEOMETRY,
 * the cell volumes (cd_volume) the cell updater divides by; uploaded
 * cd_volume arrays are the caller's CacheData volumes.  Takes effect at the
 * next rg_upload_mesh.  The source term the reference pairs with it
 * (CylindricalComplementary) is an external force, outside these passes.
 * Differentiation returns RG_ERR_INVALID_ARGUMENT with CylindricalSymmetry. */
typedef enum rg_geometry_kind { RG_GEOMETRY_SLAB = 0, RG_GEOMETRY_CYLINDRICAL = 1 } rg_geometry_kind;
typedef struct rg_physical_geometry {
  int32_t kind;         /* rg_geometry_kind */
  double origin[2];     /* axis origin (CylindricalSymmetry) */
  double direction[2];  /* axis direction: any length (normalised as Axis's constructor does,
                           physical_geometry.cpp:40-42), or Axis::direction itself with unit = 1 */
  int32_t unit;         /* 1: direction is already the Axis's normalised direction */
} rg_physical_geometry;
rg_status rg_set_physical_geometry(rg_handle* h, const rg_physical_geometry* pg);
/* point velocities, face velocities, dt, ApplyFix, face velocities, fluxes,
 * extensive update (one host synchronisation, at the end) */
rg_status rg_advance_begin(rg_handle* h, double* dt_out, double* point_velocities_out);

/* Condition/action flux schemes --------------------------------------------- */
/* ConditionActionSequence (condition_action_sequence.cpp, order 1) and
 * ConditionActionSequence2 (condition_action_sequence_2.cpp, order 2 with
 * LinearGaussImproved's face states) as the flux calculator: per face the
 * first rule of sequence 0 whose condition holds, else the first of
 * sequence 1, picks the flux action; no rule holding is reported as
 * RG_ERR_INVALID_ARGUMENT (phase 3, the face) like the reference's "Error in
 * ConditionActionSequence".  RegularSpecialEdge reads the sticker bit of
 * rg_set_stickers.  FP64 path, no tracers; n_rules = 0 restores the
 * Simple/ModularFluxCalculator of the configured order. */
#define RG_MAX_FLUX_RULES 8
typedef enum rg_flux_condition {
  RG_COND_BOUNDARY_EDGE = 0,  /* IsBoundaryEdge (:228-253) */
  RG_COND_BULK_EDGE = 1,      /* IsBulkEdge (:255-271) */
  RG_COND_SPECIAL_EDGE = 2    /* RegularSpecialEdge(sticker) (:273-289) */
} rg_flux_condition;
typedef enum rg_flux_action {
  RG_ACT_REGULAR = 0,      /* RegularFlux (:84-110): cell states */
  RG_ACT_RIGID_WALL = 1,   /* RigidWallFlux (:140-184) */
  RG_ACT_FREE_FLOW = 2,    /* FreeFlowFlux (:186-220) */
  RG_ACT_REGULAR2 = 3,     /* RegularFlux2 (condition_action_sequence_2.cpp:129-157): face states */
  RG_ACT_RIGID_WALL2 = 4,  /* RigidWallFlux2 (:183-228) */
  RG_ACT_RATCHET = 5,      /* Ratchet(in) (:232-249) */
  RG_ACT_LAGRANGIAN = 6    /* LagrangianFlux(rs, rs2, WallsMassFlux) (:252-312): face states, a
                              LagrangianHLLC (LagrangianHLLC.cpp:85-175) where the face is not a
                              self-mirror (rs), another elsewhere (rs2) */
} rg_flux_action;
typedef struct rg_flux_rule {
  int32_t sequence;   /* 0: ConditionActionSequence's list (actions 0-2), 1: ConditionActionSequence2's (3-5) */
  int32_t condition;  /* rg_flux_condition */
  int32_t sticker;    /* RG_COND_SPECIAL_EDGE's sticker bit */
  int32_t action;     /* rg_flux_action */
  int32_t ratchet_in; /* Ratchet's `in` */
  int32_t massflux;   /* LagrangianFlux: bit 0 rs's LagrangianHLLC(massflux), bit 1 rs2's */
} rg_flux_rule;
rg_status rg_set_flux_rules(rg_handle* h, int32_t n_rules, const rg_flux_rule* rules);
/* LagrangianExtensiveUpdater(lflux, SimpleExtensiveUpdater)
 * (LagrangianExtensiveUpdater.cpp:8-80) as the extensive updater (on != 0):
 * after the flux gather every cell's extensives are multiplied by
 * (V + dV) / (V + dV + dV_ws), dV and dV_ws the sums over its faces of
 * area*dt times the last LagrangianFlux pass's face speed and ws (+ as the
 * first neighbour, - as the second, in face order), V its CacheData volume.
 * Faces of other actions carry 0 (LagrangianFlux::Reset). */
rg_status rg_set_lagrangian_updater(rg_handle* h, int32_t on);
/* the last flux pass's LagrangianFlux ws_ and edge_vel_ (n_faces each), and
 * the same from the host (for fluxes given by rg_set_fluxes) */
rg_status rg_get_lagrangian_faces(rg_handle* h, double* ws, double* edge_vel);
rg_status rg_set_lagrangian_faces(rg_handle* h, const double* ws, const double* edge_vel);

/* Tracers and stickers ---------------------------------------------------- */
/* ComputationalCell::tracers / ::stickers (computational_cell_2d.hpp:19-36)
 * and Extensive::tracers (extensive.hpp) on the FP64 path, with the
 * reference's plugins that read them:
 *   hdsim's TracerStickerNames (hdsim2d.hpp:86-101, names sorted by hdsim's
 *     constructor, hdsim2d.cpp:121-136): tracer j and sticker bit k are the
 *     j-th / k-th names in sorted order;
 *   LinearGaussImproved(..., calc_tracers, skip_key)
 *     (LinearGaussImproved.hpp:45-58): tracers outside calc_tracers get zero
 *     slopes, limited ones use the velocity form of both limiters; cells
 *     carrying the skip_key sticker are left out of the limiters' neighbour
 *     max/min and of the shocked limiter's edges (this changes hydro slopes
 *     too);
 *   ModularFluxCalculator / SimpleFluxCalculator tracer fluxes
 *     (modular_flux_calculator.cpp:24-35, simple_flux_calculator.cpp:193-213):
 *     mass flux times the upwind side's tracer;
 *   SimpleExtensiveUpdater (dt*area scaling of every extensive tracer);
 *   SimpleCellUpdater (simple_cell_updater.cpp:22-106): tracer = extensive
 *     tracer / mass; the tracer named "Entropy" is recomputed as
 *     IdealGas::dp2s(d, p) = p*pow(d, -gamma) and its extensive set to s*mass;
 *     a sequence entry (HasSticker(name), SkipUpdate()) keeps the old cell of
 *     every cell with that sticker (its extensives still take the fluxes).
 * Tracer arrays are cell-major: n_cells*n_tracers (cells[i].tracers[j] at
 * i*n_tracers + j); tracer fluxes n_faces*n_tracers; tracer slopes
 * n_cells*2*n_tracers (x derivatives then y derivatives of each cell).
 * Stickers are one uint32 bit mask per cell.  Ghost points take the tracers
 * and stickers of the cell they copy.  Tracers run with TimeAdvance and
 * TimeAdvance2Heun, on single problems and batches.  On the FP32-mixed path
 * the FP32 hydro passes honour the stickers and the tracer passes run in
 * FP64 on their shock decisions and mass fluxes, with TimeAdvance (fused,
 * split or rg_advance_begin); a FP32-mixed handle with the fused
 * TimeAdvance2Heun, and differentiation, return RG_ERR_INVALID_ARGUMENT
 * while tracers or stickers are configured.  Entropy uses the device pow():
 * that one tracer agrees with the host libm to a few ulp; everything else
 * on the FP64 path is bit for bit. */
#define RG_MAX_TRACERS 8
typedef struct rg_tracer_config {
  int32_t n_tracers;        /* 0..RG_MAX_TRACERS */
  int32_t n_stickers;       /* sticker bits in use (0..32); stickers are also kept when a sticker bit
                               below is set */
  uint32_t limited_mask;    /* bit j: tracer j is in LinearGaussImproved's calc_tracers */
  int32_t entropy_tracer;   /* index of the "Entropy" tracer, -1: none */
  int32_t skip_sticker;     /* sticker bit of LinearGaussImproved's skip_key, -1: none */
  int32_t frozen_sticker;   /* sticker bit of SimpleCellUpdater's HasSticker + SkipUpdate, -1: none */
} rg_tracer_config;
/* cfg == NULL or {0, 0, 0, -1, -1, -1}: no tracers, no stickers (the default).
 * Tracer values start unset (rg_set_tracers), stickers all clear. */
rg_status rg_set_tracer_config(rg_handle* h, const rg_tracer_config* cfg);
rg_status rg_set_tracers(rg_handle* h, const double* tracers);
rg_status rg_get_tracers(rg_handle* h, double* tracers);
rg_status rg_set_extensive_tracers(rg_handle* h, const double* tracers);
rg_status rg_get_extensive_tracers(rg_handle* h, double* tracers);
rg_status rg_set_stickers(rg_handle* h, const uint32_t* stickers);
/* tracer fluxes computed elsewhere (the tracer part of rg_set_fluxes), n_faces*n_tracers */
rg_status rg_set_tracer_fluxes(rg_handle* h, const double* tracer_fluxes);
/* after rg_flux: the unscaled tracer fluxes and the tracer slopes (order 2) */
rg_status rg_get_tracer_fluxes(rg_handle* h, double* tracer_fluxes);
rg_status rg_get_tracer_slopes(rg_handle* h, double* tracer_slopes);

/* Differentiation --------------------------------------------------------- */
/* No counterpart in the reference (it has no differentiation).  The map
 * differentiated is n_steps hdsim::TimeAdvance steps (hdsim2d.cpp:149-241)
 * with a FIXED dt on the uploaded mesh: U_0 = init_extensives(W_0),
 * U_{k+1} = U_k + dt-scaled flux gather of W_k, W_{k+1} = SimpleCellUpdater
 * (U_{k+1}), W the cells.  Requires order 2 (LinearGaussImproved + Hllc),
 * periodic ghosts, FP64 and one problem; anything else returns
 * RG_ERR_INVALID_ARGUMENT.  Branches (limiter candidates, neighbour max/min,
 * HLLC wave speeds and region) are those of the forward values.
 *
 * rg_step_fwd: from the handle's cells W_0 runs n_steps, keeping W and U
 * every checkpoint_every steps on the device; afterwards the handle holds
 * W_n and U_n as rg_run leaves them (same values bit for bit as the plain
 * FP64 step with that dt).
 * rg_step_bwd: given cells_bar = dL/dW_n (host, n_cells*4) returns
 * cells0_bar = dL/dW_0 (host, n_cells*4) for the last rg_step_fwd,
 * recomputing each checkpoint interval forward once.  The handle's state is
 * left as rg_step_fwd left it.
 * rg_step_tlm: tangent-linear run: from W_0 (the handle's cells) and a
 * tangent dcells0 (host, n_cells*4) runs n_steps and returns the tangent of
 * W_n in dcells (host, n_cells*4); the handle then holds W_n and U_n. */
rg_status rg_step_fwd(rg_handle* h, int32_t n_steps, double dt, int32_t checkpoint_every);
rg_status rg_step_bwd(rg_handle* h, const double* cells_bar, double* cells0_bar);
rg_status rg_step_tlm(rg_handle* h, int32_t n_steps, double dt, const double* dcells0, double* dcells);

/* 3D first-order path ------------------------------------------------------ */
/* HDSim3D::timeAdvance (hdsim_3d.cpp:133-145) on a fixed packed 3D
 * tessellation (rg_mesh3d_view): CourantFriedrichsLewy
 * (CourantFriedrichsLewy.cpp:23-46), FirstOrderHydroFlux with Hllc
 * (FirstOrderHydroFlux.cpp:98-114; boundary faces are rigid walls),
 * update_extensive (hdsim_3d.cpp:63-76), DefaultCellUpdater
 * (default_cell_updater.cpp:5-14) with IdealGas.  FP64, the reference's
 * operation order.  Cell records are 5 doubles {density, pressure, vx, vy,
 * vz}; extensive and flux records 5 doubles {mass, px, py, pz, energy}
 * (Conserved3D order).  rg_config supplies gamma, cfl, device and precision:
 * RG_FP32_MIXED runs the per-face work and the CFL bound in FP32 and keeps
 * the extensives, volumes, the accumulation and E/m - v^2/2 in FP64. */
typedef struct rg3_handle rg3_handle;
rg_status rg3_create(const rg_config* cfg, rg3_handle** out);
rg_status rg3_destroy(rg3_handle* h);
rg_status rg3_last_error(const rg3_handle* h, rg_error* err);
rg_status rg3_upload_mesh(rg3_handle* h, const rg_mesh3d_view* mesh);
rg_status rg3_set_cells(rg3_handle* h, const double* cells);
rg_status rg3_get_cells(rg3_handle* h, double* cells);
rg_status rg3_set_extensives(rg3_handle* h, const double* extensives);
rg_status rg3_get_extensives(rg3_handle* h, double* extensives);
/* Face velocities (n_faces*3, Tessellation3D::CalcFaceVelocity of the two
 * points); NULL: faces at rest (CubeGrid). */
rg_status rg3_set_face_velocities(rg3_handle* h, const double* face_velocities);
/* ExtensiveGenerator (extensive_generator.cpp:3-28): extensives from cells */
rg_status rg3_init_extensives(rg3_handle* h);
rg_status rg3_cfl_dt(rg3_handle* h, double* dt);
/* FluxCalculator3D output, unscaled (n_faces*5, NULL: kept on the device) */
rg_status rg3_flux(rg3_handle* h, double* fluxes_out);
/* update_extensive with the fluxes of the last rg3_flux */
rg_status rg3_extensive_update(rg3_handle* h, double dt);
rg_status rg3_cell_update(rg3_handle* h);
/* One fused timeAdvance (dt on the device) / n of them, dts optional */
rg_status rg3_step(rg3_handle* h, double* dt_out);
rg_status rg3_run(rg3_handle* h, int32_t n_steps, double* dts_out);
/* rg3_step with CUDA-event times of its three kernels (CFL, fluxes, update), ms */
rg_status rg3_step_timed(rg3_handle* h, double* dt_out, float* kernel_ms);

/* Allocation-free time step ----------------------------------------------- */
/* No counterpart in the reference.  The SimpleCFL dt of rg_cfl_dt for callers
 * that may not allocate device memory (hosts whose own allocator or arena
 * owns all GPU memory and must not see cudaMalloc / cudaFree in the step
 * loop, which would synchronise the device and bypass their accounting).
 * Every pointer is a caller-owned DEVICE pointer of the current device
 * (device or managed memory; anything else returns RG_ERR_INVALID_ARGUMENT
 * before any work is enqueued):
 *   cells            n_cells*4 {density, pressure, vx, vy}, 16-byte aligned
 *   volume           n_cells cell areas, 8-byte aligned
 *   cell_face_offset n_cells+1 and cell_faces: each cell's faces, 4-byte aligned
 *   edge_velocities  n_faces*2 face velocities, 16-byte aligned
 *   dt_out           one double, 8-byte aligned: receives the dt,
 * asynchronously on `stream` (a cudaStream_t of the current device, NULL =
 * default stream).  A misaligned pointer returns RG_ERR_INVALID_ARGUMENT.
 * Indices are NOT validated (there is no face count): a cell_faces entry
 * outside edge_velocities is read out of bounds, so pass a mesh that an
 * rg_handle has accepted or that the caller has checked.
 * Allocates nothing: its reduction scratch is a fixed 32 KiB device array
 * inside the library, so n_cells is limited to 1,048,576 (larger values
 * return RG_ERR_INVALID_ARGUMENT).  All calls share that array: calls that
 * overlap on the GPU race, so serialise them.  The first call on a device
 * looks up the array's address with that device current; under lazy module
 * loading (the CUDA default) that first call also loads the library's
 * device code and creates the array, which takes driver memory: make it
 * during set-up, before the caller's allocator takes over and before any
 * stream capture. */
rg_status rg_cfl_dt_noalloc(int32_t n_cells, const double* cells, const double* volume,
                            const int32_t* cell_face_offset, const int32_t* cell_faces,
                            const double* edge_velocities, double gamma, double cfl,
                            double* dt_out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* RICH_GB300_H */
