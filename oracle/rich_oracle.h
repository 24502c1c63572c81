/*
 * rich_oracle.h -- CPU restatement of RICH's per-step hydro hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity oracle: tests/, the smoke
 * check in __graft_entry__.py and bench.py's CPU-baseline leg call it as the
 * checker.  The product (huji-rich_gb300/) never links or calls it.
 *
 * Every function restates one reference function in plain C, operation for
 * operation and in the reference's evaluation order, on the packed mesh of
 * include/rich_gb300.h.  It is pinned against fixtures produced by the
 * reference itself (tests/golden/, generated by tests/golden/make_golden.py
 * from oracle/ref/ref_dump.cpp): bit-for-bit equality is required.
 *
 * Layouts: cells N*4 {density, pressure, vx, vy}; extensives and fluxes
 * {mass, energy, px, py}; slopes N*8 {d/dx of the 4 cell fields, d/dy ...};
 * interp E*8 {first side cell, second side cell}.
 */
#ifndef RICH_ORACLE_H
#define RICH_ORACLE_H
#include <stdint.h>
#include "rich_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ro_error {
  int32_t status; /* rg_status code, 0 = ok */
  int32_t phase;
  int64_t index;
  double value;
} ro_error;

typedef struct ro_lgi_params {
  int32_t ghost_kind; /* rg_ghost_kind */
  int32_t slf;
  double delta_v, theta, delta_p;
} ro_lgi_params;

int ro_cfl(const rg_mesh_view* m, const double* cells, const double* ev, double gamma, double cfl,
           double* dt, ro_error* err);
int ro_simple_flux(const rg_mesh_view* m, const double* cells, const double* ev, double gamma,
                   double* fluxes, ro_error* err);
int ro_lgi(const rg_mesh_view* m, const double* cells, double gamma, const ro_lgi_params* lp,
           double* slopes, double* interp, ro_error* err);
int ro_modular_flux(const rg_mesh_view* m, const double* cells, const double* ev, double gamma,
                    const ro_lgi_params* lp, double* fluxes, ro_error* err);
int ro_extensive_update(const rg_mesh_view* m, const double* fluxes, double dt, double* ext,
                        ro_error* err);
int ro_cell_update(const rg_mesh_view* m, const double* ext, double gamma, double* cells_out,
                   ro_error* err);
int ro_init_extensives(const rg_mesh_view* m, const double* cells, double gamma, double* ext);
/* One hdsim::TimeAdvance hot-path pass on a fixed mesh (cfl, flux, extensive
 * update, cell update), the same edge velocities for CFL and flux.  order 1
 * ignores lp. */
int ro_step(const rg_mesh_view* m, double* cells, double* ext, const double* ev, double gamma,
            double cfl, int order, const ro_lgi_params* lp, double* dt_out, ro_error* err);

/* hdsim::TimeAdvance2Heun (hdsim2d.cpp:323-449) on a fixed mesh with fixed
 * edge velocities (its two SimpleCFL calls then agree). */
int ro_step_heun(const rg_mesh_view* m, double* cells, double* ext, const double* ev, double gamma,
                 double cfl, int order, const ro_lgi_params* lp, double* dt_out, ro_error* err);

/* Tracers and stickers (rg_tracer_config's meaning).  tr / tr_ext arrays
 * are n_cells*n cell-major; tslopes n_cells*2n (x then y); tinterp
 * n_faces*2n (first side, second side); tfluxes n_faces*n. */
typedef struct ro_tracers {
  int32_t n;
  uint32_t limited;        /* bit j: tracer j in calc_tracers */
  int32_t entropy;         /* -1: none */
  uint32_t skip_mask;      /* sticker bits of skip_key, 0: none */
  uint32_t frozen_mask;    /* sticker bits of HasSticker + SkipUpdate, 0: none */
  const uint32_t* stickers;  /* n_cells, NULL: none */
} ro_tracers;

int ro_lgi_tr(const rg_mesh_view* m, const double* cells, const double* tr, double gamma,
              const ro_lgi_params* lp, const ro_tracers* t, double* slopes, double* interp,
              double* tslopes, double* tinterp, ro_error* err);
int ro_modular_flux_tr(const rg_mesh_view* m, const double* cells, const double* tr, const double* ev,
                       double gamma, const ro_lgi_params* lp, const ro_tracers* t, double* fluxes,
                       double* tfluxes, ro_error* err);
int ro_simple_flux_tr(const rg_mesh_view* m, const double* cells, const double* tr, const double* ev,
                      double gamma, const ro_tracers* t, double* fluxes, double* tfluxes, ro_error* err);
void ro_extensive_update_tr(const rg_mesh_view* m, const double* tfluxes, int nt, double dt, double* tr_ext);
/* old cells / tracers: the state before the update (SkipUpdate keeps it);
 * tr_ext is updated in place for the entropy tracer */
int ro_cell_update_tr(const rg_mesh_view* m, const double* ext, double* tr_ext, const double* old_cells,
                      const double* old_tr, double gamma, const ro_tracers* t, double* cells_out,
                      double* tr_out, ro_error* err);
void ro_init_extensives_tr(const rg_mesh_view* m, const double* cells, const double* tr, int nt,
                           double* tr_ext);
/* hdsim::TimeAdvance on a fixed mesh with tracers and stickers */
int ro_step_tr(const rg_mesh_view* m, double* cells, double* ext, double* tr, double* tr_ext,
               const double* ev, double gamma, double cfl, int order, const ro_lgi_params* lp,
               const ro_tracers* t, double* dt_out, ro_error* err);
/* hdsim::TimeAdvance2Heun (hdsim2d.cpp:323-449) on a fixed mesh with tracers
 * and stickers: the cell updater's SkipUpdate keeps the step's old cells at
 * the midpoint and at the end, and its entropy tracer rewrites the tracer
 * extensive of the extensives it is given (mid, then the average) */
int ro_step_heun_tr(const rg_mesh_view* m, double* cells, double* ext, double* tr, double* tr_ext,
                    const double* ev, double gamma, double cfl, int order, const ro_lgi_params* lp,
                    const ro_tracers* t, double* dt_out, ro_error* err);

/* Geometry of a packed mesh from its points and face vertices, as the
 * reference's tessellation and CacheData compute it: volume (GetVolume), the
 * cell CMs of real cells (CalcCellCM) and ghosts (periodic shift or
 * reflection about the box side, box = {left, right, down, up}), cd_volume
 * (SlabSymmetry::calcVolume).  cm_xy holds (n_cells + n_ghosts)*2. */
void ro_cell_geometry(const rg_mesh_view* m, int ghost_kind, const double* box, double* volume, double* cm_xy,
                      double* cd_volume);

/* Condition/action flux schemes: ConditionActionSequence
 * (condition_action_sequence.cpp) and ConditionActionSequence2
 * (condition_action_sequence_2.cpp).  A rule: seq 0 (the first-order list,
 * evaluated first) or 1 (ConditionActionSequence2's list); cond 0
 * IsBoundaryEdge, 1 IsBulkEdge, 2 RegularSpecialEdge(sticker bit); action 0
 * RegularFlux, 1 RigidWallFlux, 2 FreeFlowFlux (cell states), 3 RegularFlux2,
 * 4 RigidWallFlux2, 5 Ratchet(in), 6 LagrangianFlux (LinearGaussImproved face
 * states, lp).  LagrangianFlux (condition_action_sequence_2.cpp:252-294) has
 * two LagrangianHLLC solvers, the first where WallsMassFlux holds (the face
 * is not a self-mirror), the second elsewhere; massflux bit 0 / bit 1 are
 * their LagrangianHLLC(massflux) flags.  lag_ws / lag_ev (NULL allowed)
 * receive the action's ws_ / edge_vel_ per face, zero for other actions. */
typedef struct ro_flux_rule {
  int32_t seq, cond, sticker, action, in, massflux;
} ro_flux_rule;
int ro_cas_flux(const rg_mesh_view* m, const double* cells, const double* ev, double gamma, int order,
                const ro_lgi_params* lp, const ro_flux_rule* rules, int n_rules, const uint32_t* stickers,
                double* fluxes, double* lag_ws, double* lag_ev, ro_error* err);
/* The same with tracers (t->n of them in tr, n_cells*n): tfluxes (n_faces*n)
 * receives each face's Mass times the tracers of the side its action takes,
 * the cell (RegularFlux: upwind; RigidWallFlux, FreeFlowFlux: the aux side)
 * or LinearGaussImproved's face value (RegularFlux2, LagrangianFlux: upwind;
 * RigidWallFlux2: the aux side), as conserved_to_extensive forms it. */
int ro_cas_flux_tr(const rg_mesh_view* m, const double* cells, const double* tr, const double* ev, double gamma,
                   int order, const ro_lgi_params* lp, const ro_tracers* t, const ro_flux_rule* rules, int n_rules,
                   const uint32_t* stickers, double* fluxes, double* tfluxes, double* lag_ws, double* lag_ev,
                   ro_error* err);
/* LagrangianExtensiveUpdater (LagrangianExtensiveUpdater.cpp:8-80) after the
 * base update: per cell dV = sum area*dt*edge_vel and dv_ws = sum area*dt*ws
 * over its faces (+ as the first neighbour, - as the second, in face order),
 * then every extensive times (V + dV) / (V + dV + dv_ws), V the CacheData
 * volume; areas NULL = the edge lengths (SlabSymmetry) */
void ro_lagrangian_update(const rg_mesh_view* m, const double* lag_ws, const double* lag_ev, double dt,
                          const double* areas, double* ext);
/* the same factor on the nt extensive tracers too (Extensive::operator*=) */
void ro_lagrangian_update_tr(const rg_mesh_view* m, const double* lag_ws, const double* lag_ev, double dt,
                             const double* areas, double* ext, double* tr_ext, int nt);
/* hdsim::TimeAdvance with a condition/action flux calculator on a fixed
 * mesh; cells with a bit of frozen_mask keep their state (SkipUpdate);
 * lagrangian_update: LagrangianExtensiveUpdater around SimpleExtensiveUpdater */
int ro_step_cas(const rg_mesh_view* m, double* cells, double* ext, const double* ev, double gamma, double cfl,
                int order, const ro_lgi_params* lp, const ro_flux_rule* rules, int n_rules, const uint32_t* stickers,
                uint32_t frozen_mask, int lagrangian_update, double* dt_out, ro_error* err);
/* ro_step_cas with tracers: the stickers, the calc_tracers mask and the
 * SkipUpdate sticker come from t */
int ro_step_cas_tr(const rg_mesh_view* m, double* cells, double* ext, double* tr, double* tr_ext, const double* ev,
                   double gamma, double cfl, int order, const ro_lgi_params* lp, const ro_flux_rule* rules,
                   int n_rules, const ro_tracers* t, int lagrangian_update, double* dt_out, ro_error* err);

/* CylindricalSymmetry (physical_geometry.cpp:62-110) about the axis through
 * origin along direction (normalised as Axis does): CacheData's face areas
 * (n_faces) and cell volumes (n_cells). */
void ro_cyl_geometry(const rg_mesh_view* m, const double* origin, const double* direction, double* areas,
                     double* volumes);
/* SimpleExtensiveUpdater with given face areas (CacheData::areas) */
void ro_extensive_update_areas(const rg_mesh_view* m, const double* fluxes, const double* areas, double dt,
                               double* ext);
/* ro_step with given face areas (the mesh's cd_volume holds the matching volumes) */
int ro_step_areas(const rg_mesh_view* m, double* cells, double* ext, const double* ev, double gamma, double cfl,
                  int order, const ro_lgi_params* lp, const double* areas, double* dt_out, ro_error* err);

/* Point motion and edge velocities (hdsim::TimeAdvance's first half). */
typedef struct ro_motion {
  int32_t kind;             /* 0 Eulerian, 1 Lagrangian, 2 RoundCells(Lagrangian) */
  int32_t edges;            /* 0 StationaryBox, 1 PeriodicEdgeVelocities */
  double chi, eta;          /* RoundCells parameters */
  int32_t cold;             /* RoundCells cold switch */
  int32_t correct_overshoot; /* RoundCells outer boundary is not periodic */
  double box[4];            /* RoundCells outer boundary {left, right, down, up} */
} ro_motion;
/* PointMotion::operator() for the n_cells points: pv n_cells*2 */
void ro_point_velocities(const rg_mesh_view* m, const double* cells, double gamma, const ro_motion* mo,
                         double* pv);
/* PointMotion::ApplyFix, in place */
void ro_apply_fix(const rg_mesh_view* m, const double* cells, double gamma, const ro_motion* mo, double dt,
                  double* pv);
/* EdgeVelocityCalculator::operator(): ev n_faces*2 */
void ro_edge_velocities(const rg_mesh_view* m, const ro_motion* mo, const double* pv, double* ev);

/* 3D first-order path on the packed 3D mesh.  Cells N*5 {density, pressure,
 * vx, vy, vz}; extensives and fluxes N*5 {mass, px, py, pz, energy}
 * (Conserved3D order).  face_velocity: n_faces*3 or NULL (faces at rest). */
void ro3_init_extensives(const rg_mesh3d_view* m, const double* cells, double gamma, double* ext);
double ro3_cfl(const rg_mesh3d_view* m, const double* cells, double gamma, double cfl);
int ro3_flux(const rg_mesh3d_view* m, const double* cells, const double* face_velocity, double gamma,
             double* fluxes, ro_error* err);
void ro3_extensive_update(const rg_mesh3d_view* m, const double* fluxes, double dt, double* ext);
int ro3_cell_update(const rg_mesh3d_view* m, const double* ext, double gamma, double* cells, ro_error* err);
/* HDSim3D::timeAdvance (hdsim_3d.cpp:133-145) on a fixed mesh */
int ro3_step(const rg_mesh3d_view* m, double* cells, double* ext, double gamma, double cfl, double* dt_out,
             ro_error* err);

#ifdef __cplusplus
}
#endif
#endif
