// ref_dump.cpp -- runs the reference RICH hot path on a seeded case and
// writes its inputs and outputs as .npy files, which
// tests/golden/make_golden.py bundles into tests/golden/<case>.npz.
//
// Test infrastructure only: it links the reference sources built by
// oracle/ref/Makefile and is never part of the product.
//
//   ref_dump <case> <outdir> <nx> <ny> <warm_steps> <run_steps> [heun]
//
// With "heun" the warm-up and run steps use hdsim::TimeAdvance2Heun
// (hdsim2d.cpp:323-449) instead of hdsim::TimeAdvance.
//
// Cases named <case>_tracers add tracers and stickers (the condition/action
// cases cas*_tracers: tracers {"A", "Z"} with "A" in calc_tracers, and the
// case's own stickers): tracer names
// {"A", "Entropy", "Z"} ("A" in LinearGaussImproved's calc_tracers,
// "Entropy" recomputed by SimpleCellUpdater, "Z" piecewise constant), sticker
// names {"frozen", "skip"} ("skip" is LinearGaussImproved's skip_key, cells
// with "frozen" keep their state through HasSticker + SkipUpdate), and dump
// the tracer / sticker arrays beside the others (tr_*).
//
// Cases mesh_rigid / mesh_periodic write only the packed tessellation of the
// points in <outdir>/points.f64 (box in <outdir>/box.f64): the pin of the
// test meshes' own tessellator (huji-rich_gb300/synthetic.py).
//
// For every other case it writes, for the state reached after <warm_steps>
// hdsim::TimeAdvance steps (hdsim2d.cpp:149-241):
//   mesh_*          the packed tessellation (huji-rich_gb300/host/rich_pack.hpp)
//   cells0, ext0    ComputationalCell / Extensive state
//   ev_cfl, dt      edge velocities given to SimpleCFL and its dt (hdsim2d.cpp:161-165)
//   ev_flux         edge velocities after PointMotion::ApplyFix (hdsim2d.cpp:167-174)
//   slopes, interp  LinearGaussImproved slopes and per-edge states (order 2)
//   fluxes          FluxCalculator output (hdsim2d.cpp:176-184)
//   ext1            after SimpleExtensiveUpdater (hdsim2d.cpp:188-195)
//   cells1          SimpleCellUpdater on ext1 with the same mesh
// and, when <run_steps> > 0, the state after that many further
// hdsim::TimeAdvance steps (run_cells, run_ext, run_time, run_times).
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <functional>
#include <memory>
#include <random>
#include <string>

#include "rich_pack.hpp"
#include "source/newtonian/common/LagrangianHLLC.hpp"
#include "source/newtonian/common/hllc.hpp"
#include "source/newtonian/common/ideal_gas.hpp"
#include "source/newtonian/two_dimensional/geometric_outer_boundaries/PeriodicBox.hpp"
#include "source/newtonian/two_dimensional/geometric_outer_boundaries/SquareBox.hpp"
#include "source/newtonian/two_dimensional/ghost_point_generators/PeriodicGhostGenerator.hpp"
#include "source/newtonian/two_dimensional/ghost_point_generators/RigidWallGenerator.hpp"
#include "source/newtonian/two_dimensional/condition_action_sequence.hpp"
#include "source/newtonian/two_dimensional/condition_action_sequence_2.hpp"
#include "source/newtonian/two_dimensional/hdsim2d.hpp"
#include "source/newtonian/two_dimensional/LagrangianExtensiveUpdater.hpp"
#include "source/newtonian/two_dimensional/interpolations/LinearGaussImproved.hpp"
#include "source/newtonian/two_dimensional/modular_flux_calculator.hpp"
#include "source/newtonian/two_dimensional/periodic_edge_velocities.hpp"
#include "source/newtonian/two_dimensional/point_motions/eulerian.hpp"
#include "source/newtonian/two_dimensional/point_motions/lagrangian.hpp"
#include "source/newtonian/two_dimensional/point_motions/round_cells.hpp"
#include "source/newtonian/two_dimensional/simple_cell_updater.hpp"
#include "source/newtonian/two_dimensional/simple_cfl.hpp"
#include "source/newtonian/two_dimensional/simple_extensive_updater.hpp"
#include "source/newtonian/two_dimensional/simple_flux_calculator.hpp"
#include "source/newtonian/two_dimensional/source_terms/zero_force.hpp"
#include "source/newtonian/two_dimensional/stationary_box.hpp"
#include "source/tessellation/VoronoiMesh.hpp"

namespace {

std::string g_out;
bool g_heun = false;
double g_box[4] = {0, 0, 0, 0};  // the OuterBoundary's (left, right, down, up)
// the case's point motion and edge velocities: kind (0 Eulerian, 1
// Lagrangian, 2 RoundCells(Lagrangian)), edges (0 StationaryBox, 1
// PeriodicEdgeVelocities), chi, eta, cold, CorrectPointsOverShoot active
double g_motion[6] = {0, 0, 0, 0, 0, 0};
// the PhysicalGeometry: kind (0 SlabSymmetry, 1 CylindricalSymmetry), axis origin, axis direction
double g_geometry[5] = {0, 0, 0, 0, 0};
// condition/action flux rules, one row each: sequence (0 ConditionActionSequence's
// first-order list, 1 ConditionActionSequence2's list), condition (0
// IsBoundaryEdge, 1 IsBulkEdge, 2 RegularSpecialEdge), sticker bit, action (0
// RegularFlux, 1 RigidWallFlux, 2 FreeFlowFlux, 3 RegularFlux2, 4
// RigidWallFlux2, 5 Ratchet, 6 LagrangianFlux), Ratchet's `in`, LagrangianFlux's
// massflux bits (bit 0 its first LagrangianHLLC's, bit 1 its second's)
std::vector<int32_t> g_rules;
// the case's LagrangianFlux: its per-face ws_ / edge_vel_ are dumped after
// the flux pass (LagrangianExtensiveUpdater reads and resets them)
const LagrangianFlux* g_lflux = nullptr;

void advance(hdsim& sim) {
  if (g_heun)
    sim.TimeAdvance2Heun();
  else
    sim.TimeAdvance();
}

void write_npy(const std::string& name, const char* descr, size_t elem, const void* data,
               size_t rows, size_t cols) {
  std::string path = g_out + "/" + name + ".npy";
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("cannot open " + path);
  char shape[64];
  if (cols == 0)
    std::snprintf(shape, sizeof shape, "(%zu,)", rows);
  else
    std::snprintf(shape, sizeof shape, "(%zu, %zu)", rows, cols);
  std::string hdr = std::string("{'descr': '") + descr + "', 'fortran_order': False, 'shape': " +
                    shape + ", }";
  while ((10 + hdr.size() + 1) % 64 != 0) hdr += ' ';
  hdr += '\n';
  const unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
  std::fwrite(magic, 1, 8, f);
  const uint16_t hl = static_cast<uint16_t>(hdr.size());
  std::fwrite(&hl, 2, 1, f);
  std::fwrite(hdr.data(), 1, hdr.size(), f);
  std::fwrite(data, elem, rows * (cols ? cols : 1), f);
  std::fclose(f);
}

void dump_f64(const std::string& n, const std::vector<double>& v, size_t cols) {
  write_npy(n, "<f8", 8, v.data(), cols ? v.size() / cols : v.size(), cols);
}
void dump_i32(const std::string& n, const std::vector<int32_t>& v, size_t cols) {
  write_npy(n, "<i4", 4, v.data(), cols ? v.size() / cols : v.size(), cols);
}
void dump_scalar(const std::string& n, double x) { write_npy(n, "<f8", 8, &x, 1, 0); }

std::vector<double> cells_flat(const std::vector<ComputationalCell>& c) {
  std::vector<double> r;
  for (const auto& x : c) {
    r.push_back(x.density);
    r.push_back(x.pressure);
    r.push_back(x.velocity.x);
    r.push_back(x.velocity.y);
  }
  return r;
}
std::vector<double> ext_flat(const std::vector<Extensive>& e) {
  std::vector<double> r;
  for (const auto& x : e) {
    r.push_back(x.mass);
    r.push_back(x.energy);
    r.push_back(x.momentum.x);
    r.push_back(x.momentum.y);
  }
  return r;
}
std::vector<double> tracers_flat(const std::vector<ComputationalCell>& c) {
  std::vector<double> r;
  for (const auto& x : c)
    for (double t : x.tracers) r.push_back(t);
  return r;
}
std::vector<double> ext_tracers_flat(const std::vector<Extensive>& e) {
  std::vector<double> r;
  for (const auto& x : e)
    for (double t : x.tracers) r.push_back(t);
  return r;
}
size_t g_ntr = 0;

std::vector<double> vec_flat(const std::vector<Vector2D>& v) {
  std::vector<double> r;
  for (const auto& x : v) {
    r.push_back(x.x);
    r.push_back(x.y);
  }
  return r;
}

void dump_mesh(const std::string& prefix, const Tessellation& tess, const PhysicalGeometry& pg) {
  CacheData cd(tess, pg);
  rich_gb300::PackedMesh m;
  rich_gb300::pack_tessellation(tess, cd, m);
  std::vector<double> areas;
  for (size_t e = 0; e < tess.getAllEdges().size(); ++e) areas.push_back(cd.areas[e]);
  dump_f64(prefix + "cd_area", areas, 0);
  dump_f64(prefix + "point_xy", m.point_xy, 2);
  dump_f64(prefix + "cm_xy", m.cm_xy, 2);
  dump_f64(prefix + "volume", m.volume, 0);
  dump_f64(prefix + "cd_volume", m.cd_volume, 0);
  dump_i32(prefix + "ghost_source", m.ghost_source, 0);
  dump_i32(prefix + "ghost_face", m.ghost_face, 0);
  dump_i32(prefix + "face_cells", m.face_cells, 2);
  dump_f64(prefix + "face_vertices", m.face_vertices, 4);
  dump_i32(prefix + "cell_face_offset", m.cell_face_offset, 0);
  dump_i32(prefix + "cell_faces", m.cell_faces, 0);
}

std::vector<Vector2D> jittered_lattice(int nx, int ny, double x0, double x1, double y0, double y1,
                                       unsigned seed, double jitter) {
  std::mt19937_64 gen(seed);
  std::uniform_real_distribution<double> u(-jitter, jitter);
  std::vector<Vector2D> r;
  const double dx = (x1 - x0) / nx, dy = (y1 - y0) / ny;
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j) {
      const double ux = u(gen), uy = u(gen);
      r.push_back(Vector2D(x0 + (i + 0.5 + ux) * dx, y0 + (j + 0.5 + uy) * dy));
    }
  return r;
}

// One hot-path pass on a fixed mesh, in hdsim::TimeAdvance's order.
void dump_components(hdsim& sim, const PhysicalGeometry& pg, const EquationOfState& eos,
                     const PointMotion& pm, const EdgeVelocityCalculator& evc,
                     const TimeStepFunction& tsf, const FluxCalculator& fc,
                     const ExtensiveUpdater& eu, const CellUpdater& cu,
                     const LinearGaussImproved* lgi) {
  const Tessellation& tess = sim.getTessellation();
  const vector<ComputationalCell>& cells = sim.getAllCells();
  const vector<Extensive>& ext = sim.getAllExtensives();
  const TracerStickerNames& tsn = sim.GetTracerStickerNames();
  const double t = sim.getTime();
  dump_mesh("mesh_", tess, pg);
  dump_f64("cells0", cells_flat(cells), 4);
  dump_f64("ext0", ext_flat(ext), 4);
  if (g_ntr) {
    dump_f64("tr_cells0", tracers_flat(cells), g_ntr);
    dump_f64("tr_ext0", ext_tracers_flat(ext), g_ntr);
    std::vector<int32_t> st;
    for (const auto& c : cells) {
      int32_t bits = 0;
      for (size_t k = 0; k < c.stickers.size(); ++k) bits |= c.stickers[k] ? (1 << k) : 0;
      st.push_back(bits);
    }
    dump_i32("tr_stickers", st, 0);
  }
  dump_scalar("time0", t);
  dump_f64("outer_box", std::vector<double>(g_box, g_box + 4), 0);
  dump_f64("motion", std::vector<double>(g_motion, g_motion + 6), 0);
  dump_f64("geometry", std::vector<double>(g_geometry, g_geometry + 5), 0);
  if (!g_rules.empty()) dump_i32("flux_rules", g_rules, 6);
  vector<Vector2D> pv = pm(tess, cells, t, tsn);
  vector<Vector2D> ev = evc(tess, pv);
  const double dt = tsf(tess, cells, eos, ev, t, tsn);
  dump_f64("pv_cfl", vec_flat(pv), 2);
  dump_f64("ev_cfl", vec_flat(ev), 2);
  dump_scalar("dt", dt);
  pv = pm.ApplyFix(tess, cells, t, dt, pv, tsn);
  ev = evc(tess, pv);
  dump_f64("pv_flux", vec_flat(pv), 2);
  dump_f64("ev_flux", vec_flat(ev), 2);
  CacheData cd(tess, pg);
  if (lgi) {
    vector<pair<ComputationalCell, ComputationalCell> > interp(
        static_cast<size_t>(tess.GetTotalSidesNumber()),
        pair<ComputationalCell, ComputationalCell>(cells[0], cells[0]));
    (*lgi)(tess, cells, t, interp, tsn, cd);
    std::vector<double> sl, ip;
    for (const Slope& s : lgi->GetSlopes()) {
      for (const ComputationalCell* c : {&s.xderivative, &s.yderivative}) {
        sl.push_back(c->density);
        sl.push_back(c->pressure);
        sl.push_back(c->velocity.x);
        sl.push_back(c->velocity.y);
      }
    }
    for (const auto& pr : interp)
      for (const ComputationalCell* c : {&pr.first, &pr.second}) {
        ip.push_back(c->density);
        ip.push_back(c->pressure);
        ip.push_back(c->velocity.x);
        ip.push_back(c->velocity.y);
      }
    dump_f64("slopes", sl, 8);
    dump_f64("interp", ip, 8);
    if (g_ntr) {
      std::vector<double> tsl, tip;
      for (const Slope& s : lgi->GetSlopes()) {
        for (double t : s.xderivative.tracers) tsl.push_back(t);
        for (double t : s.yderivative.tracers) tsl.push_back(t);
      }
      for (const auto& pr : interp) {
        for (double t : pr.first.tracers) tip.push_back(t);
        for (double t : pr.second.tracers) tip.push_back(t);
      }
      dump_f64("tr_slopes", tsl, 2 * g_ntr);
      dump_f64("tr_interp", tip, 2 * g_ntr);
    }
  }
  const vector<Extensive> fl = fc(tess, ev, cells, ext, cd, eos, t, dt, tsn);
  dump_f64("fluxes", ext_flat(fl), 4);
  if (g_lflux) {
    dump_f64("lag_ws", g_lflux->ws_, 0);
    dump_f64("lag_ev", g_lflux->edge_vel_, 0);
  }
  vector<Extensive> ext1 = ext;
  eu(fl, pg, tess, dt, cd, cells, ext1, t, tsn);
  dump_f64("ext1", ext_flat(ext1), 4);
  if (g_ntr) {
    dump_f64("tr_fluxes", ext_tracers_flat(fl), g_ntr);
    dump_f64("tr_ext1", ext_tracers_flat(ext1), g_ntr);
  }
  const vector<ComputationalCell> cells1 = cu(tess, pg, eos, ext1, cells, cd, tsn);
  dump_f64("cells1", cells_flat(cells1), 4);
  if (g_ntr) {
    dump_f64("tr_cells1", tracers_flat(cells1), g_ntr);
    dump_f64("tr_ext1b", ext_tracers_flat(ext1), g_ntr);  // after the cell updater (entropy tracer)
  }
}

void run_and_dump(hdsim& sim, int steps, const PhysicalGeometry& pg = SlabSymmetry()) {
  // hdsim keeps time_ += dt (hdsim2d.cpp:238); the sequence of times pins
  // every dt without the rounding of a difference.
  std::vector<double> times;
  for (int s = 0; s < steps; ++s) {
    advance(sim);
    times.push_back(sim.getTime());
  }
  dump_f64("run_cells", cells_flat(sim.getAllCells()), 4);
  dump_f64("run_ext", ext_flat(sim.getAllExtensives()), 4);
  if (g_ntr) {
    dump_f64("tr_run_cells", tracers_flat(sim.getAllCells()), g_ntr);
    dump_f64("tr_run_ext", ext_tracers_flat(sim.getAllExtensives()), g_ntr);
  }
  dump_scalar("run_time", sim.getTime());
  dump_f64("run_times", times, 0);
  dump_mesh("runmesh_", sim.getTessellation(), pg);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 7) {
    std::fprintf(stderr, "usage: ref_dump <case> <outdir> <nx> <ny> <warm> <run>\n");
    return 2;
  }
  std::string which = argv[1];
  const std::string sfx = "_tracers";
  const bool tracers = which.size() > sfx.size() && which.compare(which.size() - sfx.size(), sfx.size(), sfx) == 0;
  if (tracers) {
    which = which.substr(0, which.size() - sfx.size());
    g_ntr = 3;
  }
  // the condition/action cases' tracer forms carry two plain tracers {"A",
  // "Z"} ("A" in LinearGaussImproved's calc_tracers) and the case's own
  // stickers
  const bool cas_case = which.compare(0, 3, "cas") == 0;
  if (tracers && cas_case) g_ntr = 2;
  const vector<string> cas_calc = tracers ? vector<string>{"A"} : vector<string>();
  auto cas_tracers = [&](vector<ComputationalCell>& ic, const Tessellation& tess) {
    if (!tracers) return;
    for (size_t i = 0; i < ic.size(); ++i) {
      const Vector2D r = tess.GetMeshPoint(static_cast<int>(i));
      ic[i].tracers = {r.x + (r.y > 0.4 ? 0.5 : 0.0), abs(r - Vector2D(0.3, 0.3)) < 0.2 ? 1.0 : 0.0};
    }
  };
  // tracer / sticker setup of the _tracers cases (names sorted, as the
  // reference's binary_find lookups need)
  const TracerStickerNames tsn = tracers ? TracerStickerNames({"A", "Entropy", "Z"}, {"frozen", "skip"})
                                         : TracerStickerNames();
  const vector<string> calc_tracers = tracers ? vector<string>{"A"} : vector<string>();
  const string skip_key = tracers ? "skip" : "";
  // frozen_r: stickers only on cells at least this far from the origin (a
  // frozen or limiter-skipped cell next to a blast drives the state there to
  // negative pressure, which the reference asserts on)
  auto add_tracers = [&](vector<ComputationalCell>& ic, const Tessellation& tess, double gamma,
                         double frozen_r = 0.0) {
    if (!tracers) return;
    for (size_t i = 0; i < ic.size(); ++i) {
      const Vector2D r = tess.GetMeshPoint(static_cast<int>(i));
      ic[i].tracers = {r.x + (r.y > 0.1 ? 0.5 : 0.0), ic[i].pressure * std::pow(ic[i].density, -gamma),
                       abs(r) < 0.3 ? 1.0 : 0.0};
      const size_t h = std::hash<size_t>()(i * 2654435761u);
      ic[i].stickers = {h % 17 == 3 && abs(r) >= frozen_r, h % 11 == 5 && abs(r) >= frozen_r};
    }
  };
  g_out = argv[2];
  const int nx = std::atoi(argv[3]), ny = std::atoi(argv[4]);
  const int warm = std::atoi(argv[5]), run = std::atoi(argv[6]);
  g_heun = argc > 7 && std::string(argv[7]) == "heun";
  try {
    if (which == "mesh_rigid" || which == "mesh_periodic") {
      // The packed tessellation of given points: <outdir>/points.f64 holds
      // nx*ny (x, y) pairs and <outdir>/box.f64 the box (x0, x1, y0, y1); the
      // VoronoiMesh keeps the input order (no Hilbert reordering), so its
      // cells are numbered as the points are.
      std::vector<double> xy(2 * static_cast<size_t>(nx) * ny), box(4);
      for (int k = 0; k < 2; ++k) {
        std::vector<double>& dst = k == 0 ? xy : box;
        const std::string path = g_out + (k == 0 ? "/points.f64" : "/box.f64");
        FILE* f = std::fopen(path.c_str(), "rb");
        const bool ok = f && std::fread(dst.data(), sizeof(double), dst.size(), f) == dst.size();
        if (f) std::fclose(f);
        if (!ok) throw std::runtime_error("cannot read " + path);
      }
      std::vector<Vector2D> pts(xy.size() / 2);
      for (size_t i = 0; i < pts.size(); ++i) pts[i] = Vector2D(xy[2 * i], xy[2 * i + 1]);
      SlabSymmetry pg;
      std::unique_ptr<OuterBoundary> outer;
      if (which == "mesh_rigid")
        outer.reset(new SquareBox(Vector2D(box[0], box[2]), Vector2D(box[1], box[3])));
      else
        outer.reset(new PeriodicBox(box[0], box[1], box[3], box[2]));
      VoronoiMesh tess(pts, *outer, false);
      dump_mesh("mesh_", tess, pg);
      return 0;
    }
    SlabSymmetry pg;
    Hllc rs;
    ZeroForce force;
    SimpleCFL tsf(0.3);
    SimpleExtensiveUpdater eu;
    vector<pair<const SimpleCellUpdater::Condition*, const SimpleCellUpdater::Action*> > seq;
    if (tracers && !cas_case) seq.push_back({new HasSticker("frozen"), new SkipUpdate()});
    SimpleCellUpdater cu(seq);
    if (which == "sod" || which == "sod_lagrangian") {
      // 2D Sod tube: [0,1]x[0,0.2], reflective walls, piecewise-constant Hllc, gamma 1.4.
      SquareBox outer(Vector2D(0, 0), Vector2D(1, 0.2));
      g_box[0] = 0, g_box[1] = 1, g_box[2] = 0, g_box[3] = 0.2;
      VoronoiMesh tess(jittered_lattice(nx, ny, 0, 1, 0, 0.2, 1, 1e-3), outer);
      IdealGas eos(1.4);
      Eulerian eul;
      Lagrangian lag;
      const PointMotion& pm = which == "sod" ? static_cast<const PointMotion&>(eul)
                                             : static_cast<const PointMotion&>(lag);
      StationaryBox evc;
      g_motion[0] = which == "sod" ? 0 : 1;
      SimpleFluxCalculator fc(rs);
      vector<ComputationalCell> ic(static_cast<size_t>(tess.GetPointNo()));
      for (size_t i = 0; i < ic.size(); ++i) {
        const bool left = tess.GetMeshPoint(static_cast<int>(i)).x < 0.5;
        ic[i].density = left ? 1 : 0.125;
        ic[i].pressure = left ? 1 : 0.1;
      }
      add_tracers(ic, tess, 1.4);
      hdsim sim(tess, outer, pg, ic, eos, pm, evc, force, tsf, fc, eu, cu, tsn);
      for (int s = 0; s < warm; ++s) advance(sim);
      dump_scalar("gamma", 1.4);
      dump_scalar("order", 1);
      dump_scalar("ghost_kind", 0);
      dump_components(sim, pg, eos, pm, evc, tsf, fc, eu, cu, nullptr);
      if (run > 0) run_and_dump(sim, run);
    } else if (which == "sedov" || which == "sedov_eulerian") {
      // Sedov-Taylor on [-1,1]^2, RoundCells(Lagrangian) (or Eulerian),
      // LinearGaussImproved + rigid walls.
      SquareBox outer(Vector2D(-1, -1), Vector2D(1, 1));
      g_box[0] = -1, g_box[1] = 1, g_box[2] = -1, g_box[3] = 1;
      VoronoiMesh tess(jittered_lattice(nx, ny, -1, 1, -1, 1, 2, 1e-3), outer);
      IdealGas eos(5. / 3.);
      Lagrangian lag;
      RoundCells round(lag, eos);
      Eulerian eul;
      const PointMotion& pm = which == "sedov" ? static_cast<const PointMotion&>(round)
                                               : static_cast<const PointMotion&>(eul);
      StationaryBox evc;
      // RoundCells(lag, eos): chi 0.15, eta 0.02, hot, periodic default outer (no overshoot fix)
      if (which == "sedov") g_motion[0] = 2, g_motion[2] = 0.15, g_motion[3] = 0.02;
      RigidWallGenerator gpg;
      LinearGaussImproved sr(eos, gpg, true, 0.2, 0.5, 0.7, calc_tracers, skip_key);
      ModularFluxCalculator fc(sr, rs);
      const double dx = 2.0 / nx;
      const double rdep = std::max(0.02, 1.5 * dx);
      double vin = 0;
      for (int i = 0; i < tess.GetPointNo(); ++i)
        if (abs(tess.GetMeshPoint(i)) < rdep) vin += tess.GetVolume(i);
      vector<ComputationalCell> ic(static_cast<size_t>(tess.GetPointNo()));
      for (size_t i = 0; i < ic.size(); ++i) {
        ic[i].density = 1;
        ic[i].pressure = abs(tess.GetMeshPoint(static_cast<int>(i))) < rdep ? (5. / 3. - 1) / vin : 1e-6;
      }
      add_tracers(ic, tess, 5. / 3., 0.6);
      hdsim sim(tess, outer, pg, ic, eos, pm, evc, force, tsf, fc, eu, cu, tsn);
      for (int s = 0; s < warm; ++s) advance(sim);
      dump_scalar("gamma", 5. / 3.);
      dump_scalar("order", 2);
      dump_scalar("ghost_kind", 0);
      dump_components(sim, pg, eos, pm, evc, tsf, fc, eu, cu, &sr);
      if (run > 0) run_and_dump(sim, run);
    } else if (which == "periodic" || which == "periodic_lagrangian") {
      // Periodic [0,1]^2, LinearGaussImproved + PeriodicGhostGenerator, smooth bumps + velocity modes.
      PeriodicBox outer(0, 1, 1, 0);
      g_box[0] = 0, g_box[1] = 1, g_box[2] = 0, g_box[3] = 1;
      VoronoiMesh tess(jittered_lattice(nx, ny, 0, 1, 0, 1, 3, 1e-3), outer);
      IdealGas eos(5. / 3.);
      Eulerian eul;
      Lagrangian lag;
      const PointMotion& pm = which == "periodic" ? static_cast<const PointMotion&>(eul)
                                                  : static_cast<const PointMotion&>(lag);
      PeriodicEdgeVelocities evc;
      g_motion[0] = which == "periodic" ? 0 : 1;
      g_motion[1] = 1;
      PeriodicGhostGenerator gpg;
      LinearGaussImproved sr(eos, gpg, true, 0.2, 0.5, 0.7, calc_tracers, skip_key);
      ModularFluxCalculator fc(sr, rs);
      std::mt19937_64 gen(7);
      std::uniform_real_distribution<double> u01(0, 1);
      double bx[8], by[8], bw[8];
      for (int k = 0; k < 8; ++k) {
        bx[k] = u01(gen);
        by[k] = u01(gen);
        bw[k] = 0.02 + 0.08 * u01(gen);
      }
      vector<ComputationalCell> ic(static_cast<size_t>(tess.GetPointNo()));
      const double pi2 = 2 * M_PI;
      for (size_t i = 0; i < ic.size(); ++i) {
        const Vector2D r = tess.GetMeshPoint(static_cast<int>(i));
        double rho = 1;
        for (int k = 0; k < 8; ++k) {
          const double ddx = r.x - bx[k], ddy = r.y - by[k];
          rho += 0.1 * std::exp(-(ddx * ddx + ddy * ddy) / (bw[k] * bw[k]));
        }
        ic[i].density = rho;
        ic[i].pressure = 1;
        ic[i].velocity = Vector2D(0.1 * std::sin(pi2 * (r.x + 2 * r.y)), 0.1 * std::cos(pi2 * (2 * r.x - r.y)));
      }
      add_tracers(ic, tess, 5. / 3.);
      hdsim sim(tess, outer, pg, ic, eos, pm, evc, force, tsf, fc, eu, cu, tsn);
      for (int s = 0; s < warm; ++s) advance(sim);
      dump_scalar("gamma", 5. / 3.);
      dump_scalar("order", 2);
      dump_scalar("ghost_kind", 1);
      dump_components(sim, pg, eos, pm, evc, tsf, fc, eu, cu, &sr);
      if (run > 0) run_and_dump(sim, run);
    } else if (which == "cas_free" || which == "cas2_wall" || which == "cas2_ratchet") {
      // Condition/action flux schemes on [0,1]^2 with reflecting-wall ghosts:
      //  cas_free: ConditionActionSequence (first order) {(IsBoundaryEdge,
      //    FreeFlowFlux), (RegularSpecialEdge("obstacle"), RigidWallFlux),
      //    (IsBulkEdge, RegularFlux)}, a diagonal Sod problem around an
      //    obstacle disc;
      //  cas2_wall: ConditionActionSequence2 {} then {(IsBoundaryEdge,
      //    RigidWallFlux2), (RegularSpecialEdge("obstacle"), RigidWallFlux2),
      //    (IsBulkEdge, RegularFlux2)} with LinearGaussImproved, flow past an
      //    obstacle disc (RegularSpecialEdge reads both neighbours' cells, so
      //    boundary edges are matched first);
      //  cas2_ratchet: ConditionActionSequence2 {} then {(IsBoundaryEdge,
      //    Ratchet(out)), (IsBulkEdge, RegularFlux2)}, a blast venting through
      //    the walls.
      SquareBox outer(Vector2D(0, 0), Vector2D(1, 1));
      g_box[0] = 0, g_box[1] = 1, g_box[2] = 0, g_box[3] = 1;
      VoronoiMesh tess(jittered_lattice(nx, ny, 0, 1, 0, 1, 6, 1e-3), outer);
      IdealGas eos(5. / 3.);
      Eulerian eul;
      StationaryBox evc;
      RigidWallGenerator gpg;
      LinearGaussImproved sr(eos, gpg, true, 0.2, 0.5, 0.7, cas_calc);
      typedef ConditionActionSequence CAS;
      vector<pair<const CAS::Condition*, const CAS::Action*> > seq1;
      vector<pair<const CAS::Condition*, const ConditionActionSequence2::Action2*> > seq2;
      const bool first = which == "cas_free";
      if (first) {
        seq1.push_back({new IsBoundaryEdge(), new FreeFlowFlux(rs)});
        seq1.push_back({new RegularSpecialEdge("obstacle"), new RigidWallFlux(rs)});
        seq1.push_back({new IsBulkEdge(), new RegularFlux(rs)});
        g_rules = {0, 0, -1, 2, 0, 0, 0, 2, 0, 1, 0, 0, 0, 1, -1, 0, 0, 0};
      } else if (which == "cas2_wall") {
        seq2.push_back({new IsBoundaryEdge(), new RigidWallFlux2(rs)});
        seq2.push_back({new RegularSpecialEdge("obstacle"), new RigidWallFlux2(rs)});
        seq2.push_back({new IsBulkEdge(), new RegularFlux2(rs)});
        g_rules = {1, 0, -1, 4, 0, 0, 1, 2, 0, 4, 0, 0, 1, 1, -1, 3, 0, 0};
      } else {
        seq2.push_back({new IsBoundaryEdge(), new Ratchet(rs, false)});
        seq2.push_back({new IsBulkEdge(), new RegularFlux2(rs)});
        g_rules = {1, 0, -1, 5, 0, 0, 1, 1, -1, 3, 0, 0};
      }
      CAS fc1(seq1);
      ConditionActionSequence2 fc2(seq1, seq2, sr);
      const FluxCalculator& fc = first ? static_cast<const FluxCalculator&>(fc1)
                                       : static_cast<const FluxCalculator&>(fc2);
      const bool obstacle = which != "cas2_ratchet";
      const vector<string> tnames = tracers ? vector<string>{"A", "Z"} : vector<string>();
      const TracerStickerNames names = obstacle ? TracerStickerNames(tnames, {"obstacle"}) : TracerStickerNames(tnames, {});
      vector<ComputationalCell> ic(static_cast<size_t>(tess.GetPointNo()));
      for (size_t i = 0; i < ic.size(); ++i) {
        const Vector2D r = tess.GetMeshPoint(static_cast<int>(i));
        if (first) {
          const bool left = r.x + r.y < 1;
          ic[i].density = left ? 1 : 0.125;
          ic[i].pressure = left ? 1 : 0.1;
          ic[i].stickers = {abs(r - Vector2D(0.6, 0.6)) < 0.12};
        } else if (which == "cas2_wall") {
          ic[i].density = 1;
          ic[i].pressure = 1;
          ic[i].velocity = Vector2D(0.6, 0.1);
          ic[i].stickers = {abs(r - Vector2D(0.45, 0.5)) < 0.15};
        } else {
          ic[i].density = 1;
          ic[i].pressure = abs(r - Vector2D(0.5, 0.5)) < 0.2 ? 5.0 : 0.5;
          ic[i].velocity = Vector2D(0.3 * (r.x - 0.5), 0.3 * (r.y - 0.5));
        }
      }
      cas_tracers(ic, tess);
      // obstacle cells keep their state (HasSticker + SkipUpdate)
      vector<pair<const SimpleCellUpdater::Condition*, const SimpleCellUpdater::Action*> > keep;
      if (obstacle) keep.push_back({new HasSticker("obstacle"), new SkipUpdate()});
      SimpleCellUpdater ocu(keep);
      hdsim sim(tess, outer, pg, ic, eos, eul, evc, force, tsf, fc, eu, ocu, names);
      for (int s = 0; s < warm; ++s) advance(sim);
      dump_scalar("gamma", 5. / 3.);
      dump_scalar("order", first ? 1 : 2);
      dump_scalar("ghost_kind", 0);
      if (obstacle && !g_ntr) {
        std::vector<int32_t> st;
        for (const auto& c : sim.getAllCells()) st.push_back(c.stickers[0] ? 1 : 0);
        dump_i32("tr_stickers", st, 0);
      }
      dump_components(sim, pg, eos, eul, evc, tsf, fc, eu, ocu, first ? nullptr : &sr);
      if (run > 0) run_and_dump(sim, run);
    } else if (which == "cas2_lag" || which == "cas2_lag_move") {
      // LagrangianFlux (condition_action_sequence_2.cpp:252-294) with
      // LinearGaussImproved face states and two LagrangianHLLC solvers
      // chosen by WallsMassFlux, and LagrangianExtensiveUpdater around
      // SimpleExtensiveUpdater, on [0,1]^2 with reflecting walls:
      //  cas2_lag: Eulerian; {(IsBoundaryEdge, RigidWallFlux2),
      //    (IsBulkEdge, LagrangianFlux(LagrangianHLLC(false), LagrangianHLLC(true)))};
      //  cas2_lag_move: Lagrangian point motion; {(IsBulkEdge, LagrangianFlux),
      //    (IsBoundaryEdge, LagrangianFlux)} with LagrangianHLLC(true),
      //    LagrangianHLLC(false) (the wall faces take the second: WallsMassFlux
      //    is false where a ghost mirrors its cell).
      SquareBox outer(Vector2D(0, 0), Vector2D(1, 1));
      g_box[0] = 0, g_box[1] = 1, g_box[2] = 0, g_box[3] = 1;
      VoronoiMesh tess(jittered_lattice(nx, ny, 0, 1, 0, 1, 8, 1e-3), outer);
      IdealGas eos(5. / 3.);
      const bool move = which == "cas2_lag_move";
      Eulerian eul;
      Lagrangian lag;
      const PointMotion& pm = move ? static_cast<const PointMotion&>(lag) : static_cast<const PointMotion&>(eul);
      g_motion[0] = move ? 1 : 0;
      StationaryBox evc;
      RigidWallGenerator gpg;
      LinearGaussImproved sr(eos, gpg, true, 0.2, 0.5, 0.7, cas_calc);
      LagrangianHLLC lrs1(move), lrs2(!move);  // massflux: false, true (cas2_lag); true, false (cas2_lag_move)
      WallsMassFlux walls;
      LagrangianFlux lflux(lrs1, lrs2, walls);
      g_lflux = &lflux;
      typedef ConditionActionSequence CAS;
      vector<pair<const CAS::Condition*, const CAS::Action*> > seq1;
      vector<pair<const CAS::Condition*, const ConditionActionSequence2::Action2*> > seq2;
      if (!move) {
        seq2.push_back({new IsBoundaryEdge(), new RigidWallFlux2(rs)});
        seq2.push_back({new IsBulkEdge(), &lflux});
        g_rules = {1, 0, -1, 4, 0, 0, 1, 1, -1, 6, 0, 2};
      } else {
        seq2.push_back({new IsBulkEdge(), &lflux});
        seq2.push_back({new IsBoundaryEdge(), &lflux});
        g_rules = {1, 1, -1, 6, 0, 1, 1, 0, -1, 6, 0, 1};
      }
      ConditionActionSequence2 fc(seq1, seq2, sr);
      SimpleExtensiveUpdater beu;
      LagrangianExtensiveUpdater leu(lflux, beu);
      vector<ComputationalCell> ic(static_cast<size_t>(tess.GetPointNo()));
      for (size_t i = 0; i < ic.size(); ++i) {
        const Vector2D r = tess.GetMeshPoint(static_cast<int>(i));
        ic[i].density = 1 + 0.3 * std::sin(6.283185307179586 * (r.x + 0.5 * r.y));
        ic[i].pressure = abs(r - Vector2D(0.4, 0.55)) < 0.15 ? 4.0 : 0.6;
        ic[i].velocity = Vector2D(0.25 * std::cos(6.283185307179586 * r.y), -0.15 * std::sin(6.283185307179586 * r.x));
      }
      cas_tracers(ic, tess);
      const TracerStickerNames lnames(tracers ? vector<string>{"A", "Z"} : vector<string>(), {});
      hdsim sim(tess, outer, pg, ic, eos, pm, evc, force, tsf, fc, leu, cu, lnames);
      for (int s = 0; s < warm; ++s) advance(sim);
      dump_scalar("gamma", 5. / 3.);
      dump_scalar("order", 2);
      dump_scalar("ghost_kind", 0);
      dump_scalar("lagrangian_updater", 1);
      dump_components(sim, pg, eos, pm, evc, tsf, fc, leu, cu, &sr);
      if (run > 0) run_and_dump(sim, run);
      g_lflux = nullptr;
    } else if (which == "cyl_blast") {
      // Cylindrical symmetry about the y axis (r = x) on [0,1]^2: a blast at
      // the origin corner, Eulerian, LinearGaussImproved + rigid walls; the
      // PhysicalGeometry gives CacheData's face areas and cell volumes
      // (physical_geometry.cpp:62-110) and the complementary source term is
      // not applied (ZeroForce).
      SquareBox outer(Vector2D(0, 0), Vector2D(1, 1));
      g_box[0] = 0, g_box[1] = 1, g_box[2] = 0, g_box[3] = 1;
      CylindricalSymmetry cpg(Vector2D(0, 0), Vector2D(0, 1));
      g_geometry[0] = 1, g_geometry[1] = 0, g_geometry[2] = 0, g_geometry[3] = 0, g_geometry[4] = 1;
      VoronoiMesh tess(jittered_lattice(nx, ny, 0, 1, 0, 1, 5, 1e-3), outer);
      IdealGas eos(5. / 3.);
      Eulerian eul;
      StationaryBox evc;
      RigidWallGenerator gpg;
      LinearGaussImproved sr(eos, gpg);
      ModularFluxCalculator fc(sr, rs);
      vector<ComputationalCell> ic(static_cast<size_t>(tess.GetPointNo()));
      for (size_t i = 0; i < ic.size(); ++i) {
        const Vector2D r = tess.GetMeshPoint(static_cast<int>(i));
        ic[i].density = 1 + 0.3 * r.y;
        ic[i].pressure = abs(r) < 0.15 ? 10.0 : 0.1;
        ic[i].velocity = Vector2D(0.05 * r.y, -0.05 * r.x);
      }
      hdsim sim(tess, outer, cpg, ic, eos, eul, evc, force, tsf, fc, eu, cu);
      for (int s = 0; s < warm; ++s) advance(sim);
      dump_scalar("gamma", 5. / 3.);
      dump_scalar("order", 2);
      dump_scalar("ghost_kind", 0);
      dump_components(sim, cpg, eos, eul, evc, tsf, fc, eu, cu, &sr);
      if (run > 0) run_and_dump(sim, run, cpg);
    } else if (which == "wallflow_cold") {
      // Fast flow into the walls of [0,1]^2 on a RoundCells(Lagrangian, cold)
      // mesh with the box as its outer boundary: RoundCells::ApplyFix's
      // calc_dw(dt) and CorrectPointsOverShoot (round_cells.cpp:15-63,
      // 96-134) act; LinearGaussImproved + rigid walls.
      SquareBox outer(Vector2D(0, 0), Vector2D(1, 1));
      g_box[0] = 0, g_box[1] = 1, g_box[2] = 0, g_box[3] = 1;
      // some points of the last column and the last row close to the right
      // and upper walls, where the flow would carry them out of the box
      std::vector<Vector2D> pts = jittered_lattice(nx, ny, 0, 1, 0, 1, 4, 1e-3);
      const double hx = 1.0 / nx, hy = 1.0 / ny;
      for (int j = 0; j < ny; ++j) {
        Vector2D& q = pts[static_cast<size_t>((nx - 1) * ny + j)];
        if (j % 6 == 1) q.x = 1 - 0.02 * hx;
        if (j % 6 == 4) q.x = 1 - 0.12 * hx;
      }
      for (int i = 0; i < nx - 1; ++i) {
        Vector2D& q = pts[static_cast<size_t>(i * ny + ny - 1)];
        if (i % 5 == 2) q.y = 1 - 0.03 * hy;
        if (i % 5 == 0) q.y = 1 - 0.15 * hy;
      }
      VoronoiMesh tess(pts, outer);
      IdealGas eos(5. / 3.);
      Lagrangian lag;
      RoundCells round(lag, eos, outer, 0.15, 0.02, true);
      StationaryBox evc;
      g_motion[0] = 2, g_motion[2] = 0.15, g_motion[3] = 0.02, g_motion[4] = 1, g_motion[5] = 1;
      RigidWallGenerator gpg;
      LinearGaussImproved sr(eos, gpg);
      ModularFluxCalculator fc(sr, rs);
      vector<ComputationalCell> ic(static_cast<size_t>(tess.GetPointNo()));
      for (size_t i = 0; i < ic.size(); ++i) {
        const Vector2D r = tess.GetMeshPoint(static_cast<int>(i));
        ic[i].density = 1 + 0.2 * std::sin(6 * r.x) * std::cos(5 * r.y);
        ic[i].pressure = 0.01;
        ic[i].velocity = Vector2D(1.0 + 0.2 * std::sin(7 * r.y), 0.6 - 0.3 * std::cos(4 * r.x));
      }
      hdsim sim(tess, outer, pg, ic, eos, round, evc, force, tsf, fc, eu, cu);
      for (int s = 0; s < warm; ++s) advance(sim);
      dump_scalar("gamma", 5. / 3.);
      dump_scalar("order", 2);
      dump_scalar("ghost_kind", 0);
      dump_components(sim, pg, eos, round, evc, tsf, fc, eu, cu, &sr);
      if (run > 0) run_and_dump(sim, run);
    } else {
      std::fprintf(stderr, "unknown case %s\n", which.c_str());
      return 2;
    }
  } catch (UniversalError const& eo) {
    std::fprintf(stderr, "UniversalError: %s\n", eo.GetErrorMessage().c_str());
    for (size_t i = 0; i < eo.GetFields().size(); ++i)
      std::fprintf(stderr, "  %s = %.17g\n", eo.GetFields()[i].c_str(), eo.GetValues()[i]);
    return 1;
  }
  return 0;
}
