// hdsim_dropin.cpp -- hdsim driven through the GPU plugins, beside hdsim
// driven through the reference's own plugins.
//
// Test driver only: it links the reference's sources (built by
// oracle/ref/Makefile) and the product library librich_gb300.so through the
// adapters in huji-rich_gb300/host/rich_gpu_adapters.hpp, exactly as a RICH
// simulation would use them: the driver builds two (or three) complete
// simulations -- tessellation, outer boundary, point motion, edge
// velocities, source term, and the plugin set -- and calls
// hdsim::TimeAdvance / TimeAdvance2Heun (hdsim2d.cpp:149-241, 323-449) on
// each.  The stock set is SimpleCFL, SimpleFluxCalculator or
// ModularFluxCalculator(LinearGaussImproved, Hllc), SimpleExtensiveUpdater
// and SimpleCellUpdater; the GPU set is GpuCFL, GpuFluxCalculator,
// GpuExtensiveUpdater and GpuCellUpdater over one GpuContext.  Nothing else
// differs: the host rebuilds each simulation's Voronoi mesh in
// MoveMeshPoints and moves its points as the reference does.
//
//   hdsim_dropin compare <case> <n> <steps> [hostgeom]
//       stock and GPU FP64 simulations in lockstep; after every step the
//       cells, extensives (with tracers), mesh points and time of the two
//       are compared with == (the "Entropy" tracer within 1e-15 relative);
//       prints one JSON line (first differing step, counts).  The GPU
//       plugins form volumes and CMs on the device unless "hostgeom" is
//       given, which uploads the host tessellation's and CacheData's.
//   hdsim_dropin accuracy <case> <n> <steps> [stock]
//       GPU FP64 and GPU FP32-mixed simulations in lockstep (and, with
//       "stock", the stock one in a child process at the same time, whose
//       state hash after every step is compared with the FP64 one's); prints
//       the density L1 of FP32-mixed against FP64 (and of both against
//       stock) at the end, cells matched by mesh point (the runs' points
//       differ slightly, and so may their order).
//   hdsim_dropin sensitivity <case> <n> <steps> <delta> <every>
//       the problem's own sensitivity, on the CPU: the stock simulation
//       against the stock simulation from initial densities perturbed by a
//       relative delta; density L1 and relative time difference every
//       `every` steps.
//   hdsim_dropin time <case> <n> <steps> <set>
//       one simulation (set = stock | gpu | gpu32): wall time per step and
//       the time spent inside the four plugin calls, the rest being the
//       host's point motion, edge velocities and Voronoi rebuild.
//
// Cases:
//   sod       Sod tube [0,1]x[0,0.2], 5n x n jittered lattice, rigid walls,
//             Eulerian, first order (SimpleFluxCalculator), gamma 1.4
//   sedov     Sedov-Taylor on [-1,1]^2, n x n, RoundCells(Lagrangian),
//             LinearGaussImproved + RigidWallGenerator, gamma 5/3
//   periodic  periodic [0,1]^2, n x n, Eulerian, LinearGaussImproved +
//             PeriodicGhostGenerator, PeriodicEdgeVelocities,
//             TimeAdvance2Heun
//   tracers   the sedov case with tracers {"A", "Entropy", "Z"} and stickers
//             {"frozen", "skip"} (LinearGaussImproved's calc_tracers {"A"}
//             and skip_key "skip"; HasSticker("frozen") + SkipUpdate)
//   cas       the sedov case with ConditionActionSequence2 {(IsBoundaryEdge,
//             RigidWallFlux2), (IsBulkEdge, RegularFlux2)} as the flux
//             calculator (the GPU set: the same rule table) and tracers
//             {"A", "Z"} ("A" in calc_tracers); FP64 only
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include <sys/wait.h>
#include <unistd.h>

#include "rich_gpu_adapters.hpp"
#include "source/newtonian/common/hllc.hpp"
#include "source/newtonian/common/ideal_gas.hpp"
#include "source/newtonian/two_dimensional/condition_action_sequence.hpp"
#include "source/newtonian/two_dimensional/condition_action_sequence_2.hpp"
#include "source/newtonian/two_dimensional/geometric_outer_boundaries/PeriodicBox.hpp"
#include "source/newtonian/two_dimensional/geometric_outer_boundaries/SquareBox.hpp"
#include "source/newtonian/two_dimensional/ghost_point_generators/PeriodicGhostGenerator.hpp"
#include "source/newtonian/two_dimensional/ghost_point_generators/RigidWallGenerator.hpp"
#include "source/newtonian/two_dimensional/hdsim2d.hpp"
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

double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Seconds spent inside each plugin call of one simulation.
struct PluginClock {
  double tsf = 0, fc = 0, eu = 0, cu = 0;
  double total() const { return tsf + fc + eu + cu; }
};

// Forwarding plugins that time the wrapped one (the same wrappers go around
// both plugin sets).
class TimedTSF : public TimeStepFunction {
 public:
  TimedTSF(const TimeStepFunction& in, double& acc) : in_(in), acc_(acc) {}
  double operator()(const Tessellation& t, const vector<ComputationalCell>& c, const EquationOfState& e,
                    const vector<Vector2D>& ev, const double time, TracerStickerNames const& n) const override {
    const double t0 = now();
    const double r = in_(t, c, e, ev, time, n);
    acc_ += now() - t0;
    return r;
  }

 private:
  const TimeStepFunction& in_;
  double& acc_;
};

class TimedFC : public FluxCalculator {
 public:
  TimedFC(const FluxCalculator& in, double& acc) : in_(in), acc_(acc) {}
  vector<Extensive> operator()(const Tessellation& t, const vector<Vector2D>& ev, const vector<ComputationalCell>& c,
                               const vector<Extensive>& x, const CacheData& cd, const EquationOfState& e,
                               const double time, const double dt, TracerStickerNames const& n) const override {
    const double t0 = now();
    vector<Extensive> r = in_(t, ev, c, x, cd, e, time, dt, n);
    acc_ += now() - t0;
    return r;
  }

 private:
  const FluxCalculator& in_;
  double& acc_;
};

class TimedEU : public ExtensiveUpdater {
 public:
  TimedEU(const ExtensiveUpdater& in, double& acc) : in_(in), acc_(acc) {}
  void operator()(const vector<Extensive>& f, const PhysicalGeometry& pg, const Tessellation& t, const double dt,
                  const CacheData& cd, const vector<ComputationalCell>& c, vector<Extensive>& x, double time,
                  TracerStickerNames const& n) const override {
    const double t0 = now();
    in_(f, pg, t, dt, cd, c, x, time, n);
    acc_ += now() - t0;
  }

 private:
  const ExtensiveUpdater& in_;
  double& acc_;
};

class TimedCU : public CellUpdater {
 public:
  TimedCU(const CellUpdater& in, double& acc) : in_(in), acc_(acc) {}
  vector<ComputationalCell> operator()(const Tessellation& t, const PhysicalGeometry& pg, const EquationOfState& e,
                                       vector<Extensive>& x, const vector<ComputationalCell>& old,
                                       const CacheData& cd, TracerStickerNames const& n) const override {
    const double t0 = now();
    vector<ComputationalCell> r = in_(t, pg, e, x, old, cd, n);
    acc_ += now() - t0;
    return r;
  }

 private:
  const CellUpdater& in_;
  double& acc_;
};

std::vector<Vector2D> jittered_lattice(int nx, int ny, double x0, double x1, double y0, double y1, unsigned seed) {
  std::mt19937_64 gen(seed);
  std::uniform_real_distribution<double> u(-1e-3, 1e-3);
  std::vector<Vector2D> r;
  const double dx = (x1 - x0) / nx, dy = (y1 - y0) / ny;
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j) {
      const double ux = u(gen), uy = u(gen);
      r.push_back(Vector2D(x0 + (i + 0.5 + ux) * dx, y0 + (j + 0.5 + uy) * dy));
    }
  return r;
}

// Tracer compared within a relative tolerance instead of ==: the "Entropy"
// tracer, which SimpleCellUpdater recomputes as p * pow(d, -gamma)
// (simple_cell_updater.cpp:44-48) with the host's libm pow and the GPU with
// the device pow (a few ulp apart); -1 = none.  Nothing else reads it.
int g_entropy = -1;
double g_entropy_max_rel = 0;
const double kEntropyRel = 1e-15;

enum Set { kStock = 0, kGpu64 = 1, kGpu32 = 2 };

// One complete simulation: everything hdsim holds by reference lives here.
struct Sim {
  PluginClock clock;
  bool heun = false;
  std::unique_ptr<OuterBoundary> outer;
  std::unique_ptr<VoronoiMesh> tess;
  SlabSymmetry pg;
  std::unique_ptr<IdealGas> eos;
  Hllc rs;
  Eulerian eul;
  Lagrangian lag;
  std::unique_ptr<RoundCells> round;
  std::unique_ptr<EdgeVelocityCalculator> evc;
  ZeroForce force;
  std::unique_ptr<GhostPointGenerator> ghosts;
  std::unique_ptr<LinearGaussImproved> sr;
  // the cas case's conditions and actions (ConditionActionSequence2 keeps
  // pointers to them)
  std::unique_ptr<ConditionActionSequence::Condition> c_bnd, c_bulk;
  std::unique_ptr<ConditionActionSequence2::Action2> a_wall, a_reg;
  // stock plugins
  std::unique_ptr<SimpleCFL> s_tsf;
  std::unique_ptr<FluxCalculator> s_fc;
  SimpleExtensiveUpdater s_eu;
  std::unique_ptr<SimpleCellUpdater> s_cu;
  // GPU plugins
  std::unique_ptr<rich_gb300::GpuContext> ctx;
  std::unique_ptr<rich_gb300::GpuCFL> g_tsf;
  std::unique_ptr<rich_gb300::GpuFluxCalculator> g_fc;
  std::unique_ptr<rich_gb300::GpuExtensiveUpdater> g_eu;
  std::unique_ptr<rich_gb300::GpuCellUpdater> g_cu;
  // timing wrappers around whichever set is active
  std::unique_ptr<TimedTSF> t_tsf;
  std::unique_ptr<TimedFC> t_fc;
  std::unique_ptr<TimedEU> t_eu;
  std::unique_ptr<TimedCU> t_cu;
  std::unique_ptr<hdsim> sim;

  void advance() {
    if (heun)
      sim->TimeAdvance2Heun();
    else
      sim->TimeAdvance();
  }
};

// The GPU plugins form volumes and CMs on the device (the adapters'
// set_outer_boundary); false: the host packs the tessellation's and
// CacheData's own.
bool g_device_geometry = true;
// Relative perturbation of the initial densities (sensitivity mode): cell i
// gets density * (1 + delta * u_i), u_i uniform in [-1, 1] from a fixed seed.
double g_perturb = 0;

std::unique_ptr<Sim> make_sim(const std::string& which, int n, Set set) {
  std::unique_ptr<Sim> s(new Sim);
  const bool tracers = which == "tracers";
  const bool cas = which == "cas";
  g_entropy = tracers ? 1 : -1;  // sorted names {"A", "Entropy", "Z"}
  const std::string base = tracers || cas ? "sedov" : which;
  const TracerStickerNames tsn = tracers ? TracerStickerNames({"A", "Entropy", "Z"}, {"frozen", "skip"})
                                 : cas   ? TracerStickerNames({"A", "Z"}, {})
                                         : TracerStickerNames();
  const vector<string> calc_tracers = tracers || cas ? vector<string>{"A"} : vector<string>();
  const string skip_key = tracers ? "skip" : "";
  vector<pair<const SimpleCellUpdater::Condition*, const SimpleCellUpdater::Action*> > seq;
  if (tracers) seq.push_back({new HasSticker("frozen"), new SkipUpdate()});
  s->s_cu.reset(new SimpleCellUpdater(seq));
  s->s_tsf.reset(new SimpleCFL(0.3));

  rg_config cfg;
  rg_default_config(&cfg);
  cfg.precision = set == kGpu32 ? RG_FP32_MIXED : RG_FP64;
  rich_gb300::GpuTracerSpec spec;
  spec.calc_tracers = calc_tracers;
  spec.skip_key = skip_key;
  spec.frozen_sticker = tracers ? "frozen" : "";

  const PointMotion* pm = &s->eul;
  vector<ComputationalCell> ic;
  double gamma = 5.0 / 3.0;
  if (base == "sod") {
    s->outer.reset(new SquareBox(Vector2D(0, 0), Vector2D(1, 0.2)));
    s->tess.reset(new VoronoiMesh(jittered_lattice(5 * n, n, 0, 1, 0, 0.2, 1), *s->outer));
    gamma = 1.4;
    s->eos.reset(new IdealGas(gamma));
    s->evc.reset(new StationaryBox());
    s->s_fc.reset(new SimpleFluxCalculator(s->rs));
    cfg.order = 1;
    ic.resize(static_cast<size_t>(s->tess->GetPointNo()));
    for (size_t i = 0; i < ic.size(); ++i) {
      const bool left = s->tess->GetMeshPoint(static_cast<int>(i)).x < 0.5;
      ic[i].density = left ? 1 : 0.125;
      ic[i].pressure = left ? 1 : 0.1;
    }
  } else if (base == "sedov") {
    s->outer.reset(new SquareBox(Vector2D(-1, -1), Vector2D(1, 1)));
    s->tess.reset(new VoronoiMesh(jittered_lattice(n, n, -1, 1, -1, 1, 2), *s->outer));
    s->eos.reset(new IdealGas(gamma));
    s->round.reset(new RoundCells(s->lag, *s->eos));
    pm = s->round.get();
    s->evc.reset(new StationaryBox());
    s->ghosts.reset(new RigidWallGenerator());
    s->sr.reset(new LinearGaussImproved(*s->eos, *s->ghosts, true, 0.2, 0.5, 0.7, calc_tracers, skip_key));
    if (cas) {
      s->c_bnd.reset(new IsBoundaryEdge());
      s->c_bulk.reset(new IsBulkEdge());
      s->a_wall.reset(new RigidWallFlux2(s->rs));
      s->a_reg.reset(new RegularFlux2(s->rs));
      const vector<pair<const ConditionActionSequence::Condition*, const ConditionActionSequence::Action*> > seq1;
      const vector<pair<const ConditionActionSequence::Condition*, const ConditionActionSequence2::Action2*> > seq2 = {
          {s->c_bnd.get(), s->a_wall.get()}, {s->c_bulk.get(), s->a_reg.get()}};
      s->s_fc.reset(new ConditionActionSequence2(seq1, seq2, *s->sr));
    } else {
      s->s_fc.reset(new ModularFluxCalculator(*s->sr, s->rs));
    }
    cfg.order = 2;
    cfg.ghost_kind = RG_GHOST_RIGID_WALL;
    const double rdep = std::max(0.02, 1.5 * 2.0 / n);
    double vin = 0;
    for (int i = 0; i < s->tess->GetPointNo(); ++i)
      if (abs(s->tess->GetMeshPoint(i)) < rdep) vin += s->tess->GetVolume(i);
    ic.resize(static_cast<size_t>(s->tess->GetPointNo()));
    for (size_t i = 0; i < ic.size(); ++i) {
      ic[i].density = 1;
      ic[i].pressure = abs(s->tess->GetMeshPoint(static_cast<int>(i))) < rdep ? (gamma - 1) / vin : 1e-6;
    }
    if (cas)
      for (size_t i = 0; i < ic.size(); ++i) {
        const Vector2D r = s->tess->GetMeshPoint(static_cast<int>(i));
        ic[i].tracers = {r.x + (r.y > 0.1 ? 0.5 : 0.0), abs(r) < 0.3 ? 1.0 : 0.0};
      }
    if (tracers)
      for (size_t i = 0; i < ic.size(); ++i) {
        const Vector2D r = s->tess->GetMeshPoint(static_cast<int>(i));
        ic[i].tracers = {r.x + (r.y > 0.1 ? 0.5 : 0.0), ic[i].pressure * std::pow(ic[i].density, -gamma),
                         abs(r) < 0.3 ? 1.0 : 0.0};
        const size_t h = std::hash<size_t>()(i * 2654435761u);
        ic[i].stickers = {h % 17 == 3 && abs(r) >= 0.6, h % 11 == 5 && abs(r) >= 0.6};
      }
  } else if (base == "periodic") {
    s->heun = true;
    s->outer.reset(new PeriodicBox(0, 1, 1, 0));
    s->tess.reset(new VoronoiMesh(jittered_lattice(n, n, 0, 1, 0, 1, 3), *s->outer));
    s->eos.reset(new IdealGas(gamma));
    s->evc.reset(new PeriodicEdgeVelocities());
    s->ghosts.reset(new PeriodicGhostGenerator());
    s->sr.reset(new LinearGaussImproved(*s->eos, *s->ghosts, true, 0.2, 0.5, 0.7));
    s->s_fc.reset(new ModularFluxCalculator(*s->sr, s->rs));
    cfg.order = 2;
    cfg.ghost_kind = RG_GHOST_PERIODIC;
    std::mt19937_64 gen(7);
    std::uniform_real_distribution<double> u01(0, 1);
    double bx[8], by[8], bw[8];
    for (int k = 0; k < 8; ++k) {
      bx[k] = u01(gen);
      by[k] = u01(gen);
      bw[k] = 0.02 + 0.08 * u01(gen);
    }
    ic.resize(static_cast<size_t>(s->tess->GetPointNo()));
    const double pi2 = 2 * M_PI;
    for (size_t i = 0; i < ic.size(); ++i) {
      const Vector2D r = s->tess->GetMeshPoint(static_cast<int>(i));
      double rho = 1;
      for (int k = 0; k < 8; ++k) {
        const double ddx = r.x - bx[k], ddy = r.y - by[k];
        rho += 0.1 * std::exp(-(ddx * ddx + ddy * ddy) / (bw[k] * bw[k]));
      }
      ic[i].density = rho;
      ic[i].pressure = 1;
      ic[i].velocity = Vector2D(0.1 * std::sin(pi2 * (r.x + 2 * r.y)), 0.1 * std::cos(pi2 * (2 * r.x - r.y)));
    }
  } else {
    throw std::runtime_error("unknown case " + which);
  }
  if (g_perturb != 0) {
    std::mt19937_64 gen(99);
    std::uniform_real_distribution<double> u(-1, 1);
    for (ComputationalCell& c : ic) c.density *= 1 + g_perturb * u(gen);
  }
  cfg.gamma = gamma;
  cfg.time_integrator = s->heun ? RG_TIME_ADVANCE_HEUN : RG_TIME_ADVANCE;

  const TimeStepFunction* tsf = s->s_tsf.get();
  const FluxCalculator* fc = s->s_fc.get();
  const ExtensiveUpdater* eu = &s->s_eu;
  const CellUpdater* cu = s->s_cu.get();
  if (set != kStock) {
    s->ctx.reset(new rich_gb300::GpuContext(cfg, spec));
    if (g_device_geometry) s->ctx->set_outer_boundary(*s->outer);
    if (cas) {
      if (set == kGpu32) throw std::runtime_error("the cas case runs the FP64 plugins only");
      // {sequence, condition, sticker, action, ratchet_in, massflux}
      s->ctx->set_flux_rules({{1, RG_COND_BOUNDARY_EDGE, -1, RG_ACT_RIGID_WALL2, 0, 0},
                              {1, RG_COND_BULK_EDGE, -1, RG_ACT_REGULAR2, 0, 0}});
    }
    s->g_tsf.reset(new rich_gb300::GpuCFL(*s->ctx));
    s->g_fc.reset(new rich_gb300::GpuFluxCalculator(*s->ctx));
    s->g_eu.reset(new rich_gb300::GpuExtensiveUpdater(*s->ctx));
    s->g_cu.reset(new rich_gb300::GpuCellUpdater(*s->ctx));
    tsf = s->g_tsf.get();
    fc = s->g_fc.get();
    eu = s->g_eu.get();
    cu = s->g_cu.get();
  }
  s->t_tsf.reset(new TimedTSF(*tsf, s->clock.tsf));
  s->t_fc.reset(new TimedFC(*fc, s->clock.fc));
  s->t_eu.reset(new TimedEU(*eu, s->clock.eu));
  s->t_cu.reset(new TimedCU(*cu, s->clock.cu));
  s->sim.reset(new hdsim(*s->tess, *s->outer, s->pg, ic, *s->eos, *pm, *s->evc, s->force, *s->t_tsf, *s->t_fc,
                         *s->t_eu, *s->t_cu, tsn));
  return s;
}

// IEEE == of two doubles, with NaN equal to NaN (a NaN on both sides is the
// same failure; on one side only it is a difference)
bool same(double a, double b) { return a == b || (std::isnan(a) && std::isnan(b)); }

bool same_tracer(size_t j, double a, double b) {
  if (static_cast<int>(j) != g_entropy) return same(a, b);
  if (same(a, b)) return true;
  const double rel = std::fabs(a - b) / std::max(std::fabs(a), std::fabs(b));
  g_entropy_max_rel = std::max(g_entropy_max_rel, rel);
  return rel <= kEntropyRel;
}

// Number of differing values between the two simulations' cells,
// extensives (tracers included), mesh points and time.
size_t count_differences(const hdsim& a, const hdsim& b) {
  const vector<ComputationalCell>& ca = a.getAllCells();
  const vector<ComputationalCell>& cb = b.getAllCells();
  const vector<Extensive>& ea = a.getAllExtensives();
  const vector<Extensive>& eb = b.getAllExtensives();
  if (ca.size() != cb.size() || ea.size() != eb.size()) return static_cast<size_t>(-1);
  size_t d = same(a.getTime(), b.getTime()) ? 0 : 1;
  for (size_t i = 0; i < ca.size(); ++i) {
    d += !same(ca[i].density, cb[i].density) + !same(ca[i].pressure, cb[i].pressure) +
         !same(ca[i].velocity.x, cb[i].velocity.x) + !same(ca[i].velocity.y, cb[i].velocity.y);
    if (ca[i].tracers.size() != cb[i].tracers.size() || ca[i].stickers != cb[i].stickers) ++d;
    for (size_t j = 0; j < ca[i].tracers.size() && j < cb[i].tracers.size(); ++j)
      d += !same_tracer(j, ca[i].tracers[j], cb[i].tracers[j]);
  }
  for (size_t i = 0; i < ea.size(); ++i) {
    d += !same(ea[i].mass, eb[i].mass) + !same(ea[i].energy, eb[i].energy) +
         !same(ea[i].momentum.x, eb[i].momentum.x) + !same(ea[i].momentum.y, eb[i].momentum.y);
    if (ea[i].tracers.size() != eb[i].tracers.size()) ++d;
    for (size_t j = 0; j < ea[i].tracers.size() && j < eb[i].tracers.size(); ++j)
      d += !same_tracer(j, ea[i].tracers[j], eb[i].tracers[j]);
  }
  // the meshes the next step starts from
  const Tessellation& ta = a.getTessellation();
  const Tessellation& tb = b.getTessellation();
  if (ta.GetPointNo() != tb.GetPointNo()) return d + 1;
  for (int i = 0; i < ta.GetPointNo(); ++i)
    d += !same(ta.GetMeshPoint(i).x, tb.GetMeshPoint(i).x) + !same(ta.GetMeshPoint(i).y, tb.GetMeshPoint(i).y);
  return d;
}

// Mesh points, densities and time of a simulation.
// Mesh points, densities, tracers (cell-major, nt per cell) and time of a
// simulation.
struct Snapshot {
  std::vector<double> xy, rho, tr;
  size_t nt = 0;
  double time = 0;
};

Snapshot snapshot(const hdsim& a) {
  Snapshot r;
  const Tessellation& t = a.getTessellation();
  const vector<ComputationalCell>& c = a.getAllCells();
  r.nt = c.empty() ? 0 : c[0].tracers.size();
  for (int i = 0; i < t.GetPointNo(); ++i) {
    r.xy.push_back(t.GetMeshPoint(i).x);
    r.xy.push_back(t.GetMeshPoint(i).y);
    r.rho.push_back(c[static_cast<size_t>(i)].density);
    for (size_t j = 0; j < r.nt; ++j) r.tr.push_back(c[static_cast<size_t>(i)].tracers[j]);
  }
  r.time = a.getTime();
  return r;
}

// FNV-1a over the bit patterns of every cell and extensive value (tracers
// included), mesh point and the time, with -0 taken as +0: equal states
// (in the sense of count_differences without tolerances) hash equally.
uint64_t state_hash(const hdsim& a) {
  uint64_t h = 1469598103934665603ull;
  auto add = [&h](double x) {
    x = x + 0.0;  // -0 -> +0
    uint64_t b;
    std::memcpy(&b, &x, 8);
    for (int k = 0; k < 8; ++k) {
      h ^= (b >> (8 * k)) & 0xffu;
      h *= 1099511628211ull;
    }
  };
  for (const ComputationalCell& c : a.getAllCells()) {
    add(c.density), add(c.pressure), add(c.velocity.x), add(c.velocity.y);
    for (double t : c.tracers) add(t);
  }
  for (const Extensive& e : a.getAllExtensives()) {
    add(e.mass), add(e.energy), add(e.momentum.x), add(e.momentum.y);
    for (double t : e.tracers) add(t);
  }
  const Tessellation& t = a.getTessellation();
  for (int i = 0; i < t.GetPointNo(); ++i) add(t.GetMeshPoint(i).x), add(t.GetMeshPoint(i).y);
  add(a.getTime());
  return h;
}

// Density L1 of `a` against `b`, relative to b's, each cell of `a` matched
// with the cell of `b` whose mesh point is nearest (a grid of buckets over
// b's points; the runs' points differ by far less than a cell).
// column -1: density; j >= 0: tracer j
double density_l1(const Snapshot& a, const Snapshot& b, size_t* unmatched, int column = -1) {
  const size_t na = a.rho.size(), nb = b.rho.size();
  double x0 = 1e300, x1 = -1e300, y0 = 1e300, y1 = -1e300;
  for (size_t i = 0; i < nb; ++i) {
    x0 = std::min(x0, b.xy[2 * i]), x1 = std::max(x1, b.xy[2 * i]);
    y0 = std::min(y0, b.xy[2 * i + 1]), y1 = std::max(y1, b.xy[2 * i + 1]);
  }
  const int g = std::max(1, static_cast<int>(std::sqrt(static_cast<double>(nb))));
  const double hx = (x1 - x0) / g + 1e-300, hy = (y1 - y0) / g + 1e-300;
  std::vector<std::vector<size_t>> bucket(static_cast<size_t>(g) * g);
  auto cell_of = [&](double px, double py, int& bx, int& by) {
    bx = std::min(g - 1, std::max(0, static_cast<int>((px - x0) / hx)));
    by = std::min(g - 1, std::max(0, static_cast<int>((py - y0) / hy)));
  };
  for (size_t i = 0; i < nb; ++i) {
    int bx, by;
    cell_of(b.xy[2 * i], b.xy[2 * i + 1], bx, by);
    bucket[static_cast<size_t>(by) * g + bx].push_back(i);
  }
  double num = 0, den = 0;
  *unmatched = 0;
  for (size_t i = 0; i < na; ++i) {
    const double px = a.xy[2 * i], py = a.xy[2 * i + 1];
    int bx, by;
    size_t best = nb;
    double bd = 1e300;
    cell_of(px, py, bx, by);
    for (int yy = std::max(0, by - 1); yy <= std::min(g - 1, by + 1); ++yy)
      for (int xx = std::max(0, bx - 1); xx <= std::min(g - 1, bx + 1); ++xx)
        for (size_t j : bucket[static_cast<size_t>(yy) * g + xx]) {
          const double d = std::hypot(b.xy[2 * j] - px, b.xy[2 * j + 1] - py);
          if (d < bd) bd = d, best = j;
        }
    if (best == nb) {
      ++*unmatched;
      continue;
    }
    const double va = column < 0 ? a.rho[i] : a.tr[i * a.nt + static_cast<size_t>(column)];
    const double vb = column < 0 ? b.rho[best] : b.tr[best * b.nt + static_cast<size_t>(column)];
    num += std::fabs(va - vb);
    den += std::fabs(vb);
  }
  return num / den;
}

// Writes / reads a block of bytes through a pipe.
bool write_all(int fd, const void* p, size_t n) {
  const char* c = static_cast<const char*>(p);
  while (n > 0) {
    const ssize_t k = ::write(fd, c, n);
    if (k <= 0) return false;
    c += k, n -= static_cast<size_t>(k);
  }
  return true;
}
bool read_all(int fd, void* p, size_t n) {
  char* c = static_cast<char*>(p);
  while (n > 0) {
    const ssize_t k = ::read(fd, c, n);
    if (k <= 0) return false;
    c += k, n -= static_cast<size_t>(k);
  }
  return true;
}

void print_clock(const char* name, const Sim& s, int steps, double wall) {
  std::printf("\"%s\": {\"ms_per_step\": %.6f, \"plugin_ms_per_step\": %.6f, \"cfl_ms\": %.6f, \"flux_ms\": %.6f, "
              "\"extensive_update_ms\": %.6f, \"cell_update_ms\": %.6f, \"host_rest_ms_per_step\": %.6f}",
              name, 1e3 * wall / steps, 1e3 * s.clock.total() / steps, 1e3 * s.clock.tsf / steps,
              1e3 * s.clock.fc / steps, 1e3 * s.clock.eu / steps, 1e3 * s.clock.cu / steps,
              1e3 * (wall - s.clock.total()) / steps);
}

int usage() {
  std::fprintf(stderr,
               "usage: hdsim_dropin compare <case> <n> <steps>\n"
               "       hdsim_dropin accuracy <case> <n> <steps> [stock]\n"
               "       hdsim_dropin sensitivity <case> <n> <steps> <delta> <every>\n"
               "       hdsim_dropin time <case> <n> <steps> <stock|gpu|gpu32>\n");
  return 2;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 5) return usage();
  for (int k = 5; k < argc; ++k)
    if (std::string(argv[k]) == "hostgeom") g_device_geometry = false;
  const std::string mode = argv[1], which = argv[2];
  const int n = std::atoi(argv[3]), steps = std::atoi(argv[4]);
  try {
    if (mode == "compare") {
      std::unique_ptr<Sim> a = make_sim(which, n, kStock);
      std::unique_ptr<Sim> b = make_sim(which, n, kGpu64);
      int first_diff = -1;
      size_t diffs = count_differences(*a->sim, *b->sim);
      if (diffs) first_diff = 0;
      double wa = 0, wb = 0;
      for (int k = 1; k <= steps && first_diff < 0; ++k) {
        double t0 = now();
        a->advance();
        wa += now() - t0;
        t0 = now();
        b->advance();
        wb += now() - t0;
        diffs = count_differences(*a->sim, *b->sim);
        if (diffs) first_diff = k;
      }
      std::printf("{\"mode\": \"compare\", \"case\": \"%s\", \"n\": %d, \"cells\": %d, \"steps\": %d, "
                  "\"time\": %.17g, \"cycle\": %d, \"equal\": %s, \"first_differing_step\": %d, "
                  "\"differing_values\": %zu, \"device_geometry\": %s, \"entropy_max_rel_diff\": %.3e, ",
                  which.c_str(), n, a->tess->GetPointNo(), steps, b->sim->getTime(), b->sim->getCycle(),
                  first_diff < 0 ? "true" : "false", first_diff, diffs, g_device_geometry ? "true" : "false",
                  g_entropy_max_rel);
      print_clock("stock", *a, steps, wa);
      std::printf(", ");
      print_clock("gpu", *b, steps, wb);
      std::printf("}\n");
      return first_diff < 0 ? 0 : 1;
    }
    if (mode == "accuracy") {
      const bool stock = argc > 5 && std::string(argv[5]) == "stock";
      // The stock simulation runs in a child process forked before any CUDA
      // call (it never touches the GPU), concurrently with the two GPU
      // ones; it sends back its per-step state hashes, final points and
      // densities, and its timings.
      int fds[2] = {-1, -1};
      pid_t child = -1;
      if (stock) {
        if (pipe(fds) != 0) throw std::runtime_error("pipe failed");
        child = fork();
        if (child < 0) throw std::runtime_error("fork failed");
        if (child == 0) {
          ::close(fds[0]);
          int rc = 0;
          try {
            std::unique_ptr<Sim> ref = make_sim(which, n, kStock);
            std::vector<uint64_t> hashes;
            const double t0 = now();
            for (int k = 1; k <= steps; ++k) {
              ref->advance();
              hashes.push_back(state_hash(*ref->sim));
            }
            const double wall = now() - t0;
            const Snapshot sn = snapshot(*ref->sim);
            const uint64_t np = sn.rho.size();
            const double clk[6] = {wall, ref->clock.tsf, ref->clock.fc, ref->clock.eu, ref->clock.cu, sn.time};
            if (!write_all(fds[1], hashes.data(), 8 * hashes.size()) || !write_all(fds[1], &np, 8) ||
                !write_all(fds[1], sn.xy.data(), 16 * np) || !write_all(fds[1], sn.rho.data(), 8 * np) ||
                !write_all(fds[1], clk, sizeof clk))
              rc = 4;
          } catch (...) {
            rc = 5;
          }
          ::close(fds[1]);
          _exit(rc);
        }
        ::close(fds[1]);
      }
      std::unique_ptr<Sim> g64 = make_sim(which, n, kGpu64);
      std::unique_ptr<Sim> g32 = make_sim(which, n, kGpu32);
      std::vector<uint64_t> h64;
      double w64 = 0, w32 = 0;
      for (int k = 1; k <= steps; ++k) {
        double t0 = now();
        g64->advance();
        w64 += now() - t0;
        t0 = now();
        g32->advance();
        w32 += now() - t0;
        if (stock) h64.push_back(state_hash(*g64->sim));
      }
      const Snapshot s64 = snapshot(*g64->sim), s32 = snapshot(*g32->sim);
      size_t un32 = 0, un64 = 0;
      const double l1_32 = density_l1(s32, s64, &un32);
      double l1_tr = 0;  // the largest tracer column's
      for (size_t j = 0; j < s64.nt; ++j) l1_tr = std::max(l1_tr, density_l1(s32, s64, &un64, static_cast<int>(j)));
      std::printf("{\"mode\": \"accuracy\", \"case\": \"%s\", \"n\": %d, \"cells\": %d, \"steps\": %d, "
                  "\"time_fp64\": %.17g, \"time_fp32mixed\": %.17g, \"l1_density_fp32mixed_vs_fp64\": %.6e, "
                  "\"l1_tracers_fp32mixed_vs_fp64\": %.6e, \"unmatched\": %zu, ",
                  which.c_str(), n, g64->tess->GetPointNo(), steps, s64.time, s32.time, l1_32, l1_tr, un32);
      if (stock) {
        std::vector<uint64_t> hs(static_cast<size_t>(steps));
        uint64_t np = 0;
        Snapshot sr;
        double clk[6] = {0, 0, 0, 0, 0, 0};
        bool ok = read_all(fds[0], hs.data(), 8 * hs.size()) && read_all(fds[0], &np, 8);
        if (ok) {
          sr.xy.resize(2 * np);
          sr.rho.resize(np);
          ok = read_all(fds[0], sr.xy.data(), 16 * np) && read_all(fds[0], sr.rho.data(), 8 * np) &&
               read_all(fds[0], clk, sizeof clk);
        }
        ::close(fds[0]);
        int status = 0;
        waitpid(child, &status, 0);
        if (!ok || !WIFEXITED(status) || WEXITSTATUS(status) != 0)
          throw std::runtime_error("the stock simulation's process failed");
        sr.time = clk[5];
        int first_diff = -1;
        for (int k = 0; k < steps && first_diff < 0; ++k)
          if (hs[static_cast<size_t>(k)] != h64[static_cast<size_t>(k)]) first_diff = k + 1;
        const double l1_64 = density_l1(s64, sr, &un64);
        std::printf("\"l1_density_fp64_vs_stock\": %.6e, \"l1_density_fp32mixed_vs_stock\": %.6e, "
                    "\"fp64_equal_to_stock\": %s, \"first_differing_step\": %d, \"time_stock\": %.17g, "
                    "\"stock\": {\"ms_per_step\": %.6f, \"plugin_ms_per_step\": %.6f}, ",
                    l1_64, density_l1(s32, sr, &un64), first_diff < 0 ? "true" : "false", first_diff, sr.time,
                    1e3 * clk[0] / steps, 1e3 * (clk[1] + clk[2] + clk[3] + clk[4]) / steps);
      }
      print_clock("gpu_fp64", *g64, steps, w64);
      std::printf(", ");
      print_clock("gpu_fp32mixed", *g32, steps, w32);
      std::printf("}\n");
      return 0;
    }
    if (mode == "sensitivity") {
      // The problem's own sensitivity: the stock simulation against the stock
      // simulation from initial densities perturbed by a relative `delta`
      // (CPU only); density L1 every `every` steps.
      if (argc < 7) return usage();
      const double delta = std::atof(argv[5]);
      const int every = std::atoi(argv[6]);
      std::unique_ptr<Sim> a = make_sim(which, n, kStock);
      g_perturb = delta;
      std::unique_ptr<Sim> b = make_sim(which, n, kStock);
      g_perturb = 0;
      std::printf("{\"mode\": \"sensitivity\", \"case\": \"%s\", \"n\": %d, \"delta\": %g, \"l1\": [", which.c_str(), n,
                  delta);
      for (int k = 1; k <= steps; ++k) {
        a->advance();
        b->advance();
        if (k % every == 0 || k == steps) {
          size_t un = 0;
          std::printf("%s[%d, %.6e, %.6e]", k == every ? "" : ", ", k,
                      density_l1(snapshot(*b->sim), snapshot(*a->sim), &un),
                      (b->sim->getTime() - a->sim->getTime()) / a->sim->getTime());
          std::fflush(stdout);
        }
      }
      std::printf("]}\n");
      return 0;
    }
    if (mode == "time") {
      if (argc < 6) return usage();
      const std::string set = argv[5];
      const Set s = set == "stock" ? kStock : set == "gpu" ? kGpu64 : set == "gpu32" ? kGpu32 : kStock;
      std::unique_ptr<Sim> a = make_sim(which, n, s);
      a->advance();  // warm-up: first upload, module load
      a->clock = PluginClock();
      const double t0 = now();
      for (int k = 0; k < steps; ++k) a->advance();
      const double wall = now() - t0;
      std::printf("{\"mode\": \"time\", \"case\": \"%s\", \"n\": %d, \"cells\": %d, \"steps\": %d, \"set\": \"%s\", ",
                  which.c_str(), n, a->tess->GetPointNo(), steps, set.c_str());
      print_clock(set.c_str(), *a, steps, wall);
      std::printf("}\n");
      return 0;
    }
  } catch (UniversalError& e) {
    std::fprintf(stderr, "UniversalError: %s\n", e.GetErrorMessage().c_str());
    for (size_t i = 0; i < e.GetFields().size(); ++i)
      std::fprintf(stderr, "  %s = %.17g\n", e.GetFields()[i].c_str(), e.GetValues()[i]);
    return 3;
  } catch (std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 3;
  }
  return usage();
}
