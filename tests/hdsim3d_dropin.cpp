// hdsim3d_dropin.cpp -- HDSim3D driven through the GPU 3D plugins, beside
// HDSim3D driven through the reference's own.
//
// Test driver only: it links the reference's sources (built by
// oracle/ref/Makefile) and librich_gb300.so through the adapters in
// huji-rich_gb300/host/rich_gpu_adapters3d.hpp.  Two complete simulations on
// a CubeGrid differ only in their time-step and flux plugins:
// CourantFriedrichsLewy(0.3) and FirstOrderHydroFlux(Hllc), or GpuTimeStep3D
// and GpuFluxCalculator3D; both use Eulerian3D and DefaultCellUpdater, and
// HDSim3D::timeAdvance (hdsim_3d.cpp:133-145) advances both.
//
//   hdsim3d_dropin compare <case> <n> <steps>
//       lockstep; after every step the cells and the step's dt of the two
//       are compared with ==; prints one JSON line.
//   hdsim3d_dropin time <case> <n> <steps> <stock|gpu>
//       wall time per step and the time inside the two plugin calls.
//
// Cases (n x n x n CubeGrid):
//   sedov   [-0.5, 0.5]^3, rho 1, p 1e-6, energy 1 as pressure in r < 0.04
//           (at least the 8 central cells), gamma 5/3
//   random  [0,1]^3, seeded density, pressure (log-uniform in [0.5, 2]) and
//           velocity per cell, gamma 5/3
//   sod     [0,1]^3, a Sod tube along x at rest, gamma 1.4
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "rich_gpu_adapters3d.hpp"
#include "source/3D/CubeGrid/CubeGrid.hpp"
#include "source/newtonian/common/hllc.hpp"
#include "source/newtonian/common/ideal_gas.hpp"
#include "source/newtonian/three_dimensional/CourantFriedrichsLewy.hpp"
#include "source/newtonian/three_dimensional/FirstOrderHydroFlux.hpp"
#include "source/newtonian/three_dimensional/default_cell_updater.hpp"
#include "source/newtonian/three_dimensional/eulerian_3d.hpp"
#include "source/newtonian/three_dimensional/hdsim_3d.hpp"

using three_dimenssional::ComputationalCell;

namespace {

double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Forwarding plugins that time the wrapped one and keep the time steps.
class TimedTSC : public TimeStepCalculator {
 public:
  TimedTSC(const TimeStepCalculator& in, double& acc, std::vector<double>& dts) : in_(in), acc_(acc), dts_(dts) {}
  double operator()(const Tessellation3D& t, const vector<ComputationalCell>& c, const EquationOfState& e) const override {
    const double t0 = now();
    const double dt = in_(t, c, e);
    acc_ += now() - t0;
    dts_.push_back(dt);
    return dt;
  }

 private:
  const TimeStepCalculator& in_;
  double& acc_;
  std::vector<double>& dts_;
};

class TimedFC3 : public FluxCalculator3D {
 public:
  TimedFC3(const FluxCalculator3D& in, double& acc) : in_(in), acc_(acc) {}
  vector<Conserved3D> operator()(const Tessellation3D& t, const vector<ComputationalCell>& c, const EquationOfState& e,
                                 const vector<Vector3D>& pv) const override {
    const double t0 = now();
    vector<Conserved3D> r = in_(t, c, e, pv);
    acc_ += now() - t0;
    return r;
  }

 private:
  const FluxCalculator3D& in_;
  double& acc_;
};

struct Sim3 {
  double t_tsc = 0, t_fc = 0;
  std::vector<double> dts;
  std::unique_ptr<CubeGrid> tess;
  std::unique_ptr<IdealGas> eos;
  Hllc rs;
  Eulerian3D pm;
  DefaultCellUpdater cu;
  std::unique_ptr<CourantFriedrichsLewy> s_tsc;
  std::unique_ptr<FirstOrderHydroFlux> s_fc;
  std::unique_ptr<rich_gb300::GpuContext3D> ctx;
  std::unique_ptr<rich_gb300::GpuTimeStep3D> g_tsc;
  std::unique_ptr<rich_gb300::GpuFluxCalculator3D> g_fc;
  std::unique_ptr<TimedTSC> tsc;
  std::unique_ptr<TimedFC3> fc;
  std::unique_ptr<HDSim3D> sim;
};

std::unique_ptr<Sim3> make_sim(const std::string& which, size_t n, bool gpu) {
  std::unique_ptr<Sim3> s(new Sim3);
  const bool sedov = which == "sedov";
  const Vector3D lo = sedov ? Vector3D(-0.5, -0.5, -0.5) : Vector3D(0, 0, 0);
  const Vector3D hi = sedov ? Vector3D(0.5, 0.5, 0.5) : Vector3D(1, 1, 1);
  s->tess.reset(new CubeGrid(n, n, n, lo, hi));
  const double gamma = which == "sod" ? 1.4 : 5.0 / 3.0;
  s->eos.reset(new IdealGas(gamma));
  const size_t np = s->tess->GetPointNo();
  std::vector<ComputationalCell> cells(np);
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> u01(0.0, 1.0);
  if (sedov) {
    double r_hot = 0.04;
    size_t hot = 0;
    for (size_t i = 0; i < np; ++i) hot += abs(s->tess->GetMeshPoint(i)) < r_hot;
    if (hot < 8) r_hot = std::sqrt(3.0) * 0.5 * (hi.x - lo.x) / static_cast<double>(n) * 1.0001;
    double vin = 0;
    for (size_t i = 0; i < np; ++i)
      if (abs(s->tess->GetMeshPoint(i)) < r_hot) vin += s->tess->GetVolume(i);
    for (size_t i = 0; i < np; ++i) {
      cells[i].density = 1;
      cells[i].pressure = abs(s->tess->GetMeshPoint(i)) < r_hot ? (gamma - 1) / vin : 1e-6;
    }
  } else {
    for (size_t i = 0; i < np; ++i) {
      const Vector3D x = s->tess->GetMeshPoint(i);
      if (which == "random") {
        cells[i].density = std::exp(std::log(0.5) + u01(rng) * std::log(4.0));
        cells[i].pressure = std::exp(std::log(0.5) + u01(rng) * std::log(4.0));
        cells[i].velocity = Vector3D(u01(rng) - 0.5, u01(rng) - 0.5, u01(rng) - 0.5);
      } else if (which == "sod") {
        cells[i].density = x.x < 0.5 ? 1.0 : 0.125;
        cells[i].pressure = x.x < 0.5 ? 1.0 : 0.1;
      } else {
        throw std::runtime_error("unknown case " + which);
      }
    }
  }
  const TimeStepCalculator* tsc;
  const FluxCalculator3D* fc;
  if (gpu) {
    rg_config cfg;
    rg_default_config(&cfg);
    cfg.gamma = gamma;
    cfg.cfl = 0.3;
    s->ctx.reset(new rich_gb300::GpuContext3D(cfg));
    s->g_tsc.reset(new rich_gb300::GpuTimeStep3D(*s->ctx));
    s->g_fc.reset(new rich_gb300::GpuFluxCalculator3D(*s->ctx));
    tsc = s->g_tsc.get();
    fc = s->g_fc.get();
  } else {
    s->s_tsc.reset(new CourantFriedrichsLewy(0.3));
    s->s_fc.reset(new FirstOrderHydroFlux(s->rs));
    tsc = s->s_tsc.get();
    fc = s->s_fc.get();
  }
  s->tsc.reset(new TimedTSC(*tsc, s->t_tsc, s->dts));
  s->fc.reset(new TimedFC3(*fc, s->t_fc));
  s->sim.reset(new HDSim3D(*s->tess, cells, *s->eos, s->pm, *s->tsc, *s->fc, s->cu));
  return s;
}

bool same(double a, double b) { return a == b || (std::isnan(a) && std::isnan(b)); }

size_t count_differences(const Sim3& a, const Sim3& b) {
  const std::vector<ComputationalCell>& ca = a.sim->getCells();
  const std::vector<ComputationalCell>& cb = b.sim->getCells();
  if (ca.size() != cb.size() || a.dts.size() != b.dts.size()) return static_cast<size_t>(-1);
  size_t d = 0;
  for (size_t k = 0; k < a.dts.size(); ++k) d += !same(a.dts[k], b.dts[k]);
  for (size_t i = 0; i < ca.size(); ++i)
    d += !same(ca[i].density, cb[i].density) + !same(ca[i].pressure, cb[i].pressure) +
         !same(ca[i].velocity.x, cb[i].velocity.x) + !same(ca[i].velocity.y, cb[i].velocity.y) +
         !same(ca[i].velocity.z, cb[i].velocity.z);
  return d;
}

int usage() {
  std::fprintf(stderr,
               "usage: hdsim3d_dropin compare <case> <n> <steps>\n"
               "       hdsim3d_dropin time <case> <n> <steps> <stock|gpu>\n");
  return 2;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 5) return usage();
  const std::string mode = argv[1], which = argv[2];
  const size_t n = std::stoul(argv[3]);
  const int steps = std::atoi(argv[4]);
  try {
    if (mode == "compare") {
      std::unique_ptr<Sim3> a = make_sim(which, n, false), b = make_sim(which, n, true);
      int first_diff = -1;
      size_t diffs = 0;
      double wa = 0, wb = 0;
      for (int k = 1; k <= steps && first_diff < 0; ++k) {
        double t0 = now();
        a->sim->timeAdvance();
        wa += now() - t0;
        t0 = now();
        b->sim->timeAdvance();
        wb += now() - t0;
        diffs = count_differences(*a, *b);
        if (diffs) first_diff = k;
      }
      double t_end = 0;
      for (double dt : b->dts) t_end += dt;
      std::printf("{\"mode\": \"compare\", \"case\": \"%s\", \"n\": %zu, \"cells\": %zu, \"steps\": %d, "
                  "\"time\": %.17g, \"equal\": %s, \"first_differing_step\": %d, \"differing_values\": %zu, "
                  "\"stock_ms_per_step\": %.4f, \"gpu_ms_per_step\": %.4f, \"gpu_plugin_ms_per_step\": %.4f}\n",
                  which.c_str(), n, a->tess->GetPointNo(), steps, t_end, first_diff < 0 ? "true" : "false",
                  first_diff, diffs, 1e3 * wa / steps, 1e3 * wb / steps, 1e3 * (b->t_tsc + b->t_fc) / steps);
      return first_diff < 0 ? 0 : 1;
    }
    if (mode == "time") {
      if (argc < 6) return usage();
      const bool gpu = std::string(argv[5]) == "gpu";
      std::unique_ptr<Sim3> a = make_sim(which, n, gpu);
      a->sim->timeAdvance();  // warm-up
      a->t_tsc = a->t_fc = 0;
      const double t0 = now();
      for (int k = 0; k < steps; ++k) a->sim->timeAdvance();
      const double wall = now() - t0;
      std::printf("{\"mode\": \"time\", \"case\": \"%s\", \"n\": %zu, \"cells\": %zu, \"steps\": %d, \"set\": \"%s\", "
                  "\"ms_per_step\": %.4f, \"tsc_ms\": %.4f, \"flux_ms\": %.4f, \"host_rest_ms\": %.4f}\n",
                  which.c_str(), n, a->tess->GetPointNo(), steps, gpu ? "gpu" : "stock", 1e3 * wall / steps,
                  1e3 * a->t_tsc / steps, 1e3 * a->t_fc / steps, 1e3 * (wall - a->t_tsc - a->t_fc) / steps);
      return 0;
    }
  } catch (UniversalError& e) {
    std::fprintf(stderr, "UniversalError: %s\n", e.GetErrorMessage().c_str());
    return 3;
  } catch (std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 3;
  }
  return usage();
}
