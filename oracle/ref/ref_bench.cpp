// ref_bench.cpp -- the reference's own CPU implementation of the hot path,
// timed: the benchmark's reference arm and CPU baseline.
//
// Test infrastructure only: it links the reference sources built by
// oracle/ref/Makefile.  One process runs one simulation on one core (the
// reference is serial); the benchmark starts one process per host core.
//
//   ref_bench <points.f64> <cells.f64> <nx> <ny> <warmup> <steps>
//
// Workload: 2D Sedov-Taylor on [-1,1]^2 (SquareBox, rigid walls), the mesh
// points read from <points.f64> (nx*ny (x, y) pairs, little-endian float64;
// the benchmark writes the same jittered lattice its GPU arm uses), a
// VoronoiMesh of them (Hilbert-ordered, the reference's default), IdealGas(5/3),
// and the initial cells read from
// <cells.f64> (nx*ny {density, pressure, vx, vy}: the GPU arm's initial
// state, rho 1, p 1e-6, energy 1 deposited as pressure within r < 0.02).  A step is the plugin work of
// hdsim::TimeAdvance (hdsim2d.cpp:149-241) on a fixed mesh, in hdsim's
// order: SimpleCFL(0.3) (:161-165), ModularFluxCalculator(
// LinearGaussImproved(RigidWallGenerator), Hllc) (:176-184),
// SimpleExtensiveUpdater (:188-195), SimpleCellUpdater (:233).  The face
// velocities are RoundCells(Lagrangian)'s point velocities through
// StationaryBox, computed once before timing, as the GPU arm's kernels read
// the device-computed ones.  Prints one JSON line.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <utility>
#include <string>
#include <vector>

#include "source/newtonian/common/hllc.hpp"
#include "source/newtonian/common/ideal_gas.hpp"
#include "source/newtonian/two_dimensional/cache_data.hpp"
#include "source/newtonian/two_dimensional/geometric_outer_boundaries/SquareBox.hpp"
#include "source/newtonian/two_dimensional/ghost_point_generators/RigidWallGenerator.hpp"
#include "source/newtonian/two_dimensional/hdsim2d.hpp"
#include "source/newtonian/two_dimensional/interpolations/LinearGaussImproved.hpp"
#include "source/newtonian/two_dimensional/modular_flux_calculator.hpp"
#include "source/newtonian/two_dimensional/point_motions/lagrangian.hpp"
#include "source/newtonian/two_dimensional/point_motions/round_cells.hpp"
#include "source/newtonian/two_dimensional/simple_cell_updater.hpp"
#include "source/newtonian/two_dimensional/simple_cfl.hpp"
#include "source/newtonian/two_dimensional/simple_extensive_updater.hpp"
#include "source/newtonian/two_dimensional/stationary_box.hpp"
#include "source/tessellation/VoronoiMesh.hpp"

namespace {

double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 7) {
    std::fprintf(stderr, "usage: ref_bench <points.f64> <cells.f64> <nx> <ny> <warmup> <steps>\n");
    return 2;
  }
  const int nx = std::atoi(argv[3]), ny = std::atoi(argv[4]);
  const int warm = std::atoi(argv[5]), steps = std::atoi(argv[6]);
  const size_t np = static_cast<size_t>(nx) * static_cast<size_t>(ny);
  std::vector<double> xy(2 * np), c0(4 * np);
  for (int k = 0; k < 2; ++k) {
    std::vector<double>& dst = k == 0 ? xy : c0;
    FILE* f = std::fopen(argv[1 + k], "rb");
    const bool ok = f && std::fread(dst.data(), sizeof(double), dst.size(), f) == dst.size();
    if (f) std::fclose(f);
    if (!ok) {
      std::fprintf(stderr, "ref_bench: cannot read %zu values from %s\n", dst.size(), argv[1 + k]);
      return 2;
    }
  }
  try {
    const double t_setup = now();
    std::vector<Vector2D> pts(np);
    for (size_t i = 0; i < np; ++i) pts[i] = Vector2D(xy[2 * i], xy[2 * i + 1]);
    SquareBox outer(Vector2D(-1, -1), Vector2D(1, 1));
    VoronoiMesh tess(pts, outer);
    SlabSymmetry pg;
    const double gamma = 5.0 / 3.0;
    IdealGas eos(gamma);
    Hllc rs;
    RigidWallGenerator ghosts;
    LinearGaussImproved sr(eos, ghosts, true, 0.2, 0.5, 0.7);
    ModularFluxCalculator fc(sr, rs);
    SimpleCFL tsf(0.3);
    SimpleExtensiveUpdater eu;
    SimpleCellUpdater cu;
    Lagrangian lag;
    RoundCells round(lag, eos);
    StationaryBox evc;
    const TracerStickerNames tsn;

    const int n = tess.GetPointNo();
    // VoronoiMesh keeps its points in Hilbert order (its default): each mesh
    // point takes the initial cell of the input point with its coordinates
    std::map<std::pair<double, double>, size_t> input;
    for (size_t i = 0; i < np; ++i) input[std::make_pair(xy[2 * i], xy[2 * i + 1])] = i;
    std::vector<ComputationalCell> cells(static_cast<size_t>(n));
    for (int i = 0; i < n; ++i) {
      const Vector2D r = tess.GetMeshPoint(i);
      const auto it = input.find(std::make_pair(r.x, r.y));
      if (it == input.end()) throw UniversalError("ref_bench: a mesh point is not an input point");
      const size_t j = it->second;
      ComputationalCell& c = cells[static_cast<size_t>(i)];
      c.density = c0[4 * j];
      c.pressure = c0[4 * j + 1];
      c.velocity = Vector2D(c0[4 * j + 2], c0[4 * j + 3]);
    }
    CacheData cd(tess, pg);
    // hdsim's init_extensives (hdsim2d.cpp:41-67)
    std::vector<Extensive> ext(static_cast<size_t>(n));
    for (int i = 0; i < n; ++i) {
      const ComputationalCell& c = cells[static_cast<size_t>(i)];
      const double mass = c.density * cd.volumes[static_cast<size_t>(i)];
      Extensive& e = ext[static_cast<size_t>(i)];
      e.mass = mass;
      e.energy = eos.dp2e(c.density, c.pressure, c.tracers, tsn.tracer_names) * mass + 0.5 * mass * ScalarProd(c.velocity, c.velocity);
      e.momentum = mass * c.velocity;
    }
    const std::vector<Vector2D> pv = round(tess, cells, 0, tsn);
    const std::vector<Vector2D> ev = evc(tess, pv);
    double time = 0;
    auto step = [&]() {
      const double dt = tsf(tess, cells, eos, ev, time, tsn);
      const std::vector<Extensive> fluxes = fc(tess, ev, cells, ext, cd, eos, time, dt, tsn);
      eu(fluxes, pg, tess, dt, cd, cells, ext, time, tsn);
      cells = cu(tess, pg, eos, ext, cells, cd, tsn);
      time += dt;
    };
    const double setup = now() - t_setup;
    for (int k = 0; k < warm; ++k) step();
    const double t0 = now();
    for (int k = 0; k < steps; ++k) step();
    const double t = now() - t0;
    std::printf("{\"cells\": %d, \"faces\": %zu, \"warmup\": %d, \"steps\": %d, \"seconds\": %.6f, "
                "\"ms_per_step\": %.6f, \"setup_s\": %.3f, \"time\": %.17g, \"density0\": %.17g}\n",
                n, tess.getAllEdges().size(), warm, steps, t, 1e3 * t / (steps > 0 ? steps : 1), setup, time,
                cells[0].density);
  } catch (UniversalError& e) {
    std::fprintf(stderr, "UniversalError: %s\n", e.GetErrorMessage().c_str());
    return 3;
  }
  return 0;
}
