// Compile-only check of huji-rich_gb300/host/rich_gpu_adapters.hpp against the
// reference's own headers: an hdsim built from the GPU plugins, as a RICH
// driver would write it (tests/test_cpu_adapters.py runs g++ -fsyntax-only).
#include "rich_gpu_adapters.hpp"
#include "source/newtonian/common/hllc.hpp"
#include "source/newtonian/two_dimensional/geometric_outer_boundaries/SquareBox.hpp"
#include "source/newtonian/two_dimensional/hdsim2d.hpp"
#include "source/newtonian/two_dimensional/point_motions/eulerian.hpp"
#include "source/newtonian/two_dimensional/source_terms/zero_force.hpp"
#include "source/newtonian/two_dimensional/stationary_box.hpp"
#include "source/tessellation/VoronoiMesh.hpp"

void build_simulation(const std::vector<Vector2D>& points, const std::vector<ComputationalCell>& init) {
  SquareBox outer(Vector2D(0, 0), Vector2D(1, 0.2));
  VoronoiMesh tess(points, outer);
  SlabSymmetry pg;
  IdealGas eos(1.4);
  Eulerian pm;
  StationaryBox evc;
  ZeroForce force;
  rg_config cfg;
  rg_default_config(&cfg);
  cfg.gamma = 1.4;
  cfg.order = 1;
  rich_gb300::GpuContext ctx(cfg);
  rich_gb300::GpuCFL tsf(ctx);
  rich_gb300::GpuFluxCalculator fc(ctx);
  rich_gb300::GpuExtensiveUpdater eu(ctx);
  rich_gb300::GpuCellUpdater cu(ctx);
  hdsim sim(tess, outer, pg, init, eos, pm, evc, force, tsf, fc, eu, cu);
  sim.TimeAdvance();
}
