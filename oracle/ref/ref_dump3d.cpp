// ref_dump3d.cpp -- runs the reference RICH 3D first-order hot path
// (HDSim3D with CubeGrid, FirstOrderHydroFlux(Hllc), DefaultCellUpdater,
// CourantFriedrichsLewy, Eulerian3D) on a seeded case and writes its inputs
// and outputs as .npy files, which tests/golden/make_golden.py bundles into
// tests/golden/<case>.npz.
//
// Test infrastructure only: it links the reference sources built by
// oracle/ref/Makefile and is never part of the product.
//
//   ref_dump3d <case> <outdir> <nx> <ny> <nz> <run_steps>
//
// cases: random (seeded density, pressure and velocity per cell), sod
// (a Sod tube along x at rest), shear (uniform gas with a sheared velocity).
// Writes:
//   mesh3_*       the tessellation as the hot path sees it: face neighbours
//                 (-1 outside), Tessellation3D::Normal, Face::GetArea, and per
//                 cell GetVolume, GetWidth, GetCellFaces
//   cells0, ext0  ComputationalCell {density, pressure, vx, vy, vz} and the
//                 ExtensiveGenerator extensives {mass, px, py, pz, energy}
//   dt            CourantFriedrichsLewy of cells0
//   fluxes        FirstOrderHydroFlux of cells0 {mass, px, py, pz, energy}
//   cells1        after one HDSim3D::timeAdvance
//   run_cells, run_dts  after <run_steps> timeAdvance steps, and each step's dt
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "source/3D/CubeGrid/CubeGrid.hpp"
#include "source/misc/lazy_list.hpp"
#include "source/newtonian/common/hllc.hpp"
#include "source/newtonian/common/ideal_gas.hpp"
#include "source/newtonian/three_dimensional/CourantFriedrichsLewy.hpp"
#include "source/newtonian/three_dimensional/FirstOrderHydroFlux.hpp"
#include "source/newtonian/three_dimensional/default_cell_updater.hpp"
#include "source/newtonian/three_dimensional/eulerian_3d.hpp"
#include "source/newtonian/three_dimensional/extensive_generator.hpp"
#include "source/newtonian/three_dimensional/hdsim_3d.hpp"

using three_dimenssional::ComputationalCell;

namespace {

std::string g_out;

void write_npy(const std::string& name, const char* descr, size_t elem, const void* data, size_t rows,
               size_t cols) {
  std::string path = g_out + "/" + name + ".npy";
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("cannot open " + path);
  char shape[64];
  if (cols == 0)
    std::snprintf(shape, sizeof shape, "(%zu,)", rows);
  else
    std::snprintf(shape, sizeof shape, "(%zu, %zu)", rows, cols);
  std::string hdr = std::string("{'descr': '") + descr + "', 'fortran_order': False, 'shape': " + shape + ", }";
  while ((10 + hdr.size() + 1) % 64 != 0) hdr += ' ';
  hdr += '\n';
  const unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
  std::fwrite(magic, 1, 8, f);
  const uint16_t len = static_cast<uint16_t>(hdr.size());
  std::fwrite(&len, 2, 1, f);
  std::fwrite(hdr.data(), 1, hdr.size(), f);
  std::fwrite(data, elem, rows * (cols ? cols : 1), f);
  std::fclose(f);
}
void write_d(const std::string& n, const std::vector<double>& v, size_t cols) {
  write_npy(n, "<f8", 8, v.data(), cols ? v.size() / cols : v.size(), cols);
}
void write_i(const std::string& n, const std::vector<int32_t>& v, size_t cols) {
  write_npy(n, "<i4", 4, v.data(), cols ? v.size() / cols : v.size(), cols);
}

std::vector<double> pack_cells(const std::vector<ComputationalCell>& c) {
  std::vector<double> r;
  for (const auto& x : c) {
    r.push_back(x.density);
    r.push_back(x.pressure);
    r.push_back(x.velocity.x);
    r.push_back(x.velocity.y);
    r.push_back(x.velocity.z);
  }
  return r;
}
std::vector<double> pack_cons(const std::vector<Conserved3D>& c) {
  std::vector<double> r;
  for (const auto& x : c) {
    r.push_back(x.mass);
    r.push_back(x.momentum.x);
    r.push_back(x.momentum.y);
    r.push_back(x.momentum.z);
    r.push_back(x.energy);
  }
  return r;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 7) {
    std::fprintf(stderr, "usage: ref_dump3d <case> <outdir> <nx> <ny> <nz> <run_steps>\n");
    return 2;
  }
  const std::string kase = argv[1];
  g_out = argv[2];
  const size_t nx = std::stoul(argv[3]), ny = std::stoul(argv[4]), nz = std::stoul(argv[5]);
  const int run_steps = std::stoi(argv[6]);
  CubeGrid tess(nx, ny, nz, Vector3D(0, 0, 0), Vector3D(1.0, 0.8, 0.6));
  const size_t n = tess.GetPointNo();
  const double gamma = kase == "sod" ? 1.4 : 5.0 / 3.0;
  std::vector<ComputationalCell> cells(n);
  std::mt19937_64 rng(20261203);
  std::uniform_real_distribution<double> u01(0.0, 1.0);
  for (size_t i = 0; i < n; ++i) {
    const Vector3D x = tess.GetMeshPoint(i);
    if (kase == "random") {
      cells[i].density = std::exp(std::log(0.5) + u01(rng) * std::log(4.0));
      cells[i].pressure = std::exp(std::log(0.5) + u01(rng) * std::log(4.0));
      cells[i].velocity = Vector3D(u01(rng) - 0.5, u01(rng) - 0.5, u01(rng) - 0.5);
    } else if (kase == "sod") {
      const bool left = x.x < 0.5;
      cells[i].density = left ? 1.0 : 0.125;
      cells[i].pressure = left ? 1.0 : 0.1;
      cells[i].velocity = Vector3D(0, 0, 0);
    } else if (kase == "shear") {
      cells[i].density = 1.0;
      cells[i].pressure = 2.5;
      cells[i].velocity = Vector3D(0.3 * std::sin(2 * M_PI * x.y), 0.0, 0.2 * std::cos(2 * M_PI * x.x));
    } else {
      throw std::runtime_error("unknown case " + kase);
    }
  }
  // mesh as the hot path sees it
  std::vector<int32_t> fcells, off(1, 0), cf;
  std::vector<double> normal, area, volume, width;
  const size_t nf = tess.GetTotalFacesNumber();
  for (size_t f = 0; f < nf; ++f) {
    const Face& face = tess.GetFace(f);
    fcells.push_back(tess.IsGhostPoint(face.neighbors.first) ? -1 : static_cast<int32_t>(face.neighbors.first));
    fcells.push_back(tess.IsGhostPoint(face.neighbors.second) ? -1 : static_cast<int32_t>(face.neighbors.second));
    const Vector3D nn = tess.Normal(f);
    normal.push_back(nn.x);
    normal.push_back(nn.y);
    normal.push_back(nn.z);
    area.push_back(face.GetArea());
  }
  for (size_t i = 0; i < n; ++i) {
    volume.push_back(tess.GetVolume(i));
    width.push_back(tess.GetWidth(i));
    for (size_t f : tess.GetCellFaces(i)) cf.push_back(static_cast<int32_t>(f));
    off.push_back(static_cast<int32_t>(cf.size()));
  }
  write_i("mesh3_face_cells", fcells, 2);
  write_d("mesh3_normal", normal, 3);
  write_d("mesh3_area", area, 0);
  write_d("mesh3_volume", volume, 0);
  write_d("mesh3_width", width, 0);
  write_i("mesh3_cell_face_offset", off, 0);
  write_i("mesh3_cell_faces", cf, 0);
  write_d("gamma", std::vector<double>{gamma}, 0);

  IdealGas eos(gamma);
  Hllc rs;
  FirstOrderHydroFlux fc(rs);
  CourantFriedrichsLewy tsc(0.3);
  DefaultCellUpdater cu;
  Eulerian3D pm;
  write_d("cells0", pack_cells(cells), 5);
  write_d("ext0", pack_cons(serial_generate(ExtensiveGenerator(cells, tess, eos))), 5);
  write_d("dt", std::vector<double>{tsc(tess, cells, eos)}, 0);
  write_d("fluxes", pack_cons(fc(tess, cells, eos, std::vector<Vector3D>(n))), 5);
  HDSim3D sim(tess, cells, eos, pm, tsc, fc, cu);
  std::vector<double> dts;
  for (int k = 0; k < run_steps; ++k) {
    dts.push_back(tsc(tess, sim.getCells(), eos));
    sim.timeAdvance();
    if (k == 0) write_d("cells1", pack_cells(sim.getCells()), 5);
  }
  write_d("run_cells", pack_cells(sim.getCells()), 5);
  write_d("run_dts", dts, 0);
  return 0;
}
