// rich_gpu_adapters3d.hpp -- RICH's 3D plugins (HDSim3D) backed by the GB300
// library.
//
// Header-only C++ that a RICH build includes (include path = the RICH source
// root plus this directory and include/), linking librich_gb300.so.  HDSim3D
// (source/newtonian/three_dimensional/hdsim_3d.hpp) holds two plugins that
// a GPU can take over, by reference, and these classes derive from their
// abstract interfaces:
//
//   GpuTimeStep3D        : TimeStepCalculator (time_step_calculator.hpp:16-33)
//                          in place of CourantFriedrichsLewy
//   GpuFluxCalculator3D  : FluxCalculator3D   (flux_calculator_3d.hpp:16-37)
//                          in place of FirstOrderHydroFlux(Hllc)
//
// HDSim3D::timeAdvance (hdsim_3d.cpp:133-145) then runs unchanged: dt from
// the time-step plugin, point velocities on the host, the fluxes from the
// flux plugin, then its own update_extensive and the per-cell CellUpdater3D
// on the host.  Those two are not plugins of HDSim3D (update_extensive is a
// function inside hdsim_3d.cpp; CellUpdater3D is called once per cell with
// one cell's conserved density), so with HDSim3D they stay on the host.  A
// caller that wants the whole 3D step on the GPU drives the C ABI directly:
// rg3_step / rg3_run perform timeAdvance's CFL, fluxes, update_extensive and
// DefaultCellUpdater on the device for a fixed mesh.
//
// Both plugins share one GpuContext3D (one rg3_handle).  The tessellation is
// packed and uploaded only when it changed (same point and face counts and
// bitwise-equal mesh points as at the last upload); face velocities are
// Tessellation3D::CalcFaceVelocity of the point velocities
// (FirstOrderHydroFlux.cpp:100-110), or none when every point is at rest.
// Supported: IdealGas, Hllc (massflux), the first-order scheme, no tracers.
#ifndef RICH_GB300_ADAPTERS3D_HPP
#define RICH_GB300_ADAPTERS3D_HPP

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "rich_gb300.h"
#include "source/3D/GeometryCommon/Tessellation3D.hpp"
#include "source/misc/universal_error.hpp"
#include "source/newtonian/common/ideal_gas.hpp"
#include "source/newtonian/three_dimensional/computational_cell.hpp"
#include "source/newtonian/three_dimensional/conserved_3d.hpp"
#include "source/newtonian/three_dimensional/flux_calculator_3d.hpp"
#include "source/newtonian/three_dimensional/time_step_calculator.hpp"

namespace rich_gb300 {

// A Tessellation3D packed as rg_mesh3d_view describes it.
struct PackedMesh3D {
  int32_t n_cells = 0, n_faces = 0;
  std::vector<int32_t> face_cells, cell_face_offset, cell_faces;
  std::vector<double> face_normal, face_area, volume, width;

  rg_mesh3d_view view() const {
    rg_mesh3d_view v;
    v.n_cells = n_cells;
    v.n_faces = n_faces;
    v.face_cells = face_cells.data();
    v.face_normal = face_normal.data();
    v.face_area = face_area.data();
    v.volume = volume.data();
    v.width = width.data();
    v.cell_face_offset = cell_face_offset.data();
    v.cell_faces = cell_faces.data();
    return v;
  }
};

// Face neighbours (-1 for a ghost: Tessellation3D::IsGhostPoint), Normal,
// Face::GetArea, and per cell GetVolume, GetWidth and GetCellFaces (in the
// tessellation's order; the device sums a cell's faces in that order).
inline void pack_tessellation3d(const Tessellation3D& tess, PackedMesh3D& m) {
  const size_t n = tess.GetPointNo(), nf = tess.GetTotalFacesNumber();
  m.n_cells = static_cast<int32_t>(n);
  m.n_faces = static_cast<int32_t>(nf);
  m.face_cells.resize(2 * nf);
  m.face_normal.resize(3 * nf);
  m.face_area.resize(nf);
  for (size_t f = 0; f < nf; ++f) {
    const Face& face = tess.GetFace(f);
    m.face_cells[2 * f] = tess.IsGhostPoint(face.neighbors.first) ? -1 : static_cast<int32_t>(face.neighbors.first);
    m.face_cells[2 * f + 1] =
        tess.IsGhostPoint(face.neighbors.second) ? -1 : static_cast<int32_t>(face.neighbors.second);
    const Vector3D nn = tess.Normal(f);
    m.face_normal[3 * f] = nn.x;
    m.face_normal[3 * f + 1] = nn.y;
    m.face_normal[3 * f + 2] = nn.z;
    m.face_area[f] = face.GetArea();
  }
  m.volume.resize(n);
  m.width.resize(n);
  m.cell_face_offset.assign(1, 0);
  m.cell_faces.clear();
  for (size_t i = 0; i < n; ++i) {
    m.volume[i] = tess.GetVolume(i);
    m.width[i] = tess.GetWidth(i);
    for (size_t f : tess.GetCellFaces(i)) m.cell_faces.push_back(static_cast<int32_t>(f));
    m.cell_face_offset.push_back(static_cast<int32_t>(m.cell_faces.size()));
  }
}

class GpuContext3D {
 public:
  explicit GpuContext3D(const rg_config& cfg) : cfg_(cfg) {
    const rg_status st = rg3_create(&cfg_, &h_);
    if (st != RG_OK) throw UniversalError(std::string("rich_gb300: rg3_create failed: ") + rg_status_string(st));
  }
  ~GpuContext3D() { rg3_destroy(h_); }
  GpuContext3D(const GpuContext3D&) = delete;
  GpuContext3D& operator=(const GpuContext3D&) = delete;

  rg3_handle* handle() const { return h_; }
  int n_faces() const { return packed_.n_faces; }

  void check_gamma(const EquationOfState& eos) const {
    const IdealGas* ig = dynamic_cast<const IdealGas*>(&eos);
    if (!ig || ig->getAdiabaticIndex() != cfg_.gamma)
      throw UniversalError("rich_gb300: the equation of state must be IdealGas with the handle's gamma");
  }

  // Packs and uploads the tessellation unless it is the last upload's.
  void sync_mesh(const Tessellation3D& tess) const {
    if (have_mesh_ && unchanged(tess)) return;
    pack_tessellation3d(tess, packed_);
    key_.resize(3 * tess.GetPointNo());
    for (size_t i = 0; i < tess.GetPointNo(); ++i) {
      const Vector3D p = tess.GetMeshPoint(i);
      key_[3 * i] = p.x, key_[3 * i + 1] = p.y, key_[3 * i + 2] = p.z;
    }
    const rg_mesh3d_view v = packed_.view();
    check(rg3_upload_mesh(h_, &v));
    have_mesh_ = true;
    have_fv_ = false;
  }

  void upload_cells(const std::vector<three_dimenssional::ComputationalCell>& cells) const {
    if (static_cast<int32_t>(cells.size()) != packed_.n_cells)
      throw UniversalError("rich_gb300: cell count differs from the tessellation's");
    buf_.resize(5 * cells.size());
    for (size_t i = 0; i < cells.size(); ++i) {
      if (!cells[i].tracers.empty()) throw UniversalError("rich_gb300: the 3D path carries no tracers");
      buf_[5 * i] = cells[i].density;
      buf_[5 * i + 1] = cells[i].pressure;
      buf_[5 * i + 2] = cells[i].velocity.x;
      buf_[5 * i + 3] = cells[i].velocity.y;
      buf_[5 * i + 4] = cells[i].velocity.z;
    }
    check(rg3_set_cells(h_, buf_.data()));
  }

  // FirstOrderHydroFlux.cpp:100-110: a bulk face moves with
  // CalcFaceVelocity of its two points' velocities; boundary faces at rest.
  void sync_face_velocities(const Tessellation3D& tess, const std::vector<Vector3D>& pv) const {
    bool rest = true;
    for (const Vector3D& v : pv)
      if (v.x != 0 || v.y != 0 || v.z != 0) {
        rest = false;
        break;
      }
    if (rest) {
      if (!have_fv_ || !fv_rest_) check(rg3_set_face_velocities(h_, nullptr));
      fv_rest_ = true;
      have_fv_ = true;
      return;
    }
    const size_t nf = tess.GetTotalFacesNumber();
    fv_.assign(3 * nf, 0.0);
    for (size_t f = 0; f < nf; ++f) {
      if (tess.BoundaryFace(f)) continue;
      const Face& face = tess.GetFace(f);
      const Vector3D w = tess.CalcFaceVelocity(face.neighbors.first, face.neighbors.second,
                                               pv[face.neighbors.first], pv[face.neighbors.second]);
      fv_[3 * f] = w.x, fv_[3 * f + 1] = w.y, fv_[3 * f + 2] = w.z;
    }
    check(rg3_set_face_velocities(h_, fv_.data()));
    fv_rest_ = false;
    have_fv_ = true;
  }

  void check(rg_status st) const {
    if (st == RG_OK) return;
    rg_error e;
    rg3_last_error(h_, &e);
    UniversalError eo(rg_status_string(st));
    eo.AddEntry(e.phase == 3 ? "Face index" : "Cell index", static_cast<double>(e.index));
    eo.AddEntry("Value", e.value);
    throw eo;
  }

 private:
  bool unchanged(const Tessellation3D& tess) const {
    if (static_cast<int32_t>(tess.GetPointNo()) != packed_.n_cells ||
        static_cast<int32_t>(tess.GetTotalFacesNumber()) != packed_.n_faces)
      return false;
    for (size_t i = 0; i < tess.GetPointNo(); ++i) {
      const Vector3D p = tess.GetMeshPoint(i);
      if (std::memcmp(&p.x, &key_[3 * i], sizeof(double)) != 0 ||
          std::memcmp(&p.y, &key_[3 * i + 1], sizeof(double)) != 0 ||
          std::memcmp(&p.z, &key_[3 * i + 2], sizeof(double)) != 0)
        return false;
    }
    return true;
  }

  rg_config cfg_;
  rg3_handle* h_ = nullptr;
  mutable PackedMesh3D packed_;
  mutable std::vector<double> key_, buf_, fv_;
  mutable bool have_mesh_ = false, have_fv_ = false, fv_rest_ = false;
};

// CourantFriedrichsLewy (CourantFriedrichsLewy.cpp:40-46) with the handle's cfl
class GpuTimeStep3D : public TimeStepCalculator {
 public:
  explicit GpuTimeStep3D(const GpuContext3D& ctx) : ctx_(ctx) {}
  double operator()(const Tessellation3D& tess, const std::vector<three_dimenssional::ComputationalCell>& cells,
                    const EquationOfState& eos) const override {
    ctx_.check_gamma(eos);
    ctx_.sync_mesh(tess);
    ctx_.upload_cells(cells);
    double dt = 0;
    ctx_.check(rg3_cfl_dt(ctx_.handle(), &dt));
    return dt;
  }

 private:
  const GpuContext3D& ctx_;
};

// FirstOrderHydroFlux(Hllc) (FirstOrderHydroFlux.cpp:98-114)
class GpuFluxCalculator3D : public FluxCalculator3D {
 public:
  explicit GpuFluxCalculator3D(const GpuContext3D& ctx) : ctx_(ctx) {}
  std::vector<Conserved3D> operator()(const Tessellation3D& tess,
                                      const std::vector<three_dimenssional::ComputationalCell>& cells,
                                      const EquationOfState& eos,
                                      const std::vector<Vector3D>& point_velocities) const override {
    ctx_.check_gamma(eos);
    ctx_.sync_mesh(tess);
    ctx_.upload_cells(cells);
    ctx_.sync_face_velocities(tess, point_velocities);
    const size_t nf = static_cast<size_t>(ctx_.n_faces());
    std::vector<double> buf(5 * nf);
    ctx_.check(rg3_flux(ctx_.handle(), buf.data()));
    std::vector<Conserved3D> res(nf);
    for (size_t f = 0; f < nf; ++f) {
      res[f].mass = buf[5 * f];
      res[f].momentum = Vector3D(buf[5 * f + 1], buf[5 * f + 2], buf[5 * f + 3]);
      res[f].energy = buf[5 * f + 4];
    }
    return res;
  }

 private:
  const GpuContext3D& ctx_;
};

}  // namespace rich_gb300
#endif  // RICH_GB300_ADAPTERS3D_HPP
