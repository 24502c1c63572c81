// rich_gpu_adapters.hpp -- RICH plugin classes backed by the GB300 library.
//
// Header-only C++ that a RICH build includes (include path = the RICH source
// root plus this directory and include/), linking librich_gb300.so.  Each
// class derives from the reference's own abstract interface, so hdsim
// (source/newtonian/two_dimensional/hdsim2d.hpp:43) drives them unchanged:
//
//   GpuCFL                : TimeStepFunction  (time_step_function.hpp:16-39)
//   GpuFluxCalculator     : FluxCalculator    (flux_calculator_2d.hpp:19-48)
//   GpuExtensiveUpdater   : ExtensiveUpdater  (extensive_updater.hpp:19-47)
//   GpuCellUpdater        : CellUpdater       (cell_updater_2d.hpp:20-45)
//
// All four share one GpuContext (one rg_handle).  Per call they upload what
// hdsim passes, run the matching C-ABI operation and copy the result back
// into hdsim's vectors.  The tessellation is packed and uploaded only when it
// changed: the context keeps the mesh points (real and ghost) of the last
// upload, and a tessellation with the same point count, edge count and
// bitwise-equal points is the same Voronoi mesh (VoronoiMesh builds it
// deterministically from its points), so an Eulerian rebuild and the calls
// that follow a step's MoveMeshPoints reuse the upload.  With
// set_outer_boundary the device computes the volumes and CMs itself
// (RG_MESH_DEVICE_GEOMETRY, bit-identical to the reference's), so the host
// packs only points, topology and face vertices and never evaluates
// CacheData's lazy volumes.  The fluxes stay on the device between the flux
// calculator and the extensive updater.  A physical failure is rethrown as
// the reference's UniversalError with its message and diagnostic entries.
//
// Supported: IdealGas, Hllc (massflux = true), SlabSymmetry or
// CylindricalSymmetry, first order (SimpleFluxCalculator) or
// LinearGaussImproved with RigidWallGenerator or PeriodicGhostGenerator, and
// tracers and stickers: the GpuTracerSpec names what the replaced plugins
// were built with (LinearGaussImproved's calc_tracers and skip_key, the
// sticker of a SimpleCellUpdater sequence {(HasSticker, SkipUpdate)}); the
// "Entropy" tracer is recomputed as SimpleCellUpdater does.
#ifndef RICH_GB300_ADAPTERS_HPP
#define RICH_GB300_ADAPTERS_HPP

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "rich_gb300.h"
#include "rich_pack.hpp"
#include "source/misc/universal_error.hpp"
#include "source/newtonian/common/ideal_gas.hpp"
#include "source/newtonian/two_dimensional/cell_updater_2d.hpp"
#include "source/newtonian/two_dimensional/extensive_updater.hpp"
#include "source/newtonian/two_dimensional/OuterBoundary.hpp"
#include "source/newtonian/two_dimensional/flux_calculator_2d.hpp"
#include "source/newtonian/two_dimensional/physical_geometry.hpp"
#include "source/newtonian/two_dimensional/time_step_function.hpp"

namespace rich_gb300 {

// What the replaced reference plugins were constructed with.
struct GpuTracerSpec {
  std::vector<std::string> calc_tracers;  // LinearGaussImproved(..., calc_tracers, skip_key)
  std::string skip_key;                   // "" = none
  std::string frozen_sticker;             // SimpleCellUpdater's HasSticker(name) + SkipUpdate, "" = none
};

class GpuContext {
 public:
  explicit GpuContext(const rg_config& cfg, GpuTracerSpec spec = GpuTracerSpec()) : cfg_(cfg), spec_(spec) {
    const rg_status st = rg_create(&cfg_, &h_);
    if (st != RG_OK) throw UniversalError(std::string("rich_gb300: rg_create failed: ") + rg_status_string(st));
  }
  ~GpuContext() { rg_destroy(h_); }
  GpuContext(const GpuContext&) = delete;
  GpuContext& operator=(const GpuContext&) = delete;

  rg_handle* handle() const { return h_; }
  const rg_config& config() const { return cfg_; }
  int n_cells() const { return packed_.n_cells; }
  int n_faces() const { return packed_.n_faces; }

  // The PhysicalGeometry whose CacheData areas scale the fluxes; hdsim passes
  // it to the extensive and cell updaters, the flux calculator sees only the
  // CacheData, so a cylindrical simulation names it up front.
  void set_physical_geometry(const PhysicalGeometry& pg) const {
    rg_physical_geometry g{RG_GEOMETRY_SLAB, {0, 0}, {0, 1}, 1};
    if (const CylindricalSymmetry* c = dynamic_cast<const CylindricalSymmetry*>(&pg)) {
      const Axis& a = c->getAxis();
      g = rg_physical_geometry{RG_GEOMETRY_CYLINDRICAL, {a.origin.x, a.origin.y}, {a.direction.x, a.direction.y}, 1};
    }
    if (g.kind != pgeo_.kind || g.origin[0] != pgeo_.origin[0] || g.origin[1] != pgeo_.origin[1] ||
        g.direction[0] != pgeo_.direction[0] || g.direction[1] != pgeo_.direction[1]) {
      pgeo_ = g;
      check(rg_set_physical_geometry(h_, &pgeo_));
      have_mesh_ = false;  // the areas are formed at upload
    }
  }

  // The simulation's outer boundary: the device then forms the cell volumes
  // and CMs (ghost CMs reflected about, or shifted across, its sides) from
  // the points and face vertices, and the host packs no geometry.
  void set_outer_boundary(const OuterBoundary& ob) const {
    check(rg_set_outer_box(h_, ob.GetGridBoundary(Left), ob.GetGridBoundary(Right), ob.GetGridBoundary(Down),
                           ob.GetGridBoundary(Up)));
    if (!device_geometry_) have_mesh_ = false;
    device_geometry_ = true;
  }

  // Packs the tessellation and uploads it unless it is the last upload's.
  // Without device geometry the packed CacheData volumes need the
  // simulation's CacheData; a call without one (the time-step function)
  // packs slab volumes, which the next call that has the CacheData replaces.
  void sync_mesh(const Tessellation& tess, const CacheData* cd) const {
    const bool replace_provisional = provisional_ && cd && !device_geometry_;
    if (have_mesh_ && !replace_provisional && mesh_unchanged(tess)) return;
    if (device_geometry_) {
      pack_topology(tess, packed_);
      provisional_ = false;
    } else if (cd) {
      pack_tessellation(tess, *cd, packed_);
      provisional_ = false;
    } else {
      SlabSymmetry pg;
      CacheData local(tess, pg);
      pack_tessellation(tess, local, packed_);
      provisional_ = true;
    }
    remember_points(tess);
    const rg_mesh_view v = packed_.view();
    check(rg_upload_mesh(h_, &v, device_geometry_ ? RG_MESH_DEVICE_GEOMETRY : 0u));
    have_mesh_ = true;
    ++mesh_generation_;
  }
  unsigned long mesh_generation() const { return mesh_generation_; }

  // Tracer configuration from hdsim's sorted names (hdsim2d.cpp:121-136) and
  // the spec; set once, from the first cells with tracers or stickers.
  void sync_tracers(const std::vector<ComputationalCell>& cells, const TracerStickerNames& tsn) const {
    const size_t nt = cells.empty() ? 0 : cells[0].tracers.size();
    const size_t ns = cells.empty() ? 0 : cells[0].stickers.size();
    if (nt == 0 && ns == 0) return;
    if (nt > RG_MAX_TRACERS || ns > 32)
      throw UniversalError("rich_gb300: more tracers or stickers than the library holds");
    rg_tracer_config c{static_cast<int32_t>(nt), static_cast<int32_t>(ns), 0u, -1, -1, -1};
    for (size_t j = 0; j < nt && j < tsn.tracer_names.size(); ++j) {
      for (const std::string& name : spec_.calc_tracers)
        if (name == tsn.tracer_names[j]) c.limited_mask |= 1u << j;
      if (tsn.tracer_names[j] == "Entropy") c.entropy_tracer = static_cast<int32_t>(j);
    }
    for (size_t k = 0; k < ns && k < tsn.sticker_names.size(); ++k) {
      if (!spec_.skip_key.empty() && tsn.sticker_names[k] == spec_.skip_key) c.skip_sticker = static_cast<int32_t>(k);
      if (!spec_.frozen_sticker.empty() && tsn.sticker_names[k] == spec_.frozen_sticker)
        c.frozen_sticker = static_cast<int32_t>(k);
    }
    if (!have_tcfg_ || std::memcmp(&c, &tcfg_, sizeof c) != 0) {
      check(rg_set_tracer_config(h_, &c));
      tcfg_ = c;
      have_tcfg_ = true;
    }
  }
  int n_tracers() const { return have_tcfg_ ? tcfg_.n_tracers : 0; }
  // ConditionActionSequence / ConditionActionSequence2 in place of the
  // Simple/ModularFluxCalculator (rg_flux_rule rows; see rich_gb300.h).
  // RegularSpecialEdge reads the cells' stickers, which sync_tracers keeps.
  void set_flux_rules(const std::vector<rg_flux_rule>& rules) const {
    check(rg_set_flux_rules(h_, static_cast<int32_t>(rules.size()), rules.empty() ? nullptr : rules.data()));
  }
  // LagrangianExtensiveUpdater(lflux, SimpleExtensiveUpdater) in place of
  // SimpleExtensiveUpdater, for rules with RG_ACT_LAGRANGIAN (LagrangianFlux)
  void set_lagrangian_updater(bool on) const { check(rg_set_lagrangian_updater(h_, on ? 1 : 0)); }
  bool tracers_configured() const { return have_tcfg_; }

  void upload_cells(const std::vector<ComputationalCell>& cells) const {
    std::vector<double> buf(4 * cells.size());
    for (size_t i = 0; i < cells.size(); ++i) {
      buf[4 * i] = cells[i].density;
      buf[4 * i + 1] = cells[i].pressure;
      buf[4 * i + 2] = cells[i].velocity.x;
      buf[4 * i + 3] = cells[i].velocity.y;
    }
    check(rg_set_cells(h_, buf.data()));
    if (!have_tcfg_) return;
    const size_t nt = static_cast<size_t>(tcfg_.n_tracers);
    if (nt > 0) {
      std::vector<double> tr(nt * cells.size());
      for (size_t i = 0; i < cells.size(); ++i)
        for (size_t j = 0; j < nt; ++j) tr[i * nt + j] = cells[i].tracers[j];
      check(rg_set_tracers(h_, tr.data()));
    }
    std::vector<uint32_t> st(cells.size(), 0u);
    for (size_t i = 0; i < cells.size(); ++i)
      for (size_t k = 0; k < cells[i].stickers.size() && k < 32; ++k)
        if (cells[i].stickers[k]) st[i] |= 1u << k;
    check(rg_set_stickers(h_, st.data()));
  }
  void upload_extensives(const std::vector<Extensive>& ext) const {
    std::vector<double> buf(4 * ext.size());
    for (size_t i = 0; i < ext.size(); ++i) {
      buf[4 * i] = ext[i].mass;
      buf[4 * i + 1] = ext[i].energy;
      buf[4 * i + 2] = ext[i].momentum.x;
      buf[4 * i + 3] = ext[i].momentum.y;
    }
    check(rg_set_extensives(h_, buf.data()));
    const size_t nt = static_cast<size_t>(n_tracers());
    if (nt > 0) {
      std::vector<double> tr(nt * ext.size());
      for (size_t i = 0; i < ext.size(); ++i)
        for (size_t j = 0; j < nt; ++j) tr[i * nt + j] = ext[i].tracers[j];
      check(rg_set_extensive_tracers(h_, tr.data()));
    }
  }
  void download_extensives(std::vector<Extensive>& ext) const {
    std::vector<double> buf(4 * ext.size());
    check(rg_get_extensives(h_, buf.data()));
    for (size_t i = 0; i < ext.size(); ++i) {
      ext[i].mass = buf[4 * i];
      ext[i].energy = buf[4 * i + 1];
      ext[i].momentum.x = buf[4 * i + 2];
      ext[i].momentum.y = buf[4 * i + 3];
    }
    const size_t nt = static_cast<size_t>(n_tracers());
    if (nt > 0) {
      std::vector<double> tr(nt * ext.size());
      check(rg_get_extensive_tracers(h_, tr.data()));
      for (size_t i = 0; i < ext.size(); ++i) {
        ext[i].tracers.resize(nt);
        for (size_t j = 0; j < nt; ++j) ext[i].tracers[j] = tr[i * nt + j];
      }
    }
  }
  void upload_edge_velocities(const std::vector<Vector2D>& ev) const {
    std::vector<double> buf(2 * ev.size());
    for (size_t i = 0; i < ev.size(); ++i) {
      buf[2 * i] = ev[i].x;
      buf[2 * i + 1] = ev[i].y;
    }
    check(rg_set_edge_velocities(h_, buf.data()));
  }

  // Fluxes the GPU flux calculator left on the device, identified by the
  // buffer hdsim received (hdsim2d.cpp:176-195 passes that same vector on).
  void mark_device_fluxes(const std::vector<Extensive>& f) const {
    flux_data_ = f.data();
    flux_size_ = f.size();
    flux_generation_ = mesh_generation_;
  }
  bool device_fluxes_match(const std::vector<Extensive>& f) const {
    return flux_data_ == f.data() && flux_size_ == f.size() && flux_generation_ == mesh_generation_;
  }

  void check_gamma(const EquationOfState& eos) const {
    const IdealGas* ig = dynamic_cast<const IdealGas*>(&eos);
    if (!ig || ig->getAdiabaticIndex() != cfg_.gamma)
      throw UniversalError("rich_gb300: the equation of state must be IdealGas with the handle's gamma");
  }

  // Converts a failure into the reference's UniversalError.
  void check(rg_status st) const {
    if (st == RG_OK) return;
    rg_error e;
    rg_last_error(h_, &e);
    UniversalError eo(rg_status_string(st));
    if (st == RG_ERR_NEGATIVE_DENSITY || st == RG_ERR_NEGATIVE_ENERGY ||
        st == RG_ERR_SINGULAR_MATRIX || st == RG_ERR_TOO_MANY_NEIGHBORS)
      eo.AddEntry("Cell index", static_cast<double>(e.index));
    else
      eo.AddEntry("Edge index", static_cast<double>(e.index));
    eo.AddEntry("Value", e.value);
    throw eo;
  }

 private:
  // Same point count, edge count and bitwise-equal points (real and ghost)
  // as at the last upload.
  bool mesh_unchanged(const Tessellation& tess) const {
    const int total = tess.GetTotalPointNumber();
    if (tess.GetPointNo() != packed_.n_cells || static_cast<int>(tess.getAllEdges().size()) != packed_.n_faces ||
        2 * static_cast<size_t>(total) != key_points_.size())
      return false;
    for (int i = 0; i < total; ++i) {
      const Vector2D p = tess.GetMeshPoint(i);
      if (std::memcmp(&p.x, &key_points_[2 * static_cast<size_t>(i)], sizeof(double)) != 0 ||
          std::memcmp(&p.y, &key_points_[2 * static_cast<size_t>(i) + 1], sizeof(double)) != 0)
        return false;
    }
    return true;
  }
  void remember_points(const Tessellation& tess) const {
    const int total = tess.GetTotalPointNumber();
    key_points_.resize(2 * static_cast<size_t>(total));
    for (int i = 0; i < total; ++i) {
      const Vector2D p = tess.GetMeshPoint(i);
      key_points_[2 * static_cast<size_t>(i)] = p.x;
      key_points_[2 * static_cast<size_t>(i) + 1] = p.y;
    }
  }

  rg_config cfg_;
  GpuTracerSpec spec_;
  rg_handle* h_ = nullptr;
  mutable rg_tracer_config tcfg_{0, 0, 0u, -1, -1, -1};
  mutable bool have_tcfg_ = false;
  mutable rg_physical_geometry pgeo_{RG_GEOMETRY_SLAB, {0, 0}, {0, 1}, 1};
  mutable PackedMesh packed_;
  mutable std::vector<double> key_points_;
  mutable bool have_mesh_ = false;
  mutable bool device_geometry_ = false;
  mutable bool provisional_ = false;
  mutable unsigned long mesh_generation_ = 0;
  mutable const Extensive* flux_data_ = nullptr;
  mutable size_t flux_size_ = 0;
  mutable unsigned long flux_generation_ = 0;
};

// SimpleCFL (simple_cfl.cpp:58-71)
class GpuCFL : public TimeStepFunction {
 public:
  explicit GpuCFL(const GpuContext& ctx) : ctx_(ctx) {}
  double operator()(const Tessellation& tess, const vector<ComputationalCell>& cells, const EquationOfState& eos,
                    const vector<Vector2D>& edge_velocities, const double /*time*/,
                    TracerStickerNames const& tsn) const override {
    ctx_.check_gamma(eos);
    ctx_.sync_mesh(tess, nullptr);
    ctx_.sync_tracers(cells, tsn);
    ctx_.upload_cells(cells);
    ctx_.upload_edge_velocities(edge_velocities);
    double dt = 0;
    ctx_.check(rg_cfl_dt(ctx_.handle(), &dt));
    return dt;
  }

 private:
  const GpuContext& ctx_;
};

// SimpleFluxCalculator / ModularFluxCalculator(LinearGaussImproved, Hllc)
class GpuFluxCalculator : public FluxCalculator {
 public:
  explicit GpuFluxCalculator(const GpuContext& ctx) : ctx_(ctx) {}
  vector<Extensive> operator()(const Tessellation& tess, const vector<Vector2D>& edge_velocities,
                               const vector<ComputationalCell>& cells, const vector<Extensive>& /*extensives*/,
                               const CacheData& cd, const EquationOfState& eos, const double /*time*/,
                               const double dt, TracerStickerNames const& tsn) const override {
    ctx_.check_gamma(eos);
    ctx_.sync_mesh(tess, &cd);
    ctx_.sync_tracers(cells, tsn);
    ctx_.upload_cells(cells);
    ctx_.upload_edge_velocities(edge_velocities);
    std::vector<double> buf(4 * static_cast<size_t>(ctx_.n_faces()));
    ctx_.check(rg_flux(ctx_.handle(), dt, buf.data()));
    vector<Extensive> res(static_cast<size_t>(ctx_.n_faces()));
    for (size_t i = 0; i < res.size(); ++i) {
      res[i].mass = buf[4 * i];
      res[i].energy = buf[4 * i + 1];
      res[i].momentum.x = buf[4 * i + 2];
      res[i].momentum.y = buf[4 * i + 3];
    }
    const size_t nt = static_cast<size_t>(ctx_.n_tracers());
    if (nt > 0) {
      std::vector<double> tf(nt * res.size());
      ctx_.check(rg_get_tracer_fluxes(ctx_.handle(), tf.data()));
      for (size_t i = 0; i < res.size(); ++i) res[i].tracers.assign(tf.begin() + i * nt, tf.begin() + (i + 1) * nt);
    }
    ctx_.mark_device_fluxes(res);
    return res;
  }

 private:
  const GpuContext& ctx_;
};

// SimpleExtensiveUpdater (simple_extensive_updater.cpp:11-35)
class GpuExtensiveUpdater : public ExtensiveUpdater {
 public:
  explicit GpuExtensiveUpdater(const GpuContext& ctx) : ctx_(ctx) {}
  void operator()(const vector<Extensive>& fluxes, const PhysicalGeometry& pg, const Tessellation& tess,
                  const double dt, const CacheData& cd, const vector<ComputationalCell>& cells,
                  vector<Extensive>& extensives, double /*time*/, TracerStickerNames const& tsn) const override {
    ctx_.set_physical_geometry(pg);
    ctx_.sync_mesh(tess, &cd);
    ctx_.sync_tracers(cells, tsn);
    if (!ctx_.device_fluxes_match(fluxes)) {
      std::vector<double> buf(4 * fluxes.size());
      for (size_t i = 0; i < fluxes.size(); ++i) {
        buf[4 * i] = fluxes[i].mass;
        buf[4 * i + 1] = fluxes[i].energy;
        buf[4 * i + 2] = fluxes[i].momentum.x;
        buf[4 * i + 3] = fluxes[i].momentum.y;
      }
      ctx_.check(rg_set_fluxes(ctx_.handle(), buf.data()));
      const size_t nt = static_cast<size_t>(ctx_.n_tracers());
      if (nt > 0) {
        std::vector<double> tf(nt * fluxes.size());
        for (size_t i = 0; i < fluxes.size(); ++i)
          for (size_t j = 0; j < nt; ++j) tf[i * nt + j] = fluxes[i].tracers[j];
        ctx_.check(rg_set_tracer_fluxes(ctx_.handle(), tf.data()));
      }
    }
    ctx_.upload_extensives(extensives);
    ctx_.check(rg_extensive_update(ctx_.handle(), dt));
    ctx_.download_extensives(extensives);
  }

 private:
  const GpuContext& ctx_;
};

// SimpleCellUpdater without a condition/action sequence (simple_cell_updater.cpp:85-106)
class GpuCellUpdater : public CellUpdater {
 public:
  explicit GpuCellUpdater(const GpuContext& ctx) : ctx_(ctx) {}
  vector<ComputationalCell> operator()(const Tessellation& tess, const PhysicalGeometry& pg,
                                       const EquationOfState& eos, vector<Extensive>& extensives,
                                       const vector<ComputationalCell>& old, const CacheData& cd,
                                       TracerStickerNames const& tsn) const override {
    ctx_.check_gamma(eos);
    ctx_.set_physical_geometry(pg);
    ctx_.sync_mesh(tess, &cd);
    ctx_.sync_tracers(old, tsn);
    if (ctx_.tracers_configured()) ctx_.upload_cells(old);  // tracers / SkipUpdate read the old cells
    ctx_.upload_extensives(extensives);
    ctx_.check(rg_cell_update(ctx_.handle()));
    std::vector<double> buf(4 * extensives.size());
    ctx_.check(rg_get_cells(ctx_.handle(), buf.data()));
    vector<ComputationalCell> res(extensives.size());
    for (size_t i = 0; i < res.size(); ++i) {
      res[i].density = buf[4 * i];
      res[i].pressure = buf[4 * i + 1];
      res[i].velocity = Vector2D(buf[4 * i + 2], buf[4 * i + 3]);
      if (i < old.size()) res[i].stickers = old[i].stickers;  // simple_cell_updater.cpp:36
    }
    const size_t nt = static_cast<size_t>(ctx_.n_tracers());
    if (nt > 0) {
      std::vector<double> tr(nt * res.size());
      ctx_.check(rg_get_tracers(ctx_.handle(), tr.data()));
      for (size_t i = 0; i < res.size(); ++i) res[i].tracers.assign(tr.begin() + i * nt, tr.begin() + (i + 1) * nt);
      ctx_.download_extensives(extensives);  // the entropy tracer's extensive (simple_cell_updater.cpp:47)
    }
    return res;
  }

 private:
  const GpuContext& ctx_;
};

}  // namespace rich_gb300
#endif  // RICH_GB300_ADAPTERS_HPP
