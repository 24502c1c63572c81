// rich_pack.hpp -- packs a RICH Tessellation (+ CacheData) into the flat
// rg_mesh_view the GB300 hot path consumes.
//
// Header-only; compiled together with RICH's own headers (include path = the
// RICH source root).  Used by the plugin adapters in rich_gpu_adapters.hpp and
// by the fixture generator oracle/ref/ref_dump.cpp.
//
// What is read, and where the reference reads the same thing:
//   mesh points      Tessellation::GetMeshPoint      (simple_flux_calculator.cpp:92-93,
//                                                     LinearGaussImproved.cpp:11-25)
//   cell CMs         Tessellation::GetCellCM          (LinearGaussImproved.cpp:27-41)
//   volumes          Tessellation::GetVolume          (LinearGaussImproved.cpp:467, via GetWidth simple_cfl.cpp:31)
//   cd volumes       CacheData::volumes               (simple_cell_updater.cpp:31)
//   edges            Tessellation::getAllEdges        (simple_extensive_updater.cpp:21)
//   cell->edges      Tessellation::GetCellEdges       (LinearGaussImproved.cpp:565, simple_cfl.cpp:40)
//   ghost origin     Tessellation::GetOriginalIndex   (RigidWallGenerator.cpp:28, PeriodicGhostGenerator.cpp:11)
// Ghost points (index >= GetPointNo()) are renumbered densely in the order
// in which ascending edges first touch them; ghost_face records that first
// edge, which is the entry RigidWallGenerator's flat_map keeps
// (RigidWallGenerator.cpp:20-35 inserts per boundary edge, first one wins).
#ifndef RICH_GB300_PACK_HPP
#define RICH_GB300_PACK_HPP

#include <cstdint>
#include <stdexcept>
#include <vector>

#include "rich_gb300.h"
#include "source/newtonian/two_dimensional/cache_data.hpp"
#include "source/tessellation/tessellation.hpp"

namespace rich_gb300 {

struct PackedMesh {
  int32_t n_cells = 0, n_ghosts = 0, n_faces = 0;
  std::vector<double> point_xy, cm_xy, volume, cd_volume, face_vertices;
  std::vector<int32_t> ghost_source, ghost_face, face_cells, cell_face_offset, cell_faces;
  std::vector<int> ghost_point;  // reference point index of each packed ghost

  rg_mesh_view view() const {
    rg_mesh_view v;
    v.n_cells = n_cells;
    v.n_ghosts = n_ghosts;
    v.n_faces = n_faces;
    v.reserved = 0;
    v.point_xy = point_xy.data();
    v.cm_xy = cm_xy.empty() ? nullptr : cm_xy.data();
    v.volume = volume.empty() ? nullptr : volume.data();
    v.cd_volume = cd_volume.empty() ? nullptr : cd_volume.data();
    v.ghost_source = ghost_source.data();
    v.ghost_face = ghost_face.data();
    v.face_cells = face_cells.data();
    v.face_vertices = face_vertices.data();
    v.cell_face_offset = cell_face_offset.data();
    v.cell_faces = cell_faces.data();
    return v;
  }
};

// Topology, mesh points and face vertices: what the device needs when it
// computes the volumes and CMs itself (RG_MESH_DEVICE_GEOMETRY).  cm_xy,
// volume and cd_volume are left empty.
inline void pack_topology(const Tessellation& tess, PackedMesh& m) {
  const int n = tess.GetPointNo();
  const int total = tess.GetTotalPointNumber();
  const std::vector<Edge>& edges = tess.getAllEdges();
  const int ne = static_cast<int>(edges.size());
  m.n_cells = n;
  m.n_faces = ne;
  m.ghost_point.clear();
  m.ghost_face.clear();
  // ghost points are tessellation indices in [n, total): a dense slot table
  std::vector<int32_t> slot(total > n ? static_cast<size_t>(total - n) : 0, -1);
  m.face_cells.resize(2 * static_cast<size_t>(ne));
  m.face_vertices.resize(4 * static_cast<size_t>(ne));
  for (int e = 0; e < ne; ++e) {
    const Edge& edge = edges[static_cast<size_t>(e)];
    const int nb[2] = {edge.neighbors.first, edge.neighbors.second};
    for (int s = 0; s < 2; ++s) {
      int32_t id = nb[s];
      if (nb[s] < 0 || nb[s] >= total) throw std::runtime_error("rich_pack: edge neighbour outside the tessellation");
      if (nb[s] >= n) {
        int32_t& g = slot[static_cast<size_t>(nb[s] - n)];
        if (g < 0) {
          g = static_cast<int32_t>(m.ghost_point.size());
          m.ghost_point.push_back(nb[s]);
          m.ghost_face.push_back(e);
        }
        id = n + g;
      }
      m.face_cells[2 * static_cast<size_t>(e) + s] = id;
    }
    double* fv = &m.face_vertices[4 * static_cast<size_t>(e)];
    fv[0] = edge.vertices.first.x;
    fv[1] = edge.vertices.first.y;
    fv[2] = edge.vertices.second.x;
    fv[3] = edge.vertices.second.y;
  }
  const int ng = static_cast<int>(m.ghost_point.size());
  m.n_ghosts = ng;
  const size_t np = static_cast<size_t>(n + ng);
  m.point_xy.resize(2 * np);
  m.ghost_source.resize(static_cast<size_t>(ng));
  for (size_t p = 0; p < np; ++p) {
    const int ref = p < static_cast<size_t>(n) ? static_cast<int>(p) : m.ghost_point[p - n];
    const Vector2D x = tess.GetMeshPoint(ref);
    m.point_xy[2 * p] = x.x;
    m.point_xy[2 * p + 1] = x.y;
    if (p >= static_cast<size_t>(n)) m.ghost_source[p - n] = tess.GetOriginalIndex(ref);
  }
  m.cell_face_offset.resize(static_cast<size_t>(n) + 1);
  m.cell_faces.resize(static_cast<size_t>(2 * ne));
  m.cell_face_offset[0] = 0;
  size_t k = 0;
  for (int i = 0; i < n; ++i) {
    const std::vector<int>& ce = tess.GetCellEdges(i);
    if (k + ce.size() > m.cell_faces.size()) throw std::runtime_error("rich_pack: more cell faces than 2 per edge");
    for (size_t j = 0; j < ce.size(); ++j) {
      if (j > 0 && ce[j] <= ce[j - 1])
        throw std::runtime_error("rich_pack: GetCellEdges is not in ascending edge order");
      m.cell_faces[k++] = ce[j];
    }
    m.cell_face_offset[static_cast<size_t>(i) + 1] = static_cast<int32_t>(k);
  }
  m.cell_faces.resize(k);
  m.cm_xy.clear();
  m.volume.clear();
  m.cd_volume.clear();
}

// Everything, with the volumes and CMs the host tessellation and CacheData
// computed (uploaded without RG_MESH_DEVICE_GEOMETRY).
inline void pack_tessellation(const Tessellation& tess, const CacheData& cd, PackedMesh& m) {
  pack_topology(tess, m);
  const int n = m.n_cells;
  const size_t np = static_cast<size_t>(n + m.n_ghosts);
  m.cm_xy.resize(2 * np);
  for (size_t p = 0; p < np; ++p) {
    const int ref = p < static_cast<size_t>(n) ? static_cast<int>(p) : m.ghost_point[p - n];
    const Vector2D& c = tess.GetCellCM(ref);
    m.cm_xy[2 * p] = c.x;
    m.cm_xy[2 * p + 1] = c.y;
  }
  m.volume.resize(static_cast<size_t>(n));
  m.cd_volume.resize(static_cast<size_t>(n));
  for (int i = 0; i < n; ++i) {
    m.volume[static_cast<size_t>(i)] = tess.GetVolume(i);
    m.cd_volume[static_cast<size_t>(i)] = cd.volumes[static_cast<size_t>(i)];
  }
}

}  // namespace rich_gb300
#endif  // RICH_GB300_PACK_HPP
