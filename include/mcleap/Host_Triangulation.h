// Drop-in HostTriangulation (reference: include/Host_Triangulation.h:24-98).
//
// The host container of the mesh in the reference's AoS layout.  Construction
// seeds the +-1e7 bounding square; addDelaunayPoints sorts the caller's points
// in place into the reference's Morton order (vertex id = 4 + sorted index)
// and builds the Delaunay triangulation on the GPU through libmcl_gb300.so.
// delonize()/untangle() run the GPU engine on a temporary device copy.
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "../mcl_gb300.h"
#include "Common_Triangulation.h"

namespace mcleap_detail {
inline void check(int rc) {
  if (rc != MCL_OK) throw std::runtime_error(std::string("mcleap: ") + mcl_last_error());
}
}  // namespace mcleap_detail

struct HostTriangulation {
  std::vector<glm::vec2> m_pos;
  std::vector<Vertex> m_v;
  std::vector<HalfEdge> m_he;
  std::vector<Triangle> m_t;

  HostTriangulation() {
    m_pos = {glm::vec2(cood_min, cood_min), glm::vec2(cood_max, cood_min), glm::vec2(cood_max, cood_max),
             glm::vec2(cood_min, cood_max)};
    m_v = {{0, 0}, {1, 2}, {2, 6}, {3, 8}};
    m_he = {{2, 0, 0, 2}, {9, 1, -1, -1}, {4, 1, 0, 0}, {1, 2, -1, -1}, {0, 2, 0, 1},
            {6, 0, 1, 3}, {8, 2, 1, 0},   {3, 3, -1, -1}, {5, 3, 1, 2}, {7, 0, -1, -1}};
    m_t = {{4}, {5}};
  }

  // include/Host_Triangulation.h:296-300: sorts `points` in place.
  bool addDelaunayPoints(std::vector<glm::vec2>& points) {
    mcl_mesh* m = nullptr;
    mcleap_detail::check(
        mcl_mesh_build(reinterpret_cast<mcl_float2*>(points.data()), (int64_t)points.size(), &m));
    download(m);
    mcl_mesh_destroy(m);
    return true;
  }

  // include/Host_Triangulation.h:403-406
  bool movePoint(int p_index, glm::vec2 d) {
    m_pos[p_index] += d;
    return true;
  }

  // include/Host_Triangulation.h:77-80 (bodies at :408-413 return false in the
  // reference): move point p_index by d and leave a valid mesh.  Here every
  // variant steps a device copy of the mesh with that single displacement, so
  // the mesh is also Delaunay afterwards.
  bool moveFlipflop(int p_index, glm::vec2 d) { return move_one(p_index, d); }
  bool moveFlipflopDelaunay(int p_index, glm::vec2 d) { return move_one(p_index, d); }
  bool moveUntangling(int p_index, glm::vec2 d) { return move_one(p_index, d); }
  bool moveUntanglingDelaunay(int p_index, glm::vec2 d) { return move_one(p_index, d); }

  // include/Host_Triangulation.h:305-319 and :417-423, on the GPU: the result is
  // the Delaunay triangulation of the current positions.
  bool delonize() { return run_on_device(); }
  bool untangle() { return run_on_device(); }

  mcl_aos_view view() const {
    mcl_aos_view a;
    a.pos = reinterpret_cast<const mcl_float2*>(m_pos.data());
    a.v = reinterpret_cast<const int32_t*>(m_v.data());
    a.he = reinterpret_cast<const int32_t*>(m_he.data());
    a.t = reinterpret_cast<const int32_t*>(m_t.data());
    a.V = (int64_t)m_v.size();
    a.HE = (int64_t)m_he.size();
    a.T = (int64_t)m_t.size();
    return a;
  }

  void download(mcl_mesh* m) {
    int64_t V = 0, HE = 0, T = 0;
    mcleap_detail::check(mcl_mesh_sizes(m, &V, &HE, &T));
    m_pos.resize(V);
    m_v.resize(V);
    m_he.resize(HE);
    m_t.resize(T);
    mcleap_detail::check(mcl_mesh_download_aos(m, reinterpret_cast<mcl_float2*>(m_pos.data()),
                                               reinterpret_cast<int32_t*>(m_v.data()),
                                               reinterpret_cast<int32_t*>(m_he.data()),
                                               reinterpret_cast<int32_t*>(m_t.data())));
  }

 private:
  bool move_one(int p, glm::vec2 d) {
    if (p < 4 || p >= (int)m_pos.size()) return false;  // the bounding corners stay
    std::vector<glm::vec2> disp(m_pos.size(), glm::vec2(0.f, 0.f));
    disp[(size_t)p] = d;
    mcl_aos_view a = view();
    mcl_mesh* m = nullptr;
    mcleap_detail::check(mcl_mesh_create_from_aos(&a, &m));
    mcl_step_stats st;
    const int rc = mcl_step_host(m, reinterpret_cast<const mcl_float2*>(disp.data()), nullptr, &st);
    if (rc == MCL_OK) download(m);
    mcl_mesh_destroy(m);
    mcleap_detail::check(rc);
    return true;
  }
  bool run_on_device() {
    mcl_aos_view a = view();
    mcl_mesh* m = nullptr;
    mcleap_detail::check(mcl_mesh_create_from_aos(&a, &m));
    mcl_step_stats st;
    const int rc = mcl_delaunay_restore(m, nullptr, &st);
    if (rc == MCL_OK) download(m);
    mcl_mesh_destroy(m);
    mcleap_detail::check(rc);
    return st.lawson_flips > 0 || st.removed_vertices > 0;
  }
};
