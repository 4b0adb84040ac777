// Periodic (flat torus) triangulation for C++ callers, over libmcl_gb300.so.
//
// The reference only announces this class (include/Host_PeriodicTriangulation.h:
// a HostTriangulation whose constructor keeps a CGAL periodic domain, :101-104,
// commented out; none of its members work).  This header gives the working form
// with the reference's member names where they apply: points on the torus
// [2L, 3L)^2 (L a power of two, so translates by one period are exact floats),
// ids in the caller's order, no bounding corners, 3n edges and 2n faces.  The
// device mesh stores ev / en as the planar engine plus one offset word per edge
// (include/mcl_gb300.h, "periodic meshes").
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../mcl_gb300.h"
#include "Common_Triangulation.h"

struct PeriodicTriangulation {
  int64_t n = 0, E = 0;
  float L = 0.f;
  mcl_step_stats last_stats{};
  int64_t last_wrapped = 0;

  // the exact periodic Delaunay triangulation of `points` (built on the GPU)
  PeriodicTriangulation(const std::vector<glm::vec2>& points, float period) {
    check(mcl_periodic_build(reinterpret_cast<const mcl_float2*>(points.data()), (int64_t)points.size(), period,
                             &mesh));
    check(mcl_periodic_sizes(mesh, &n, &E, &L));
  }
  ~PeriodicTriangulation() { mcl_periodic_destroy(mesh); }
  PeriodicTriangulation(const PeriodicTriangulation&) = delete;
  PeriodicTriangulation& operator=(const PeriodicTriangulation&) = delete;

  // movePoints + untangle + delonize on the torus (d: device array of n
  // glm::vec2): moves that would turn faces over are refused vertex by vertex,
  // resumed by sub-steps, the rest removed and reinserted at their targets;
  // false (message in mcl_last_error()) on failure
  bool step(const glm::vec2* d, void* stream = nullptr) {
    return mcl_periodic_step(mesh, reinterpret_cast<const mcl_float2*>(d), stream, &last_stats, &last_wrapped) ==
           MCL_OK;
  }

  // step with the displacements in host memory
  bool step_host(const std::vector<glm::vec2>& d, void* stream = nullptr) {
    if ((int64_t)d.size() != n) return false;
    return mcl_periodic_step_host(mesh, reinterpret_cast<const mcl_float2*>(d.data()), stream, &last_stats,
                                  &last_wrapped) == MCL_OK;
  }

  // oneRing<M> / oneRing2<M>: clockwise from the smallest (id, offset); offs
  // (may be null): each neighbour's copy offset byte
  template <int M>
  bool oneRing(int* ring, uint8_t* offs = nullptr, void* stream = nullptr) {
    return mcl_periodic_one_ring(mesh, M, MCL_LAYOUT_COLUMN, ring, offs, stream, nullptr) == MCL_OK;
  }
  template <int M>
  bool oneRing2(int* ring, uint8_t* offs = nullptr, void* stream = nullptr) {
    return mcl_periodic_one_ring(mesh, M, MCL_LAYOUT_ROW, ring, offs, stream, nullptr) == MCL_OK;
  }
  // closestNeighbors<M> from a oneRing<M> table and its offsets
  template <int M>
  bool closestNeighbors(const int* ring, const uint8_t* offs, int* closest, void* stream = nullptr) {
    return mcl_periodic_closest(mesh, M, MCL_LAYOUT_COLUMN, ring, offs, closest, stream) == MCL_OK;
  }
  // getFRNN<M, F>: every other point with a copy within r (< L / 2); the
  // ring table of the reference's signature is not needed
  template <int M, int F>
  bool getFRNN(float r, const int* /*ring*/, int* neighbors, uint8_t* offs = nullptr, void* stream = nullptr) {
    return mcl_periodic_frnn(mesh, r, F, MCL_LAYOUT_COLUMN, neighbors, offs, stream, nullptr) == MCL_OK;
  }

  // transferToHost: positions (canonical, in [2L, 3L)^2) and the edge records
  void transferToHost(std::vector<glm::vec2>& pos, std::vector<int32_t>& ev, std::vector<int32_t>& en,
                      std::vector<uint32_t>& eo) {
    pos.resize((size_t)n);
    ev.resize((size_t)(4 * E));
    en.resize((size_t)(4 * E));
    eo.resize((size_t)E);
    check(mcl_periodic_download(mesh, reinterpret_cast<mcl_float2*>(pos.data()), ev.data(), en.data(), eo.data()));
  }
  // m_pos on the device (n glm::vec2)
  glm::vec2* positions() {
    mcl_float2* p = nullptr;
    check(mcl_periodic_positions(mesh, &p));
    return reinterpret_cast<glm::vec2*>(p);
  }

 private:
  mcl_periodic* mesh = nullptr;
  static void check(int rc) {
    if (rc != MCL_OK) throw std::runtime_error(std::string("mcleap periodic: ") + mcl_last_error());
  }
};
