// Drop-in DeviceTriangulation (reference: include/Device_Triangulation.h:128-223).
//
// Same member names, template parameters and buffer layouts as the reference;
// every call forwards to libmcl_gb300.so.  Differences a caller can observe:
//  - untangle()/untangle2() always return a valid triangulation (the reference
//    handles only its B/C cases) and, like delonize(), leave it Delaunay;
//  - m_pos is refreshed after every call that moves points (positions are
//    double-buffered on the device), so read the member, do not cache it;
//  - neighbour lists start at the smallest neighbour id (clockwise, as the
//    reference walks) and FRNN lists are sorted ascending;
//  - getFRNN ignores the ring table argument (the search walks the mesh);
//  - calls return false (and keep the error in mcl_last_error()) on failure;
//  - m_v, m_he, m_t are device copies of the mesh in the reference's records,
//    rewritten from the engine's own layout after every call that changes
//    the topology (construction, transferToDevice, untangle, delonize, step,
//    the single-point moves): read them, do not write them (a write is not
//    seen by the engine; change the host arrays and call transferToDevice).
#pragma once

#include <cuda_runtime.h>

#include "Host_Triangulation.h"

struct DeviceTriangulation {
  HostTriangulation* h_triangulation;
  int m_pos_size = 0, m_v_size = 0, m_he_size = 0, m_t_size = 0;
  glm::vec2* m_pos = nullptr;
  Vertex* m_v = nullptr;
  HalfEdge* m_he = nullptr;
  Triangle* m_t = nullptr;
  mcl_mesh* mesh = nullptr;
  mcl_step_stats last_stats{};

  explicit DeviceTriangulation(HostTriangulation* ht) : h_triangulation(ht) {
    allocateMemory();
  }
  ~DeviceTriangulation() { freeMemory(); }
  DeviceTriangulation(const DeviceTriangulation&) = delete;
  DeviceTriangulation& operator=(const DeviceTriangulation&) = delete;

  bool allocateMemory() {
    freeMemory();
    mcl_aos_view a = h_triangulation->view();
    mcleap_detail::check(mcl_mesh_create_from_aos(&a, &mesh));
    int64_t V = 0, HE = 0, T = 0;
    mcl_mesh_sizes(mesh, &V, &HE, &T);
    m_pos_size = m_v_size = (int)V;
    m_he_size = (int)HE;
    m_t_size = (int)T;
    const bool ok = cudaMalloc((void**)&m_v, sizeof(Vertex) * (size_t)V) == cudaSuccess &&
                    cudaMalloc((void**)&m_he, sizeof(HalfEdge) * (size_t)HE) == cudaSuccess &&
                    cudaMalloc((void**)&m_t, sizeof(Triangle) * (size_t)(T > 0 ? T : 1)) == cudaSuccess;
    if (!ok) mcleap_detail::check(MCL_ERR_OUT_OF_MEMORY);
    refresh();
    return export_aos();
  }
  bool freeMemory() {
    if (mesh) mcl_mesh_destroy(mesh);
    mesh = nullptr;
    m_pos = nullptr;
    cudaFree(m_v);
    cudaFree(m_he);
    cudaFree(m_t);
    m_v = nullptr;
    m_he = nullptr;
    m_t = nullptr;
    return true;
  }
  bool transferToHost() {
    h_triangulation->download(mesh);
    return true;
  }
  bool transferToDevice() {
    mcl_aos_view a = h_triangulation->view();
    const bool ok = mcl_mesh_upload_aos(mesh, &a) == MCL_OK;
    refresh();
    return ok && export_aos();
  }

  bool delonize() { return restore(); }
  bool delonize2() { return restore(); }
  bool untangle() { return restore(); }
  bool untangle2() { return restore(); }

  bool movePoints(glm::vec2* d) {
    const bool ok = mcl_move(mesh, reinterpret_cast<const mcl_float2*>(d), nullptr) == MCL_OK;
    refresh();
    return ok;
  }
  bool integrateMovePoints(float* dt, glm::vec2* v) {
    const bool ok = mcl_integrate(mesh, dt, reinterpret_cast<const mcl_float2*>(v), nullptr) == MCL_OK;
    refresh();
    return ok;
  }
  // include/Device_Triangulation.h:183-186 (bodies at :411-417 return false
  // in the reference): move point p_index by d and leave a valid mesh.  Here
  // every variant runs the kinetic step on a displacement with one nonzero
  // entry (through host memory), so the mesh is also Delaunay afterwards.
  bool moveFlipflop(int p_index, glm::vec2 d) { return move_one(p_index, d); }
  bool moveFlipflopDelaunay(int p_index, glm::vec2 d) { return move_one(p_index, d); }
  bool moveUntangling(int p_index, glm::vec2 d) { return move_one(p_index, d); }
  bool moveUntanglingDelaunay(int p_index, glm::vec2 d) { return move_one(p_index, d); }

  // movePoints + untangle + delonize in one launch (no counterpart in the reference).
  bool step(glm::vec2* d) {
    const bool ok = mcl_step(mesh, reinterpret_cast<const mcl_float2*>(d), nullptr, &last_stats) == MCL_OK;
    refresh();
    return ok && export_aos();
  }

  template <int maxRingSize>
  bool oneRing(int* ring_neighbors) {
    return mcl_one_ring(mesh, MCL_LAYOUT_COLUMN, maxRingSize, ring_neighbors, nullptr, nullptr) == MCL_OK;
  }
  template <int maxRingSize>
  bool oneRing2(int* ring_neighbors) {
    return mcl_one_ring(mesh, MCL_LAYOUT_ROW, maxRingSize, ring_neighbors, nullptr, nullptr) == MCL_OK;
  }
  template <int maxRingSize>
  bool closestNeighbors(int* ring_neighbors, int* closest_neighbors) {
    return mcl_closest_neighbors(mesh, MCL_LAYOUT_COLUMN, maxRingSize, ring_neighbors, closest_neighbors,
                                 nullptr) == MCL_OK;
  }
  template <int maxRingSize>
  bool closestNeighbors2(int* ring_neighbors, int* closest_neighbors) {
    return mcl_closest_neighbors(mesh, MCL_LAYOUT_ROW, maxRingSize, ring_neighbors, closest_neighbors,
                                 nullptr) == MCL_OK;
  }
  template <int maxRingSize, int maxFRNNSize>
  bool getFRNN(float r, int* /*ring_neighbors*/, int* neighbors) {
    return mcl_mesh_frnn(mesh, r, MCL_LAYOUT_COLUMN, maxFRNNSize, neighbors, nullptr, nullptr) == MCL_OK;
  }
  template <int maxRingSize, int maxFRNNSize>
  bool getFRNN2(float r, int* /*ring_neighbors*/, int* neighbors) {
    return mcl_mesh_frnn(mesh, r, MCL_LAYOUT_ROW, maxFRNNSize, neighbors, nullptr, nullptr) == MCL_OK;
  }

 private:
  std::vector<glm::vec2> one_;  // host displacement of a single-point move
  bool move_one(int p, glm::vec2 d) {
    if (p < 4 || p >= m_pos_size) return false;  // the bounding corners stay
    one_.assign((size_t)m_pos_size, glm::vec2(0.f, 0.f));
    one_[(size_t)p] = d;
    const bool ok =
        mcl_step_host(mesh, reinterpret_cast<const mcl_float2*>(one_.data()), nullptr, &last_stats) == MCL_OK;
    refresh();
    return ok && export_aos();
  }
  // m_v / m_he / m_t from the engine's layout (default stream)
  bool export_aos() {
    return mcl_mesh_export_aos(mesh, reinterpret_cast<int32_t*>(m_v), reinterpret_cast<int32_t*>(m_he),
                               reinterpret_cast<int32_t*>(m_t), nullptr) == MCL_OK;
  }
  void refresh() {
    mcl_float2* p = nullptr;
    mcl_mesh_positions(mesh, &p);
    m_pos = reinterpret_cast<glm::vec2*>(p);
  }
  bool restore() {
    const bool ok = mcl_delaunay_restore(mesh, nullptr, &last_stats) == MCL_OK;
    refresh();
    return ok && export_aos();
  }
};
