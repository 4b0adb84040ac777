// Oracle half-edge mesh (test infrastructure only).
//
// The interchange format is the reference's AoS layout, which has to be alike
// because callers exchange meshes through it
// (include/Common_Triangulation.h:42-57):
//   Vertex   {pos_index, he}          he  = one outgoing half-edge
//   HalfEdge {next, v, t, op}          v   = origin, t = face (-1 outside),
//                                      op  = vertex opposite in face t,
//                                      twin of half-edge i is i^1
//   Triangle {he}                      one half-edge of the face
// Vertex ids 0..3 are the corners of the +-1e7 bounding square
// (include/Common_Triangulation.h:12-13, include/Host_Triangulation.h:107-137).
#pragma once
#include <cstdint>
#include <vector>

#include "exact.h"

namespace oracle {

struct Vtx { int pos_index, he; };
struct HE { int next, v, t, op; };
struct Tri { int he; };

enum PredMode { PRED_REF = 0, PRED_EXACT = 1 };

struct Mesh {
  std::vector<P2> pos;
  std::vector<Vtx> v;
  std::vector<HE> he;
  std::vector<Tri> t;
  int mode = PRED_EXACT;
  int64_t flips = 0;       // f2to2 calls
  int error = 0;           // 0 ok; see OERR_* below

  Mesh();  // bounding square seed

  int orient(const P2& a, const P2& b, const P2& c) const;
  // incircle of the quad tested by the reference's delonizeEdge
  int incircle_q(int v0, int v1, int v2, int v3) const;

  void f2to2(int he_index);
  void f1to3(int t_index, int v_new, int t_a, int t_b, int he_a, int he_b, int he_c);
  void f2to4(int he_index, int v_new);

  // reference algorithm pieces (citations in mesh.cpp)
  int walk_centroid(P2 p, int t_guess) const;
  bool add_delaunay_point_ref(P2 p);
  bool delonize_edge(int he_index);
  void delonize_vertex(int v_index);
  bool delonize_restart_scan(long long max_flips = -1);
  bool capped = false;  // the last capped restart-scan stopped at its cap
  bool untangle_pass();
  bool untangle_edge(int he_index);
  bool is_ccw_face(int t_index) const;
  bool is_inside_face(const P2& p, int t_index, bool inverted) const;
  bool is_creased(int he_index) const;
  std::vector<int> one_ring_ref(int v_index) const;
  std::vector<int> frnn_ref(int v_index, float r) const;

  // exact builder pieces
  int locate_exact(P2 p, int t_guess, int* on_he) const;
  bool add_delaunay_point_exact(P2 p);
};

enum {
  OERR_OK = 0,
  OERR_WALK_CAP = 1,       // point location did not terminate within the cap
  OERR_DUPLICATE = 2,      // point coincides with an existing vertex
  OERR_OUTSIDE = 3,        // point outside the bounding square
  OERR_DELONIZE_CAP = 4,   // Lawson flips did not converge within the cap
};

// Morton order used by HostTriangulation::addDelaunayPoints
// (include/Host_Triangulation.h:287-300): std::sort on a 2-D bit interleave of
// the coordinates truncated to integers (x in the even bits).
uint64_t morton_key(float x, float y);
void morton_sort(std::vector<P2>& pts);

// Sorted undirected edge list (u < v) of the mesh.
std::vector<std::pair<int, int>> edge_set(const Mesh& m);
// Counts used by the reference experiments' self-validation
// (experiments/moving_device_mesh.cu:212-242).
struct MeshCheck { int non_delaunay, creased, inverted_faces, zero_faces; };
MeshCheck check_mesh(const Mesh& m, bool exact);

}  // namespace oracle
