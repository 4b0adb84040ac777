// Mesh records of the reference's interchange layout
// (include/Common_Triangulation.h:42-57 in the reference): these layouts have to
// be alike because meshes cross the boundary in exactly this form.
#pragma once

#include "mcl_glm.h"

constexpr float cood_min = -10000000;
constexpr float cood_max = 10000000;

struct Vertex {
  int pos_index;  // = vertex id
  int he;         // one outgoing half-edge
};

struct HalfEdge {
  int next;  // next half-edge of the face (twin of half-edge i is i^1)
  int v;     // origin vertex
  int t;     // face, -1 outside the bounding square
  int op;    // vertex opposite the half-edge in its face
};

struct Triangle {
  int he;  // one half-edge of the face
};

static_assert(sizeof(Vertex) == 8 && sizeof(HalfEdge) == 16 && sizeof(Triangle) == 4, "interchange layout");
