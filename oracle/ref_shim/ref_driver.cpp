// C entry points around the reference's own HostTriangulation and Shewchuk's
// predicates.c, compiled from the reference sources where they lie (the
// Makefile's `ref` target).  Used only to pin the oracle restatement and to
// generate the golden fixtures under tests/golden/.
#include <cstdlib>
#include <math.h>
#include <cmath>
#include <cstdint>
#include <limits>
#include <algorithm>
#include <vector>
#include <cstring>

#include "Host_Triangulation.h"
#include "predicates.h"
#include <random>

extern "C" {

// The reference tests' input generator (tests/test_frnn.cu:21-28,
// tests/test_closest_neighbors.cu:21-28): std::mt19937 seeded with `seed`,
// uniform_real_distribution<float>(-bounds, bounds), x then y per point.
void ref_gen_points(unsigned seed, long n, float bounds, float* out) {
  std::mt19937 rng{seed};
  std::uniform_real_distribution<float> pos_r(-bounds, bounds);
  for (long i = 0; i < n; ++i) { out[2 * i] = pos_r(rng); out[2 * i + 1] = pos_r(rng); }
}

void* ref_build(float* xy, long n) {
  std::vector<glm::vec2> pts;
  pts.reserve(n);
  for (long i = 0; i < n; ++i) pts.push_back(glm::vec2(xy[2 * i], xy[2 * i + 1]));
  HostTriangulation* ht = new HostTriangulation();
  ht->addDelaunayPoints(pts);  // sorts pts in place (Morton order)
  for (long i = 0; i < n; ++i) { xy[2 * i] = pts[i].x; xy[2 * i + 1] = pts[i].y; }
  return ht;
}

void ref_free(void* h) { delete (HostTriangulation*)h; }

void ref_counts(void* h, long long* out) {
  HostTriangulation* ht = (HostTriangulation*)h;
  out[0] = ht->m_v.size(); out[1] = ht->m_he.size(); out[2] = ht->m_t.size();
}

void ref_export(void* h, float* pos, int* v, int* he, int* t) {
  HostTriangulation* ht = (HostTriangulation*)h;
  std::memcpy(pos, ht->m_pos.data(), 8 * ht->m_pos.size());
  std::memcpy(v, ht->m_v.data(), 8 * ht->m_v.size());
  std::memcpy(he, ht->m_he.data(), 16 * ht->m_he.size());
  std::memcpy(t, ht->m_t.data(), 4 * ht->m_t.size());
}

void ref_move_all(void* h, const float* d) {
  HostTriangulation* ht = (HostTriangulation*)h;
  for (size_t i = 4; i < ht->m_pos.size(); ++i) ht->movePoint((int)i, glm::vec2(d[2 * i], d[2 * i + 1]));
}

int ref_untangle(void* h) { return ((HostTriangulation*)h)->untangle() ? 1 : 0; }
int ref_delonize(void* h) { return ((HostTriangulation*)h)->delonize() ? 1 : 0; }

long ref_one_ring(void* h, int v, int* out, long cap) {
  auto r = ((HostTriangulation*)h)->oneRing(v);
  for (size_t i = 0; i < r.size() && (long)i < cap; ++i) out[i] = r[i];
  return (long)r.size();
}

long ref_frnn(void* h, int v, float rad, int* out, long cap) {
  auto r = ((HostTriangulation*)h)->getFRNN(v, rad);
  for (size_t i = 0; i < r.size() && (long)i < cap; ++i) out[i] = r[i];
  return (long)r.size();
}

// Reference FP64 predicates (include/Helpers_Triangulation.h) on n records.
void ref_helpers_orient(const float* p, long n, int* out) {
  for (long i = 0; i < n; ++i) {
    const float* q = p + 6 * i;
    out[i] = orient2d(glm::vec2(q[0], q[1]), glm::vec2(q[2], q[3]), glm::vec2(q[4], q[5]));
  }
}
void ref_helpers_incircle(const float* p, long n, int* out) {
  for (long i = 0; i < n; ++i) {
    const float* q = p + 8 * i;
    out[i] = inCircle(glm::vec2(q[0], q[1]), glm::vec2(q[2], q[3]), glm::vec2(q[4], q[5]),
                      glm::vec2(q[6], q[7]));
  }
}

// Shewchuk's adaptive exact predicates (experiments/predicates.c) on n records.
void ref_shewchuk_orient(const float* p, long n, int* out) {
  static bool init = false;
  if (!init) { exactinit(); init = true; }
  for (long i = 0; i < n; ++i) {
    const float* q = p + 6 * i;
    double a[2] = {q[0], q[1]}, b[2] = {q[2], q[3]}, c[2] = {q[4], q[5]};
    double r = orient2d(a, b, c);
    out[i] = r > 0 ? 1 : (r < 0 ? -1 : 0);
  }
}
void ref_shewchuk_incircle(const float* p, long n, int* out) {
  static bool init = false;
  if (!init) { exactinit(); init = true; }
  for (long i = 0; i < n; ++i) {
    const float* q = p + 8 * i;
    double a[2] = {q[0], q[1]}, b[2] = {q[2], q[3]}, c[2] = {q[4], q[5]}, d[2] = {q[6], q[7]};
    double r = incircle(a, b, c, d);
    out[i] = r > 0 ? 1 : (r < 0 ? -1 : 0);
  }
}

}  // extern "C"
