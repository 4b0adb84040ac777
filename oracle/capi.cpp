// Oracle C entry points for the Python tests (ctypes).  Test infrastructure
// only: the shipped engine never links this library.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "exact.h"
#include "mesh.h"

using namespace oracle;

extern "C" {

int orc_version() { return 1; }

// ---- predicates -----------------------------------------------------------
// pts: n records of 6 floats (ax ay bx by cx cy); mode 0 = reference FP64,
// 1 = exact.
void orc_orient2d_batch(const float* pts, long n, int mode, int* out) {
  for (long i = 0; i < n; ++i) {
    const float* q = pts + 6 * i;
    P2 a{q[0], q[1]}, b{q[2], q[3]}, c{q[4], q[5]};
    out[i] = mode ? orient2d_exact(a, b, c) : orient2d_ref(a, b, c);
  }
}

// pts: n records of 8 floats; ids: n records of 4 ints (used by mode 2 = SoS).
void orc_incircle_batch(const float* pts, const int* ids, long n, int mode, int* out) {
  for (long i = 0; i < n; ++i) {
    const float* q = pts + 8 * i;
    P2 a{q[0], q[1]}, b{q[2], q[3]}, c{q[4], q[5]}, d{q[6], q[7]};
    if (mode == 0) out[i] = incircle_ref(a, b, c, d);
    else if (mode == 1) out[i] = incircle_exact(a, b, c, d);
    else {
      const int* k = ids + 4 * i;
      out[i] = incircle_sos(a, b, c, d, k[0], k[1], k[2], k[3]);
    }
  }
}

void orc_exact_stats(unsigned long long* out5) {
  ExactStats s = exact_stats();
  out5[0] = s.orient_calls; out5[1] = s.orient_exact; out5[2] = s.incircle_calls;
  out5[3] = s.incircle_exact; out5[4] = s.sos_used;
}
void orc_exact_stats_reset() { exact_stats_reset(); }

// ---- Morton order ---------------------------------------------------------
void orc_morton_sort(float* xy, long n) {
  std::vector<P2> p((size_t)n);
  std::memcpy(p.data(), xy, sizeof(float) * 2 * n);
  morton_sort(p);
  std::memcpy(xy, p.data(), sizeof(float) * 2 * n);
}
unsigned long long orc_morton_key(float x, float y) { return morton_key(x, y); }

// ---- meshes -----------------------------------------------------------------
// Build by inserting xy[0..n) in the given order (vertex id = 4 + index).
// mode 0 = reference algorithm with FP64 predicates (include/Host_Triangulation.h),
// mode 1 = exact predicates with symbolic perturbation (the oracle DT).
void* orc_mesh_build(const float* xy, long n, int mode) {
  Mesh* m = new Mesh();
  m->mode = mode ? PRED_EXACT : PRED_REF;
  m->pos.reserve(n + 4); m->v.reserve(n + 4); m->he.reserve(6 * n + 10); m->t.reserve(2 * n + 2);
  for (long i = 0; i < n; ++i) {
    P2 p{xy[2 * i], xy[2 * i + 1]};
    bool ok = mode ? m->add_delaunay_point_exact(p) : m->add_delaunay_point_ref(p);
    if (!ok) break;
  }
  return m;
}

void* orc_mesh_import(const float* pos, long V, const int* vv, const int* he, long HEn,
                      const int* tt, long T, int mode) {
  Mesh* m = new Mesh();
  m->mode = mode ? PRED_EXACT : PRED_REF;
  m->pos.assign((const P2*)pos, (const P2*)pos + V);
  m->v.assign((const Vtx*)vv, (const Vtx*)vv + V);
  m->he.assign((const HE*)he, (const HE*)he + HEn);
  m->t.assign((const Tri*)tt, (const Tri*)tt + T);
  return m;
}

void orc_mesh_free(void* h) { delete (Mesh*)h; }
void orc_mesh_set_mode(void* h, int mode) { ((Mesh*)h)->mode = mode ? PRED_EXACT : PRED_REF; }

// out: V, HE, T, error, flips
void orc_mesh_counts(void* h, long long* out) {
  Mesh* m = (Mesh*)h;
  out[0] = (long long)m->v.size(); out[1] = (long long)m->he.size();
  out[2] = (long long)m->t.size(); out[3] = m->error; out[4] = m->flips;
}

void orc_mesh_export(void* h, float* pos, int* vv, int* he, int* tt) {
  Mesh* m = (Mesh*)h;
  if (pos) std::memcpy(pos, m->pos.data(), sizeof(P2) * m->pos.size());
  if (vv) std::memcpy(vv, m->v.data(), sizeof(Vtx) * m->v.size());
  if (he) std::memcpy(he, m->he.data(), sizeof(HE) * m->he.size());
  if (tt) std::memcpy(tt, m->t.data(), sizeof(Tri) * m->t.size());
}

void orc_mesh_set_positions(void* h, const float* pos) {
  Mesh* m = (Mesh*)h;
  std::memcpy(m->pos.data(), pos, sizeof(P2) * m->pos.size());
}

// movePoint for every vertex id >= 4 (include/Host_Triangulation.h:403-406;
// the four corners stay fixed as in include/kernels.cuh:38-43).
void orc_mesh_move(void* h, const float* d) {
  Mesh* m = (Mesh*)h;
  for (size_t i = 4; i < m->pos.size(); ++i) {
    m->pos[i].x += d[2 * i];
    m->pos[i].y += d[2 * i + 1];
  }
}

// Sorted undirected edge list, 2 ints per edge; returns the edge count.
long orc_mesh_edges(void* h, int* out) {
  auto e = edge_set(*(Mesh*)h);
  if (out)
    for (size_t i = 0; i < e.size(); ++i) { out[2 * i] = e[i].first; out[2 * i + 1] = e[i].second; }
  return (long)e.size();
}

// non_delaunay, creased, inverted_faces, zero_faces
void orc_mesh_check(void* h, int exact, int* out) {
  MeshCheck c = check_mesh(*(Mesh*)h, exact != 0);
  out[0] = c.non_delaunay; out[1] = c.creased; out[2] = c.inverted_faces; out[3] = c.zero_faces;
}

// ---- the reference's CPU kinetic path ---------------------------------------
int orc_ref_untangle_pass(void* h) { return ((Mesh*)h)->untangle_pass() ? 1 : 0; }
int orc_ref_delonize(void* h) { return ((Mesh*)h)->delonize_restart_scan() ? 1 : 0; }

// One kinetic step as the reference composes it: movePoint for every point,
// untangle() until it stops flipping (capped), then delonize().
// out: untangle_passes, untangle_flips, delonize_flips, seconds*1e6
void orc_ref_kinetic_step(void* h, const float* d, long long* out) {
  Mesh* m = (Mesh*)h;
  auto t0 = std::chrono::steady_clock::now();
  orc_mesh_move(h, d);
  long long f0 = m->flips;
  int passes = 0;
  while (passes < 64 && m->untangle_pass()) ++passes;
  long long f1 = m->flips;
  // cap the Lawson loop at 64 flips per edge: the reference never stops on a
  // mesh its untangling left tangled
  m->capped = false;
  m->delonize_restart_scan(64ll * (long long)(m->he.size() / 2));
  long long f2 = m->flips;
  auto t1 = std::chrono::steady_clock::now();
  out[0] = passes; out[1] = f1 - f0; out[2] = f2 - f1;
  out[3] = (long long)std::chrono::duration<double, std::micro>(t1 - t0).count();
  out[4] = m->capped ? 1 : 0;
}

long orc_ref_one_ring(void* h, int vi, int* out, long cap) {
  auto r = ((Mesh*)h)->one_ring_ref(vi);
  for (size_t i = 0; i < r.size() && (long)i < cap; ++i) out[i] = r[i];
  return (long)r.size();
}

long orc_ref_frnn(void* h, int vi, float r, int* out, long cap) {
  auto nb = ((Mesh*)h)->frnn_ref(vi, r);
  for (size_t i = 0; i < nb.size() && (long)i < cap; ++i) out[i] = nb[i];
  return (long)nb.size();
}

// Reference getFRNN for every vertex into CSR (sorted per vertex); returns
// total count (writes ids only while total <= cap).
long orc_ref_frnn_all(void* h, float r, int* counts, int* ids, long cap) {
  Mesh* m = (Mesh*)h;
  long total = 0;
  for (size_t i = 0; i < m->pos.size(); ++i) {
    auto nb = m->frnn_ref((int)i, r);
    std::sort(nb.begin(), nb.end());
    counts[i] = (int)nb.size();
    for (int x : nb) { if (total < cap) ids[total] = x; ++total; }
  }
  return total;
}

// ---- brute-force fixed-radius neighbours -------------------------------------
// Membership {j != i : fl(fl(dx*dx) + fl(dy*dy)) <= fl(r*r)} with dx = p_i - p_j
// in float (the reference's sqrtDist, include/kernels.cuh:125-127, and
// getFRNN's dot, include/Host_Triangulation.h:550).  periodic != 0 applies the
// minimum image on a torus of side L: dx > L/2 -> dx - L, dx < -L/2 -> dx + L.
// Neighbours sorted ascending per point; CSR output; returns the total.
// A bucket grid (cells >= r) only prunes candidates; every candidate is tested
// with the formula above.  Points with a coordinate of magnitude >= 1e6 (the
// bounding-square corners) are tested against everything.
long orc_frnn_brute(const float* xy, long n, float r, int periodic, float L, int* counts,
                    int* ids, long cap) {
  const float r2 = r * r;
  const float half = 0.5f * L;
  std::vector<char> is_far((size_t)n, 0);
  std::vector<long> far;
  double minx = 1e300, maxx = -1e300, miny = 1e300, maxy = -1e300;
  for (long i = 0; i < n; ++i) {
    const float x = xy[2 * i], y = xy[2 * i + 1];
    if (std::fabs(x) >= 1e6f || std::fabs(y) >= 1e6f) { is_far[i] = 1; far.push_back(i); continue; }
    minx = std::min(minx, (double)x); maxx = std::max(maxx, (double)x);
    miny = std::min(miny, (double)y); maxy = std::max(maxy, (double)y);
  }
  if (periodic) { minx = 0; miny = 0; maxx = L; maxy = L; }
  if (minx > maxx) { minx = maxx = miny = maxy = 0; }
  const double cell = std::max((double)r, 1e-20);
  long nx = std::max(1L, std::min(8192L, (long)std::floor((maxx - minx) / cell)));
  long ny = std::max(1L, std::min(8192L, (long)std::floor((maxy - miny) / cell)));
  const double cx = std::max((maxx - minx) / nx, cell), cy = std::max((maxy - miny) / ny, cell);
  nx = std::max(1L, (long)std::floor((maxx - minx) / cx));
  ny = std::max(1L, (long)std::floor((maxy - miny) / cy));
  std::vector<std::vector<long>> cells((size_t)(nx * ny));
  auto cell_of = [&](float x, float y, long& ix, long& iy) {
    ix = (long)std::floor((x - minx) / cx); iy = (long)std::floor((y - miny) / cy);
    ix = std::min(std::max(ix, 0L), nx - 1); iy = std::min(std::max(iy, 0L), ny - 1);
  };
  for (long i = 0; i < n; ++i) {
    if (is_far[i]) continue;
    long ix, iy; cell_of(xy[2 * i], xy[2 * i + 1], ix, iy);
    cells[(size_t)(iy * nx + ix)].push_back(i);
  }
  long total = 0;
  std::vector<int> nb;
  for (long i = 0; i < n; ++i) {
    nb.clear();
    const float px = xy[2 * i], py = xy[2 * i + 1];
    auto test = [&](long j) {
      if (j == i) return;
      float dx = px - xy[2 * j], dy = py - xy[2 * j + 1];
      if (periodic) {
        if (dx > half) dx = dx - L; else if (dx < -half) dx = dx + L;
        if (dy > half) dy = dy - L; else if (dy < -half) dy = dy + L;
      }
      const float dx2 = dx * dx, dy2 = dy * dy;
      if (dx2 + dy2 <= r2) nb.push_back((int)j);
    };
    if (is_far[i] || nx < 3 || ny < 3) {
      for (long j = 0; j < n; ++j) test(j);
    } else {
      long ix, iy; cell_of(px, py, ix, iy);
      for (long oy = -1; oy <= 1; ++oy)
        for (long ox = -1; ox <= 1; ++ox) {
          long jx = ix + ox, jy = iy + oy;
          if (periodic) { jx = (jx + nx) % nx; jy = (jy + ny) % ny; }
          if (jx < 0 || jy < 0 || jx >= nx || jy >= ny) continue;
          for (long j : cells[(size_t)(jy * nx + jx)]) test(j);
        }
      for (long j : far) test(j);
    }
    std::sort(nb.begin(), nb.end());
    nb.erase(std::unique(nb.begin(), nb.end()), nb.end());
    counts[i] = (int)nb.size();
    for (int x : nb) { if (total < cap) ids[total] = x; ++total; }
  }
  return total;
}

}  // extern "C"
