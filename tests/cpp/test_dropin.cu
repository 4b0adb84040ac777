// C++ drop-in check: the reference's test drivers (tests/test_frnn.cu,
// tests/test_closest_neighbors.cu, tests/grid2d_frnn.cu in the reference),
// restated against include/mcleap/*.h and libmcl_gb300.so.  Prints one line per
// check and exits non-zero on any failure.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>
#include <set>
#include <vector>

#include "mcleap/Device_Triangulation.h"
#include "mcleap/gridCount2d.h"

static int g_fail = 0;
#define CHECK(cond, ...)                 \
  do {                                   \
    if (!(cond)) {                       \
      ++g_fail;                          \
      std::printf("FAIL: " __VA_ARGS__); \
      std::printf("\n");                 \
    }                                    \
  } while (0)

static float sqdist(glm::vec2 a, glm::vec2 b) {
  const float dx = a.x - b.x, dy = a.y - b.y;
  const float dx2 = dx * dx, dy2 = dy * dy;
  return dx2 + dy2;
}

static std::vector<glm::vec2> ref_points(int n, float bounds) {
  std::mt19937 rng{3};
  std::uniform_real_distribution<float> pos_r(-bounds, bounds);
  std::vector<glm::vec2> p;
  for (int i = 0; i < n; ++i) {
    const float x = pos_r(rng), y = pos_r(rng);
    p.push_back(glm::vec2(x, y));
  }
  return p;
}

// tests/test_frnn.cu: FRNN through oneRing + getFRNN, against brute force
static void test_frnn(float radius) {
  const int n = 1000, M = 20, F = 100;
  auto pts = ref_points(n, 1000.f);
  HostTriangulation* ht = new HostTriangulation();
  ht->addDelaunayPoints(pts);
  DeviceTriangulation dt(ht);
  const int V = (int)ht->m_pos.size();
  int *d_ring, *d_nb;
  cudaMalloc(&d_ring, sizeof(int) * V * M);
  cudaMalloc(&d_nb, sizeof(int) * V * F);
  dt.oneRing<M>(d_ring);
  dt.getFRNN<M, F>(radius, d_ring, d_nb);
  std::vector<int> nb((size_t)V * F);
  cudaMemcpy(nb.data(), d_nb, sizeof(int) * V * F, cudaMemcpyDeviceToHost);
  const float rr = radius * radius;
  int bad = 0;
  for (int i = 0; i < V; ++i) {
    std::vector<int> want;
    for (int j = 0; j < V; ++j)
      if (j != i && sqdist(ht->m_pos[i], ht->m_pos[j]) <= rr) want.push_back(j);
    std::vector<int> got;
    for (int k = 0; k < nb[i]; ++k) got.push_back(nb[(size_t)(k + 1) * V + i]);
    std::sort(got.begin(), got.end());
    if (got != want) ++bad;
  }
  CHECK(bad == 0, "frnn r=%g: %d vertices differ", radius, bad);
  std::printf("frnn r=%g vertices=%d mismatching=%d\n", radius, V, bad);
  cudaFree(d_ring);
  cudaFree(d_nb);
  delete ht;
}

// tests/test_closest_neighbors.cu
static void test_closest(int n) {
  const int M = 100;
  auto pts = ref_points(n, 1000.f);
  HostTriangulation ht;
  ht.addDelaunayPoints(pts);
  DeviceTriangulation dt(&ht);
  const int V = (int)ht.m_pos.size();
  int *d_ring, *d_cl;
  cudaMalloc(&d_ring, sizeof(int) * V * M);
  cudaMalloc(&d_cl, sizeof(int) * V);
  dt.oneRing<M>(d_ring);
  dt.closestNeighbors<M>(d_ring, d_cl);
  std::vector<int> cl(V);
  cudaMemcpy(cl.data(), d_cl, sizeof(int) * V, cudaMemcpyDeviceToHost);
  int bad = 0;
  for (int i = 0; i < V; ++i) {
    int best = i == 0 ? 1 : 0;
    float bd = sqdist(ht.m_pos[i], ht.m_pos[best]);
    for (int j = 0; j < V; ++j) {
      if (j == i) continue;
      const float d = sqdist(ht.m_pos[i], ht.m_pos[j]);
      if (d < bd) { bd = d; best = j; }
    }
    if (cl[i] != best) ++bad;
  }
  CHECK(bad == 0, "closest n=%d: %d differ", n, bad);
  std::printf("closest n=%d mismatching=%d\n", n, bad);
  cudaFree(d_ring);
  cudaFree(d_cl);
}

// tests/grid2d_frnn.cu SaveNeighborsFunctor
struct SaveNeighborsFunctor {
  float rad;
  int max_nb;
  int* num;
  int* ids;
  __device__ void operator()(const int& i, const int& j, const glm::vec2 d, const double dist) {
    if (i != j && dist <= rad) {
      const int k = num[i]++;
      if (k < max_nb) ids[i * max_nb + k] = j;
    }
  }
};

static void test_grid_lattice(int side, float step, float rad) {
  const int n = side * side, max_nb = 40;
  std::vector<glm::vec2> pos(n);
  for (int x = 0; x < side; ++x)
    for (int y = 0; y < side; ++y) pos[x + side * y] = glm::vec2(x * step, y * step);
  glm::vec2* d_pos;
  cudaMalloc(&d_pos, sizeof(glm::vec2) * n);
  cudaMemcpy(d_pos, pos.data(), sizeof(glm::vec2) * n, cudaMemcpyHostToDevice);
  GridCount2d gc(n, glm::vec2(0.f), glm::vec2(1.f), glm::ivec2(10));
  gc.update(d_pos);
  SaveNeighborsFunctor f{rad, max_nb, nullptr, nullptr};
  cudaMalloc(&f.num, sizeof(int) * n);
  cudaMalloc(&f.ids, sizeof(int) * n * max_nb);
  cudaMemset(f.num, 0, sizeof(int) * n);
  gc.apply_f_frnn<SaveNeighborsFunctor>(f, d_pos, rad);
  cudaDeviceSynchronize();
  std::vector<int> num(n);
  cudaMemcpy(num.data(), f.num, sizeof(int) * n, cudaMemcpyDeviceToHost);
  cudaMemcpy(pos.data(), d_pos, sizeof(glm::vec2) * n, cudaMemcpyDeviceToHost);
  int bad = 0;
  for (int i = 0; i < n; ++i) {
    int want = 0;
    for (int j = 0; j < n; ++j)
      if (i != j && sqdist(pos[i], pos[j]) <= rad * rad) ++want;
    if (num[i] != want) ++bad;
  }
  CHECK(bad == 0, "grid lattice %d x %d step %g: %d differ", side, side, step, bad);
  std::printf("grid lattice %dx%d step=%g mismatching=%d\n", side, side, step, bad);
  cudaFree(d_pos);
  cudaFree(f.num);
  cudaFree(f.ids);
}

// A few kinetic steps through movePoints + untangle2 + delonize2: every face
// must stay positively oriented (checked in double on the host).
static void test_kinetic() {
  const int n = 5000;
  std::mt19937 rng{7};
  std::uniform_real_distribution<float> u(0.f, 8192.f);
  std::normal_distribution<float> g(0.f, 0.3f * 8192.f / 70.7f);
  std::vector<glm::vec2> pts(n);
  for (auto& p : pts) p = glm::vec2(u(rng), u(rng));
  HostTriangulation ht;
  ht.addDelaunayPoints(pts);
  DeviceTriangulation dt(&ht);
  const int V = (int)ht.m_pos.size();
  glm::vec2* d_move;
  cudaMalloc(&d_move, sizeof(glm::vec2) * V);
  for (int step = 0; step < 3; ++step) {
    std::vector<glm::vec2> mv(V, glm::vec2(0.f));
    dt.transferToHost();
    for (int i = 4; i < V; ++i) {
      glm::vec2 t = ht.m_pos[i] + glm::vec2(g(rng), g(rng));
      t.x = std::min(std::max(t.x, 0.f), 8191.f);
      t.y = std::min(std::max(t.y, 0.f), 8191.f);
      mv[i] = t - ht.m_pos[i];
    }
    cudaMemcpy(d_move, mv.data(), sizeof(glm::vec2) * V, cudaMemcpyHostToDevice);
    CHECK(dt.movePoints(d_move), "movePoints");
    CHECK(dt.untangle2(), "untangle2: %s", mcl_last_error());
    CHECK(dt.delonize2(), "delonize2: %s", mcl_last_error());
    dt.transferToHost();
    int inverted = 0;
    for (size_t t = 0; t < ht.m_t.size(); ++t) {
      const HalfEdge& h = ht.m_he[ht.m_t[t].he];
      const glm::vec2 a = ht.m_pos[h.v], b = ht.m_pos[ht.m_he[ht.m_t[t].he ^ 1].v], c = ht.m_pos[h.op];
      const double o = ((double)b.x - a.x) * ((double)c.y - a.y) - ((double)b.y - a.y) * ((double)c.x - a.x);
      if (!(o > 0)) ++inverted;
    }
    CHECK(inverted == 0, "kinetic step %d: %d faces not positive", step, inverted);
    // the public device arrays hold the same records as the host download
    {
      std::vector<Vertex> dv(ht.m_v.size());
      std::vector<HalfEdge> dh(ht.m_he.size());
      std::vector<Triangle> dtr(ht.m_t.size());
      cudaMemcpy(dv.data(), dt.m_v, sizeof(Vertex) * dv.size(), cudaMemcpyDeviceToHost);
      cudaMemcpy(dh.data(), dt.m_he, sizeof(HalfEdge) * dh.size(), cudaMemcpyDeviceToHost);
      cudaMemcpy(dtr.data(), dt.m_t, sizeof(Triangle) * dtr.size(), cudaMemcpyDeviceToHost);
      int diff = 0;
      for (size_t i = 0; i < dv.size(); ++i) diff += dv[i].pos_index != ht.m_v[i].pos_index || dv[i].he != ht.m_v[i].he;
      for (size_t i = 0; i < dh.size(); ++i)
        diff += dh[i].next != ht.m_he[i].next || dh[i].v != ht.m_he[i].v || dh[i].t != ht.m_he[i].t ||
                dh[i].op != ht.m_he[i].op;
      for (size_t i = 0; i < dtr.size(); ++i) diff += dtr[i].he != ht.m_t[i].he;
      CHECK(diff == 0, "kinetic step %d: device m_v/m_he/m_t differ from the download in %d records", step, diff);
    }
    std::printf("kinetic step %d removed=%lld flips=%lld inverted_after=%d\n", step,
                (long long)dt.last_stats.removed_vertices, (long long)dt.last_stats.lawson_flips, inverted);
  }
  cudaFree(d_move);

  // Single-point moves (moveUntangling on the device mesh, moveFlipflopDelaunay
  // on the host one): the point lands where asked, across many triangles, and
  // every face stays positive; the bounding corners refuse to move.
  auto positive_faces = [&](const HostTriangulation& h) {
    int bad = 0;
    for (size_t t = 0; t < h.m_t.size(); ++t) {
      const HalfEdge& e = h.m_he[h.m_t[t].he];
      const glm::vec2 a = h.m_pos[e.v], b = h.m_pos[h.m_he[h.m_t[t].he ^ 1].v], c = h.m_pos[e.op];
      const double o = ((double)b.x - a.x) * ((double)c.y - a.y) - ((double)b.y - a.y) * ((double)c.x - a.x);
      if (!(o > 0)) ++bad;
    }
    return bad;
  };
  dt.transferToHost();
  const int p = 4 + n / 2;
  const glm::vec2 target(4096.5f, 4100.25f);
  const glm::vec2 dp = target - ht.m_pos[p];
  CHECK(!dt.moveUntangling(2, glm::vec2(1.f, 1.f)), "a bounding corner moved");
  CHECK(dt.moveUntangling(p, dp), "moveUntangling: %s", mcl_last_error());
  dt.transferToHost();
  CHECK(std::fabs(ht.m_pos[p].x - target.x) < 1e-2f && std::fabs(ht.m_pos[p].y - target.y) < 1e-2f,
        "moveUntangling put point %d at (%g, %g)", p, ht.m_pos[p].x, ht.m_pos[p].y);
  int bad = positive_faces(ht);
  CHECK(bad == 0, "moveUntangling: %d faces not positive", bad);
  const int q = 4 + n / 3;
  const glm::vec2 tq = glm::vec2(100.f, 8000.f);
  CHECK(ht.moveFlipflopDelaunay(q, tq - ht.m_pos[q]), "moveFlipflopDelaunay: %s", mcl_last_error());
  CHECK(std::fabs(ht.m_pos[q].x - tq.x) < 1e-2f && std::fabs(ht.m_pos[q].y - tq.y) < 1e-2f,
        "moveFlipflopDelaunay put point %d at (%g, %g)", q, ht.m_pos[q].x, ht.m_pos[q].y);
  bad = positive_faces(ht);
  CHECK(bad == 0, "moveFlipflopDelaunay: %d faces not positive", bad);
  std::printf("single-point moves ok\n");
}

int main() {
  for (float r : {5.f, 10.f, 20.f, 30.f, 40.f, 50.f}) test_frnn(r);
  for (int n : {10, 100, 1000}) test_closest(n);
  test_grid_lattice(10, 1.f, 1.f);
  test_grid_lattice(20, 0.5f, 1.f);
  test_grid_lattice(40, 0.25f, 0.25f);
  test_kinetic();
  std::printf(g_fail ? "FAILED %d\n" : "ALL PASSED\n", g_fail);
  return g_fail ? 1 : 0;
}
