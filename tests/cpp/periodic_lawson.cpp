// Sequential Lawson flips on a periodic (flat torus) mesh, on the CPU, with the
// engine's own periodic offset helpers (mcleap_gb300/csrc/periodic.cuh) and
// predicate ladder (predicates.cuh).  Test harness: reads a mesh and moved
// positions, wraps the positions into the domain and the vertices' wraps into
// the edge words, flips until every edge is locally Delaunay, writes the mesh.
//
//   periodic_lawson IN OUT
//   IN : int32 n, int32 E, float L, float pos[n][2] (old canonical + move),
//        int32 ev[E][4], int32 en[E][4], uint32 eo[E]
//   OUT: int32 status, int32 flips, int32 wrapped, int32 nonpositive_before,
//        int32 nonpositive_after, float pos[n][2], int32 ev[E][4], int32 en[E][4],
//        uint32 eo[E]
// status: 0 ok, 1 an offset outside -1..+1, 2 a predicate overflow, 3 I/O.
#include <cstdint>
#include <cstdio>
#include <vector>

#include "periodic.cuh"

namespace {

struct P2f {
  float x, y;
};
struct NoCount {
  int incircle_fp64, incircle_exact, orient_fp64, orient_exact, sos;
};
struct I4 {
  int x, y, z, w;
};

int n, E;
float L;
std::vector<P2f> pos;
std::vector<I4> ev, en;
std::vector<uint32_t> eo;
int overflow = 0;

int orient(P2f a, P2f b, P2f c) {
  return mcl::orient2d(a.x, a.y, b.x, b.y, c.x, c.y, (NoCount*)nullptr, &overflow);
}

// face of half-edge h in its origin's frame
int face_sign(int h) {
  const int e = h >> 1, s = h & 1;
  const I4 q = ev[e];
  const int o = s ? q.y : q.x, t = s ? q.x : q.y, x = s ? q.w : q.z;
  const P2f pt = mcl::off_translate(pos[t], mcl::eo_target(eo[e], s), L);
  const P2f px = mcl::off_translate(pos[x], mcl::eo_apex(eo[e], s), L);
  return orient(pos[o], pt, px);
}

void set_face(int h, int apex, int next, int prev) {
  I4& q = ev[h >> 1];
  I4& w = en[h >> 1];
  if (h & 1) { q.w = apex; w.z = next; w.w = prev; }
  else { q.z = apex; w.x = next; w.y = prev; }
}

void set_apex_byte(int h, unsigned b) {
  const int sh = 8 * (1 + (h & 1));
  eo[h >> 1] = (eo[h >> 1] & ~(0xFFu << sh)) | (b << sh);
}

// the planar engine's flip of edge e, plus the periodic offsets
void flip(int e) {
  const I4 q = ev[e], w = en[e];
  const int a = q.x, b = q.y, c = q.z, d = q.w;
  const int n0 = w.x, p0 = w.y, n1 = w.z, p1 = w.w;
  const int h0 = 2 * e, h1 = 2 * e + 1;
  const mcl::FlipOffsets f = mcl::flip_offsets(eo[e]);
  ev[e] = I4{d, c, a, b};
  en[e] = I4{p0, n1, p1, n0};
  eo[e] = f.eo;
  set_face(p0, d, n1, h0);
  set_face(n1, c, h0, p0);
  set_face(p1, c, n0, h1);
  set_face(n0, d, h1, p1);
  set_apex_byte(p0, f.p0);
  set_apex_byte(n1, f.n1);
  set_apex_byte(p1, f.p1);
  set_apex_byte(n0, f.n0);
}

template <typename T>
bool rd(FILE* f, T* p, size_t k) { return fread(p, sizeof(T), k, f) == k; }
template <typename T>
void wr(FILE* f, const T* p, size_t k) { fwrite(p, sizeof(T), k, f); }

}  // namespace

int main(int argc, char** argv) {
  if (argc != 3) return 3;
  FILE* in = fopen(argv[1], "rb");
  if (!in || !rd(in, &n, 1) || !rd(in, &E, 1) || !rd(in, &L, 1)) return 3;
  pos.resize(n);
  ev.resize(E);
  en.resize(E);
  eo.resize(E);
  if (!rd(in, pos.data(), n) || !rd(in, ev.data(), E) || !rd(in, en.data(), E) || !rd(in, eo.data(), E)) return 3;
  fclose(in);

  // wrap positions, then the wraps into the edge words (any order)
  const float lo = 2.0f * L;
  std::vector<mcl::Off> wv(n);
  int wrapped = 0;
  for (int v = 0; v < n; ++v) {
    wv[v] = mcl::wrap_position(pos[v], lo, L);
    wrapped += !mcl::off_zero(wv[v]);
  }
  for (int e = 0; e < E; ++e) {
    const int role_v[4] = {ev[e].x, ev[e].y, ev[e].z, ev[e].w};
    for (int r = 0; r < 4; ++r)
      if (!mcl::off_zero(wv[role_v[r]])) eo[e] += (uint32_t)mcl::eo_wrap_delta(r, wv[role_v[r]]);
  }

  int status = 0, before = 0, after = 0, flips = 0;
  for (int h = 0; h < 2 * E; ++h) before += face_sign(h) <= 0;

  std::vector<int> stack;
  std::vector<char> queued(E, 1);
  for (int e = E - 1; e >= 0; --e) stack.push_back(e);
  while (!stack.empty() && status == 0) {
    const int e = stack.back();
    stack.pop_back();
    queued[e] = 0;
    const I4 q = ev[e];
    P2f qb, qc, qd;
    if (!mcl::quad_frame(eo[e], pos[q.y], pos[q.z], pos[q.w], L, qb, qc, qd)) {
      status = 1;
      break;
    }
    const P2f pa = pos[q.x];
    if (orient(pa, qb, qc) <= 0 || orient(qb, pa, qd) <= 0) continue;
    if (mcl::incircle_sos(pa.x, pa.y, qb.x, qb.y, qc.x, qc.y, qd.x, qd.y, q.x, q.y, q.z, q.w, (NoCount*)nullptr,
                          &overflow) <= 0)
      continue;
    const I4 w = en[e];
    flip(e);
    ++flips;
    for (int h : {w.x, w.y, w.z, w.w})
      if (!queued[h >> 1]) {
        queued[h >> 1] = 1;
        stack.push_back(h >> 1);
      }
  }
  if (overflow && status == 0) status = 2;
  for (int h = 0; h < 2 * E; ++h) after += face_sign(h) <= 0;

  FILE* out = fopen(argv[2], "wb");
  if (!out) return 3;
  const int32_t head[5] = {status, flips, wrapped, before, after};
  wr(out, head, 5);
  wr(out, pos.data(), n);
  wr(out, ev.data(), E);
  wr(out, en.data(), E);
  wr(out, eo.data(), E);
  fclose(out);
  return 0;
}
