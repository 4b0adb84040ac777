// Oracle half-edge mesh: a CPU restatement of the reference's HostTriangulation
// (include/Host_Triangulation.h) plus an exact Delaunay builder.
// Test infrastructure only: the shipped library never links this.
#include "mesh.h"

#include <algorithm>
#include <cmath>
#include <stack>

namespace oracle {

// ---------------------------------------------------------------------------
// Bounding-square seed.  The initial arrays are the reference's interchange
// state (include/Host_Triangulation.h:107-137): four corners at +-1e7
// (include/Common_Triangulation.h:12-13), two triangles, ten half-edges, the
// odd half-edges of the four hull edges bordering the outside (t = -1).
Mesh::Mesh() {
  const float lo = -10000000.0f, hi = 10000000.0f;
  pos = {{lo, lo}, {hi, lo}, {hi, hi}, {lo, hi}};
  v = {{0, 0}, {1, 2}, {2, 6}, {3, 8}};
  he = {{2, 0, 0, 2},  {9, 1, -1, -1}, {4, 1, 0, 0},  {1, 2, -1, -1}, {0, 2, 0, 1},
        {6, 0, 1, 3},  {8, 2, 1, 0},   {3, 3, -1, -1}, {5, 3, 1, 2},  {7, 0, -1, -1}};
  t = {{4}, {5}};
}

int Mesh::orient(const P2& a, const P2& b, const P2& c) const {
  return mode == PRED_EXACT ? orient2d_exact(a, b, c) : orient2d_ref(a, b, c);
}

int Mesh::incircle_q(int v0, int v1, int v2, int v3) const {
  if (mode == PRED_EXACT)
    return incircle_sos(pos[v0], pos[v1], pos[v2], pos[v3], v0, v1, v2, v3);
  return incircle_ref(pos[v0], pos[v1], pos[v2], pos[v3]);
}

// ---------------------------------------------------------------------------
// Edge flip with the reference's slot semantics (include/Common_Triangulation.h:69-127):
// the two faces keep their ids, half-edge h0 becomes the new diagonal's
// half-edge in face t0, and every rewritten half-edge is listed once as
// {slot, next, origin, face, opposite}.
void Mesh::f2to2(int h0) {
  const int h1 = h0 ^ 1;
  const int h2 = he[h0].next, h3 = he[h2].next;
  const int h4 = he[h1].next, h5 = he[h4].next;
  const int t0 = he[h0].t, t1 = he[h1].t;
  const int a = he[h0].v, b = he[h1].v, c = he[h3].v, d = he[h5].v;
  t[t0].he = h0;
  t[t1].he = h1;
  v[b].he = h2;
  v[a].he = h4;
  const int rows[6][5] = {{h0, h5, c, t0, b}, {h5, h2, d, t0, c}, {h2, h0, b, t0, d},
                          {h1, h3, d, t1, a}, {h3, h4, c, t1, d}, {h4, h1, a, t1, c}};
  for (const auto& r : rows) he[r[0]] = {r[1], r[2], r[3], r[4]};
  ++flips;
}

// 1-to-3 split of face t_index by the new vertex v_new
// (include/Common_Triangulation.h:129-209).  t_a/t_b are the two new faces and
// he_a/he_b/he_c the even-or-odd half-edges of the three new spokes as passed by
// addDelaunayPoint (Host_Triangulation.h:265-272).
void Mesh::f1to3(int t_index, int v_new, int t_a, int t_b, int he_a, int he_b, int he_c) {
  const int g0 = t[t_index].he, g1 = he[g0].next, g2 = he[g1].next;
  const int s8 = he_a, s7 = he_a ^ 1, s6 = he_b, s5 = he_b ^ 1, s4 = he_c, s3 = he_c ^ 1;
  const int x0 = he[g0].v, x1 = he[g1].v, x2 = he[g2].v;
  t[t_index].he = g0;
  t[t_a].he = g1;
  t[t_b].he = g2;
  v[v_new].he = s4;
  const int rows[9][5] = {{g0, s3, x0, t_index, v_new}, {s3, s5, x1, t_index, x0},
                          {s5, g0, v_new, t_index, x1}, {g1, s7, x1, t_a, v_new},
                          {s7, s4, x2, t_a, x1},        {s4, g1, v_new, t_a, x2},
                          {g2, s6, x2, t_b, v_new},     {s6, s8, x0, t_b, x2},
                          {s8, g2, v_new, t_b, x0}};
  for (const auto& r : rows) he[r[0]] = {r[1], r[2], r[3], r[4]};
}

// 2-to-4 split of the edge of half-edge h0 by a vertex lying exactly on it.
// The reference leaves this case as a stub (Common_Triangulation.h:211); the
// oracle needs it for inputs with collinear points.  Uses the last two faces and
// last six half-edges (pushed by the caller, like addDelaunayPoint does).
void Mesh::f2to4(int h0, int vn) {
  const int h1 = h0 ^ 1;
  const int n0 = he[h0].next, p0 = he[n0].next;  // b->c, c->a
  const int n1 = he[h1].next, p1 = he[n1].next;  // a->d, d->b
  const int t0 = he[h0].t, t1 = he[h1].t;
  const int a = he[h0].v, b = he[h1].v, c = he[p0].v, d = he[p1].v;
  const int HEn = (int)he.size(), Tn = (int)t.size();
  const int vb = HEn - 6, bv = HEn - 5, vc = HEn - 4, cv = HEn - 3, vd = HEn - 2, dv = HEn - 1;
  const int ta = Tn - 2, tb = Tn - 1;
  // faces: (a,vn,c)=t0, (vn,b,c)=ta, (b,vn,d)=t1, (vn,a,d)=tb
  const int rows[12][5] = {{h0, vc, a, t0, c},  {vc, p0, vn, t0, a}, {p0, h0, c, t0, vn},
                           {vb, n0, vn, ta, c}, {n0, cv, b, ta, vn}, {cv, vb, c, ta, b},
                           {bv, vd, b, t1, d},  {vd, p1, vn, t1, b}, {p1, bv, d, t1, vn},
                           {h1, n1, vn, tb, d}, {n1, dv, a, tb, vn}, {dv, h1, d, tb, a}};
  for (const auto& r : rows) he[r[0]] = {r[1], r[2], r[3], r[4]};
  t[t0].he = h0;
  t[ta].he = vb;
  t[t1].he = p1;
  t[tb].he = h1;
  v[vn].he = vb;
  if (v[b].he == h1) v[b].he = n0;
}

// ---------------------------------------------------------------------------
// Point location by the reference's centroid walk
// (include/Host_Triangulation.h:148-186), with an iteration cap added.
int Mesh::walk_centroid(P2 p, int tg) const {
  int tprev = -1;
  const long cap = 20L * (long)t.size() + 1000;
  for (long it = 0; it < cap; ++it) {
    const int h[3] = {t[tg].he, he[t[tg].he].next, he[he[t[tg].he].next].next};
    const P2 pe[3] = {pos[he[h[0]].v], pos[he[h[0] ^ 1].v], pos[he[h[0]].op]};
    P2 cen;
    cen.x = (pe[0].x + pe[1].x + pe[2].x) / 3.f;
    cen.y = (pe[0].y + pe[1].y + pe[2].y) / 3.f;
    bool moved = false;
    for (int i = 0; i < 3 && !moved; ++i) {
      const int tn = he[h[i] ^ 1].t;
      if (tn == tprev) continue;
      const P2& s = pe[i];
      const P2& r = pe[(i + 1) % 3];
      if (orient(cen, p, s) != orient(cen, p, r) && orient(s, r, cen) != orient(s, r, p)) {
        if (tn < 0) return -2;  // walked out of the bounding square
        tprev = tg;
        tg = tn;
        moved = true;
      }
    }
    if (!moved) return tg;
  }
  return -1;
}

// addDelaunayPoint (include/Host_Triangulation.h:248-280): locate, 1-to-3 split,
// then delonizeVertex on the new vertex.
bool Mesh::add_delaunay_point_ref(P2 p) {
  const int ti = walk_centroid(p, (int)t.size() - 1);
  if (ti < 0) { error = ti == -1 ? OERR_WALK_CAP : OERR_OUTSIDE; return false; }
  pos.push_back(p);
  v.push_back({(int)pos.size() - 1, 0});
  t.push_back({0});
  t.push_back({0});
  for (int k = 0; k < 6; ++k) he.push_back({0, 0, 0, 0});
  const int V = (int)v.size(), T = (int)t.size(), H = (int)he.size();
  f1to3(ti, V - 1, T - 1, T - 2, H - 1, H - 3, H - 5);
  delonize_vertex(V - 1);
  return true;
}

// delonizeEdge (include/Host_Triangulation.h:323-346).
bool Mesh::delonize_edge(int h) {
  if (he[h].t == -1 || he[h ^ 1].t == -1) return false;
  const int q0 = he[h].v, q1 = he[h ^ 1].op, q2 = he[h ^ 1].v, q3 = he[h].op;
  if (incircle_q(q0, q1, q2, q3) > 0) {
    f2to2(h);
    return true;
  }
  return false;
}

// delonizeVertex (include/Host_Triangulation.h:368-395): walk the outgoing
// spokes with NEXT_OUTGOING(h) = next(next(h))^1 and legalise each link edge
// until it stops flipping.
void Mesh::delonize_vertex(int vi) {
  const int first = v[vi].he;
  int cur = first;
  long guard = 0;
  const long cap = 64L * (long)he.size() + 1000;
  do {
    int link = he[cur].next;
    while (delonize_edge(link)) {
      link = he[cur].next;
      if (++guard > cap) { error = OERR_DELONIZE_CAP; return; }
    }
    cur = he[he[cur].next].next ^ 1;
    if (++guard > cap) { error = OERR_DELONIZE_CAP; return; }
  } while (cur != first);
}

// delonize (include/Host_Triangulation.h:305-319): restart the scan from edge 0
// after every flip.  This is the reference CPU algorithm timed as the baseline.
bool Mesh::delonize_restart_scan(long long max_flips) {
  bool flipped = false;
  bool ready = false;
  long long n = 0;
  while (!ready) {
    // the reference loops until no edge flips; on a mesh its untangling left
    // tangled that may never happen, so the CPU baseline passes a cap
    if (max_flips >= 0 && n++ >= max_flips) {
      capped = true;
      break;
    }
    ready = true;
    for (int i = 0; i < (int)he.size(); i += 2) {
      if (delonize_edge(i)) {
        ready = false;
        flipped = true;
        break;
      }
    }
  }
  return flipped;
}

// isCCW / isInside / isInsideInverted / isCreased
// (include/Helpers_Triangulation.h:163-209).
bool Mesh::is_ccw_face(int ti) const {
  const int h = t[ti].he;
  return orient(pos[he[h].v], pos[he[h ^ 1].v], pos[he[h].op]) >= 0;
}

bool Mesh::is_inside_face(const P2& p, int ti, bool inverted) const {
  const int h = t[ti].he;
  const int q[3] = {he[h].v, he[h ^ 1].v, he[h].op};
  for (int i = 0; i < 3; ++i) {
    const int s = orient(pos[q[i]], pos[q[(i + 1) % 3]], p);
    if (!inverted && s <= 0) return false;
    if (inverted && s >= 0) return false;
  }
  return true;
}

bool Mesh::is_creased(int h) const {
  if (he[h].t == -1 || he[h ^ 1].t == -1) return false;
  return is_ccw_face(he[h ^ 1].t) != is_ccw_face(he[h].t);
}

// untangleEdge: the reference's B-step and C-step
// (include/Host_Triangulation.h:425-471).  A/D/E are not implemented there.
bool Mesh::untangle_edge(int h) {
  if (!is_creased(h)) return false;
  int up = h, inv = h ^ 1;
  if (!is_ccw_face(he[up].t)) std::swap(up, inv);
  const P2 op_up = pos[he[he[he[up].next].next].v];
  const P2 op_inv = pos[he[he[he[inv].next].next].v];
  const int t_up = he[up].t, t_inv = he[inv].t;
  if (is_inside_face(op_inv, t_up, false)) { f2to2(h); return true; }
  if (is_inside_face(op_up, t_inv, true)) { f2to2(h); return true; }
  return false;
}

// untangle (include/Host_Triangulation.h:417-423): one pass over all edges.
bool Mesh::untangle_pass() {
  bool any = false;
  for (int i = 0; i < (int)he.size(); i += 2) any |= untangle_edge(i);
  return any;
}

// oneRing (include/Host_Triangulation.h:492-519), restated literally: forward
// with NEXT_OUTGOING until back at the start or a face of -1, then backward
// with PREV_OUTGOING(h) = next(h^1).  Interior vertices list neighbours twice.
std::vector<int> Mesh::one_ring_ref(int vi) const {
  std::vector<int> ring;
  int h0 = v[vi].he;
  if (he[h0].t == -1) h0 ^= 1;
  int cur = he[he[h0].next].next ^ 1;
  ring.push_back(he[h0 ^ 1].v);
  int guard = 0;
  while (cur != h0 && guard++ < 1 << 20) {
    if (he[cur].t == -1) break;
    ring.push_back(he[cur ^ 1].v);
    cur = he[he[cur].next].next ^ 1;
  }
  cur = he[h0 ^ 1].next;
  guard = 0;
  while (cur != h0 && guard++ < 1 << 20) {
    if (he[cur].t == -1) break;
    ring.push_back(he[cur ^ 1].v);
    cur = he[cur ^ 1].next;
  }
  return ring;
}

// getFRNN (include/Host_Triangulation.h:525-560): depth-first search over
// one-rings, keeping vertices with dot(p-q, p-q) <= r*r in float.
std::vector<int> Mesh::frnn_ref(int vi, float r) const {
  std::vector<int> nb;
  std::vector<char> visited(pos.size(), 0);
  std::stack<int> st;
  const P2 c = pos[vi];
  const float r2 = r * r;
  visited[vi] = 1;
  st.push(vi);
  while (!st.empty()) {
    const int s = st.top();
    st.pop();
    for (int a : one_ring_ref(s)) {
      if (visited[a]) continue;
      visited[a] = 1;
      const float dx = c.x - pos[a].x, dy = c.y - pos[a].y;
      const float dx2 = dx * dx, dy2 = dy * dy;
      if (dx2 + dy2 <= r2) {
        nb.push_back(a);
        st.push(a);
      }
    }
  }
  return nb;
}

// ---------------------------------------------------------------------------
// Exact builder: visibility walk with exact orientation.  Returns the face
// containing p; *on_he is the half-edge p lies on (or -1).  Negative returns:
// -1 cap, -2 outside, -3 duplicate vertex.
int Mesh::locate_exact(P2 p, int tg, int* on_he) const {
  *on_he = -1;
  const long cap = 20L * (long)t.size() + 1000;
  for (long it = 0; it < cap; ++it) {
    const int h[3] = {t[tg].he, he[t[tg].he].next, he[he[t[tg].he].next].next};
    int s[3];
    bool moved = false;
    for (int k = 0; k < 3; ++k) {
      const int i = (k + (int)it) % 3;
      s[i] = orient(pos[he[h[i]].v], pos[he[he[h[i]].next].v], p);
      if (s[i] < 0) {
        const int tn = he[h[i] ^ 1].t;
        if (tn < 0) return -2;
        tg = tn;
        moved = true;
        break;
      }
    }
    if (moved) continue;
    int zeros = 0, zi = -1;
    for (int i = 0; i < 3; ++i)
      if (s[i] == 0) { ++zeros; zi = i; }
    if (zeros >= 2) return -3;
    if (zeros == 1) {
      if (he[h[zi] ^ 1].t < 0) return -2;  // on the bounding square
      *on_he = h[zi];
    }
    return tg;
  }
  return -1;
}

// addDelaunayPoint with exact predicates and symbolic perturbation: locate,
// split (1-to-3 inside a face, 2-to-4 on an edge), then delonizeVertex.
bool Mesh::add_delaunay_point_exact(P2 p) {
  int on_he = -1;
  const int ti = locate_exact(p, (int)t.size() - 1, &on_he);
  if (ti < 0) {
    error = ti == -1 ? OERR_WALK_CAP : (ti == -3 ? OERR_DUPLICATE : OERR_OUTSIDE);
    return false;
  }
  pos.push_back(p);
  v.push_back({(int)pos.size() - 1, 0});
  t.push_back({0});
  t.push_back({0});
  for (int k = 0; k < 6; ++k) he.push_back({0, 0, 0, 0});
  const int V = (int)v.size(), T = (int)t.size(), H = (int)he.size();
  if (on_he < 0) f1to3(ti, V - 1, T - 1, T - 2, H - 1, H - 3, H - 5);
  else f2to4(on_he, V - 1);
  delonize_vertex(V - 1);
  return error == 0;
}

// ---------------------------------------------------------------------------
uint64_t morton_key(float x, float y) {
  // libmorton's m2D_e_LUT<uint_fast32_t,uint_fast32_t>(x, y) on float arguments
  // converted to a 64-bit unsigned integer; the conversion truncates toward
  // zero (negative values wrap as two's complement) and only the low 32 bits
  // of each coordinate are interleaved, x into the even bits.
  const uint64_t xi = (uint64_t)(int64_t)x, yi = (uint64_t)(int64_t)y;
  auto spread = [](uint64_t w) {
    w &= 0xFFFFFFFFull;
    w = (w | (w << 16)) & 0x0000FFFF0000FFFFull;
    w = (w | (w << 8)) & 0x00FF00FF00FF00FFull;
    w = (w | (w << 4)) & 0x0F0F0F0F0F0F0F0Full;
    w = (w | (w << 2)) & 0x3333333333333333ull;
    w = (w | (w << 1)) & 0x5555555555555555ull;
    return w;
  };
  return spread(xi) | (spread(yi) << 1);
}

void morton_sort(std::vector<P2>& pts) {
  std::sort(pts.begin(), pts.end(),
            [](const P2& a, const P2& b) { return morton_key(a.x, a.y) < morton_key(b.x, b.y); });
}

std::vector<std::pair<int, int>> edge_set(const Mesh& m) {
  std::vector<std::pair<int, int>> e;
  e.reserve(m.he.size() / 2);
  for (size_t i = 0; i + 1 < m.he.size(); i += 2) {
    int a = m.he[i].v, b = m.he[i + 1].v;
    if (a > b) std::swap(a, b);
    e.push_back({a, b});
  }
  std::sort(e.begin(), e.end());
  return e;
}

MeshCheck check_mesh(const Mesh& m, bool exact) {
  MeshCheck c = {0, 0, 0, 0};
  Mesh& mm = const_cast<Mesh&>(m);
  const int saved = mm.mode;
  mm.mode = exact ? PRED_EXACT : PRED_REF;
  for (size_t i = 0; i + 1 < m.he.size(); i += 2) {
    const int h = (int)i;
    if (m.he[h].t == -1 || m.he[h ^ 1].t == -1) continue;
    if (mm.incircle_q(m.he[h].v, m.he[h ^ 1].op, m.he[h ^ 1].v, m.he[h].op) > 0) ++c.non_delaunay;
    if (mm.is_creased(h)) ++c.creased;
  }
  for (size_t ti = 0; ti < m.t.size(); ++ti) {
    const int h = m.t[ti].he;
    const int s = mm.orient(m.pos[m.he[h].v], m.pos[m.he[h ^ 1].v], m.pos[m.he[h].op]);
    if (s < 0) ++c.inverted_faces;
    if (s == 0) ++c.zero_faces;
  }
  mm.mode = saved;
  return c;
}

}  // namespace oracle
