// Flat-torus (periodic) meshes: the lattice offsets of an edge's quad.
//
// A periodic mesh has no bounding square: n vertices on the torus
// [2L, 3L)^2 (L a power of two), 3n edges, 2n faces.  An edge's four vertices
// are stored by id in ev[e] = (a, b, c, d) exactly as for the planar engine
// (h0 = 2e: a -> b with apex c, h1 = 2e + 1: b -> a with apex d); which copy
// of each vertex the quad uses is given by three lattice offsets, in periods:
//
//   B  = t(h0)  the copy of b that h0 ends at, relative to a;
//   C  = x(h0)  the copy of the apex c in h0's face, relative to a;
//   X1 = x(h1)  the copy of the apex d in h1's face, relative to b
//               (so d sits at D = B + X1 in a's frame).
//
// Each component is -1, 0 or +1 for a mesh whose edges and face circumcircles
// are shorter than half a period.  They are packed one byte per offset into a
// u32 per edge (byte 0 = B, byte 1 = C, byte 2 = X1), a nibble per component
// biased by 8: x(h) of half-edge 2e + s is byte 1 + s of eo[e], so a flip can
// rewrite the apex offset of a wing half-edge with a byte store, and the wraps
// of an edge's vertices update its word with signed adds (the bias keeps every
// nibble in 0..15, so no borrow crosses a field).
//
// Exact translates: with positions in [2L, 3L), x + L stays in the binade
// [2L, 4L) and x - L lands in [L, 2L), whose grid is finer, so every
// translated coordinate the predicates see is an exact float and the
// FP32-filter / exact ladder applies unchanged.  The lifted-perturbation
// incircle (ids ascending) is invariant under translation, so the copies of a
// vertex are perturbed alike.
#pragma once

#include "predicates.cuh"
#include "../../include/mcl_gb300.h"
#if defined(__CUDACC__)
#include <cooperative_groups.h>
#include <cooperative_groups/scan.h>
#endif

namespace mcl {

struct Off {
  int x, y;
};

MCL_HD Off off_add(Off a, Off b) { return Off{a.x + b.x, a.y + b.y}; }
MCL_HD Off off_sub(Off a, Off b) { return Off{a.x - b.x, a.y - b.y}; }
MCL_HD Off off_neg(Off a) { return Off{-a.x, -a.y}; }
MCL_HD bool off_small(Off a) { return a.x >= -1 && a.x <= 1 && a.y >= -1 && a.y <= 1; }
MCL_HD bool off_zero(Off a) { return a.x == 0 && a.y == 0; }

MCL_HD unsigned off_byte(Off o) { return (unsigned)(o.x + 8) | ((unsigned)(o.y + 8) << 4); }
MCL_HD Off off_from_byte(unsigned b) { return Off{(int)(b & 15u) - 8, (int)((b >> 4) & 15u) - 8}; }

// eo of an edge with all three offsets zero (an edge away from the sides)
constexpr unsigned kEoZero = 0x888888u;

MCL_HD unsigned eo_pack(Off B, Off C, Off X1) {
  return off_byte(B) | (off_byte(C) << 8) | (off_byte(X1) << 16);
}
MCL_HD Off eo_b(unsigned w) { return off_from_byte(w & 0xFFu); }
MCL_HD Off eo_c(unsigned w) { return off_from_byte((w >> 8) & 0xFFu); }
MCL_HD Off eo_x1(unsigned w) { return off_from_byte((w >> 16) & 0xFFu); }
// apex offset of half-edge 2e + side, relative to its own origin
MCL_HD Off eo_apex(unsigned w, int side) { return side ? eo_x1(w) : eo_c(w); }
// target offset of half-edge 2e + side, relative to its own origin
MCL_HD Off eo_target(unsigned w, int side) { return side ? off_neg(eo_b(w)) : eo_b(w); }

// p translated by o periods (exact for positions in [2L, 3L) and |o| <= 1)
template <typename F2>
MCL_HD F2 off_translate(F2 p, Off o, float L) {
  F2 q = p;
  q.x = fadd(p.x, (float)o.x * L);
  q.y = fadd(p.y, (float)o.y * L);
  return q;
}

// The quad of an edge in a's frame: the copies of b, c and d as the edge's
// faces see them.  False when an offset falls outside -1..+1 (a mesh with
// edges longer than half a period, which the caller reports).
template <typename F2>
MCL_HD bool quad_frame(unsigned w, F2 pb, F2 pc, F2 pd, float L, F2& qb, F2& qc, F2& qd) {
  const Off B = eo_b(w), C = eo_c(w), D = off_add(B, eo_x1(w));
  if (!off_small(B) || !off_small(C) || !off_small(D)) return false;
  qb = off_translate(pb, B, L);
  qc = off_translate(pc, C, L);
  qd = off_translate(pd, D, L);
  return true;
}

// Offsets after flipping edge e, whose quad (a, b, c, d) becomes
// ev[e] = (d, c, a, b) with en[e] = (p0, n1, p1, n0) (the planar engine's
// flip).  In a's frame b sits at B, c at C, d at D = B + X1; the new edge runs
// d -> c with apex a and c -> d with apex b, and the wing half-edges get new
// apexes: p0 (c -> a) apex d, n1 (a -> d) apex c, p1 (d -> b) apex c,
// n0 (b -> c) apex d.  Each wing offset is relative to that wing's origin and
// is stored as byte 1 + (h & 1) of the wing's edge word.
struct FlipOffsets {
  unsigned eo;           // new word of the flipped edge
  unsigned char p0, n1, p1, n0;  // new apex-offset bytes of the wings
};

MCL_HD FlipOffsets flip_offsets(unsigned w) {
  const Off B = eo_b(w), C = eo_c(w), D = off_add(B, eo_x1(w));
  FlipOffsets f;
  f.eo = eo_pack(off_sub(C, D), off_neg(D), off_sub(B, C));
  f.p0 = (unsigned char)off_byte(off_sub(D, C));
  f.n1 = (unsigned char)off_byte(C);
  f.p1 = (unsigned char)off_byte(off_sub(C, D));
  f.n0 = (unsigned char)off_byte(off_sub(D, B));
  return f;
}

// Signed addend to an edge word when one of its quad's vertices changes its
// canonical copy: the vertex's new position is old - w periods.  `role` is the
// vertex's place in ev[e]: 0 = a (origin of h0), 1 = b, 2 = c, 3 = d.  Adding
// the results for the four roles (in any order) gives B' = B + w_b - w_a,
// C' = C + w_c - w_a, X1' = X1 + w_d - w_b.
MCL_HD int eo_wrap_delta(int role, Off w) {
  auto field = [](int byte, Off o) { return o.x * (1 << (8 * byte)) + o.y * (1 << (8 * byte + 4)); };
  switch (role) {
    case 0: return -field(0, w) - field(1, w);
    case 1: return field(0, w) - field(2, w);
    case 2: return field(1, w);
    default: return field(2, w);
  }
}

// Brings a moved position (old canonical + displacement, rounded) back into
// [lo, lo + L) (lo = 2L) and returns the periods w subtracted per axis (-1, 0
// or +1 for a move shorter than a period).  Above the domain the subtraction
// is exact; below it, q + L is rounded to the domain's grid, and that rounded
// value is the vertex's new position (if it rounds up to lo + L, q was within
// half a grid step of lo: the vertex lands on lo itself, w = 0).
MCL_HD float wrap_axis(float q, float lo, float L, int& w) {
  w = 0;
  if (q >= lo + L) {
    w = 1;
    return fsub(q, L);
  }
  if (q < lo) {
    const float r = fadd(q, L);
    if (r >= lo + L) return lo;
    w = -1;
    return r;
  }
  return q;
}

template <typename F2>
MCL_HD Off wrap_position(F2& p, float lo, float L) {
  Off w;
  p.x = wrap_axis(p.x, lo, L, w.x);
  p.y = wrap_axis(p.y, lo, L, w.y);
  return w;
}

// ---------------------------------------------------------------------------
// The periodic step's per-thread bodies.  Each kernel of the step is one of
// these over a flat index; they compile for host and device, so the CPU test
// suite runs the very same code serially (a serial run of a launch gives the
// GPU's result: claims are max-reductions and the flips of one round write
// disjoint fields).

struct alignas(8) PF2 {
  float x, y;
};
struct alignas(16) PI4 {
  int x, y, z, w;
};

// step counters, reset by the host before each step (nondelaunay before each round)
struct PCount {
  unsigned long long wrapped, inverted, nondelaunay, flips, incircle_fp64, incircle_exact, orient_fp64, orient_exact,
      sos, overflow, error, error_site, truncated, reverted, behind;
  unsigned long long lcount[2];  // entries of the two edge work-lists
  unsigned long long reinserted;  // vertices removed and reinserted at their targets
  unsigned long long hard;        // edges a classification left to the full predicates
};

struct PView {
  int n;          // vertices
  int E;          // edges (3n)
  float L, lo;    // period, lower side of the domain (2L)
  PF2* pos;       // canonical positions, in [lo, lo + L)^2
  PI4* ev;        // (a, b, c, d)
  PI4* en;        // (next h0, prev h0, next h1, prev h1)
  unsigned* eo;   // offsets (B, C, X1)
  unsigned char* wv;          // wraps still to fold into the edge words (an offset byte per vertex)
  unsigned char* wt;          // this step's net wrap of each vertex
  unsigned char* mark;        // vertices of faces the move turned over
  PF2* pos_old;               // positions before the current move
  PF2* target;                // where the step's move puts each vertex (wrapped)
  unsigned* cand;             // round stamp of the non-Delaunay edges
  unsigned long long* claim;  // face claims, by the smallest half-edge id of the face
  PCount* cnt;
  int* clist;                 // this round's non-Delaunay edges (cnt->nondelaunay of them)
  int* wl0;                   // edge work-lists: the edges whose quads a round's flips changed
  int* wl1;
  unsigned* qstamp;           // the round an edge was last queued for
};

MCL_HD void p_add(unsigned long long* p, unsigned long long v) {
#if defined(__CUDA_ARCH__)
  atomicAdd(p, v);
#else
  *p += v;
#endif
}
// a slot of a list counted by *p; on the device the threads that reach the
// call together (which all count on the same *p in every caller) share one
// atomicAdd
// k slots of a list counted by *p (the same sharing as p_inc)
MCL_HD unsigned long long p_inc_n(unsigned long long* p, unsigned k) {
#if defined(__CUDA_ARCH__)
  cooperative_groups::coalesced_group grp = cooperative_groups::coalesced_threads();
  const unsigned before = cooperative_groups::exclusive_scan(grp, k);
  unsigned long long base = 0;
  if (grp.thread_rank() == grp.size() - 1) base = atomicAdd(p, (unsigned long long)(before + k));
  base = grp.shfl(base, grp.size() - 1);
  return base + before;
#else
  const unsigned long long at = *p;
  *p += k;
  return at;
#endif
}
MCL_HD unsigned long long p_inc(unsigned long long* p) {
#if defined(__CUDA_ARCH__)
  cooperative_groups::coalesced_group grp = cooperative_groups::coalesced_threads();
  unsigned long long base = 0;
  if (grp.thread_rank() == 0) base = atomicAdd(p, (unsigned long long)grp.size());
  base = grp.shfl(base, 0);
  return base + grp.thread_rank();
#else
  return (*p)++;
#endif
}
MCL_HD unsigned p_exch(unsigned* p, unsigned v) {
#if defined(__CUDA_ARCH__)
  return atomicExch(p, v);
#else
  const unsigned old = *p;
  *p = v;
  return old;
#endif
}
MCL_HD void p_max(unsigned long long* p, unsigned long long v) {
#if defined(__CUDA_ARCH__)
  atomicMax(p, v);
#else
  if (v > *p) *p = v;
#endif
}
MCL_HD void p_error(const PView& V, int code, int site) {
#if defined(__CUDA_ARCH__)
  atomicCAS(&V.cnt->error, 0ull, (unsigned long long)code);
  atomicCAS(&V.cnt->error_site, 0ull, (unsigned long long)site);
#else
  if (!V.cnt->error) V.cnt->error = (unsigned long long)code;
  if (!V.cnt->error_site) V.cnt->error_site = (unsigned long long)site;
#endif
}

MCL_HD bool p_vertices_ok(const PView& V, PI4 q) {
  return (unsigned)q.x < (unsigned)V.n && (unsigned)q.y < (unsigned)V.n && (unsigned)q.z < (unsigned)V.n &&
         (unsigned)q.w < (unsigned)V.n;
}
MCL_HD bool p_halfedges_ok(const PView& V, PI4 w) {
  const unsigned H = 2u * (unsigned)V.E;
  return (unsigned)w.x < H && (unsigned)w.y < H && (unsigned)w.z < H && (unsigned)w.w < H;
}

// a bijective 32-bit mix (xor-shift / multiply rounds) for claim priorities
MCL_HD unsigned p_mix(unsigned x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}
MCL_HD unsigned long long p_key(int e, unsigned stamp) {
  return ((unsigned long long)stamp << 32) | (unsigned)(~p_mix((unsigned)e ^ stamp));
}
MCL_HD int p_min(int a, int b) { return a < b ? a : b; }
MCL_HD int p_face_a(int e, PI4 w) { return p_min(2 * e, p_min(w.x, w.y)); }
MCL_HD int p_face_b(int e, PI4 w) { return p_min(2 * e + 1, p_min(w.z, w.w)); }

struct PLocal {
  int incircle_fp64 = 0, incircle_exact = 0, orient_fp64 = 0, orient_exact = 0, sos = 0, overflow = 0;
};
MCL_HD void p_flush(const PView& V, const PLocal& lc) {
  if (lc.incircle_fp64) p_add(&V.cnt->incircle_fp64, lc.incircle_fp64);
  if (lc.incircle_exact) p_add(&V.cnt->incircle_exact, lc.incircle_exact);
  if (lc.orient_fp64) p_add(&V.cnt->orient_fp64, lc.orient_fp64);
  if (lc.orient_exact) p_add(&V.cnt->orient_exact, lc.orient_exact);
  if (lc.sos) p_add(&V.cnt->sos, lc.sos);
  if (lc.overflow) p_add(&V.cnt->overflow, 1);
}

// vertex v at p: move by dv, wrap into the domain, record the wrap
MCL_HD void p_move_with(const PView& V, int v, PF2 p, PF2 dv) {
  V.pos_old[v] = p;
  V.mark[v] = 0;
  V.wt[v] = (unsigned char)off_byte(Off{0, 0});
  p.x = fadd(p.x, dv.x);
  p.y = fadd(p.y, dv.y);
  const Off w = wrap_position(p, V.lo, V.L);
  if (!(p.x >= V.lo && p.x < V.lo + V.L && p.y >= V.lo && p.y < V.lo + V.L)) {
    p_error(V, MCL_ERR_INVALID_ARGUMENT, 1);  // a move of a period or more, or not finite
    V.wv[v] = (unsigned char)off_byte(Off{0, 0});
    return;
  }
  V.pos[v] = p;
  V.wv[v] = (unsigned char)off_byte(w);
  V.wt[v] = (unsigned char)off_byte(w);
  if (!off_zero(w)) p_add(&V.cnt->wrapped, 1);
}
// vertex v: move by d[v]
MCL_HD void p_body_move(const PView& V, const PF2* d, int v) { p_move_with(V, v, V.pos[v], d[v]); }

// vertex v at p before the step: its target, the wrapped p + dv (the same
// arithmetic as p_move_with)
MCL_HD void p_target_with(const PView& V, int v, PF2 p, PF2 dv) {
  p.x = fadd(p.x, dv.x);
  p.y = fadd(p.y, dv.y);
  wrap_position(p, V.lo, V.L);
  V.target[v] = p;
}
MCL_HD void p_body_target(const PView& V, const PF2* d, int v) { p_target_with(V, v, V.pos[v], d[v]); }

// the exact difference to the copy of t nearest to p along one axis (both in
// [lo, lo + L); t - p, t - L - p and t + L - p are exact by Sterbenz's lemma)
MCL_HD float p_toward(float t, float p, float L) {
  const float r = fsub(t, p);
  if (r > 0.5f * L) return fsub(fsub(t, L), p);
  if (r < -0.5f * L) return fsub(fadd(t, L), p);
  return r;
}

// vertex v, between sub-steps: the displacement still owed to a vertex that
// is not at its target: half of it, or (last) all of it, which lands the
// vertex exactly on its target; zero for the others.  Counts the vertices
// still behind.
MCL_HD void p_resume_with(const PView& V, PF2* d, int v, PF2 p, PF2 t, bool last) {
  PF2 r{0.f, 0.f};
  if (p.x != t.x || p.y != t.y) {
    r.x = p_toward(t.x, p.x, V.L);
    r.y = p_toward(t.y, p.y, V.L);
    if (!last) {
      r.x = fmul(r.x, 0.5f);
      r.y = fmul(r.y, 0.5f);
    }
    p_add(&V.cnt->behind, 1);
  }
  d[v] = r;
}
MCL_HD void p_body_resume(const PView& V, PF2* d, int v, bool last) {
  p_resume_with(V, d, v, V.pos[v], V.target[v], last);
}

// vertex v, after a classification that found faces turned over: a marked
// vertex (the farthest-moved of a turned face) goes back to its old position,
// and its wrap is undone in the next fold; every other vertex folds nothing.
// Repeated until no face is turned over, this ends: a turned face always has a
// moved vertex, and at worst every moved vertex is back where the valid mesh
// had it.
MCL_HD void p_body_revert(const PView& V, int v) {
  const Off none{0, 0};
  V.wv[v] = (unsigned char)off_byte(none);
  if (!V.mark[v]) return;
  V.mark[v] = 0;
  const PF2 p = V.pos[v], q = V.pos_old[v];
  if (p.x == q.x && p.y == q.y) return;
  V.pos[v] = q;
  V.wv[v] = (unsigned char)off_byte(off_neg(off_from_byte(V.wt[v])));
  V.wt[v] = (unsigned char)off_byte(none);
  p_add(&V.cnt->reverted, 1);
}

// edge e of quad q: the wraps of its vertices (offset bytes wa..wd) into its
// offset word
MCL_HD void p_wrap_with(const PView& V, int e, unsigned char wa, unsigned char wb, unsigned char wc,
                        unsigned char wd) {
  const unsigned char r[4] = {wa, wb, wc, wd};
  int delta = 0;
  for (int k = 0; k < 4; ++k) {
    const Off w = off_from_byte(r[k]);
    if (!off_zero(w)) delta += eo_wrap_delta(k, w);
  }
  if (delta) V.eo[e] = V.eo[e] + (unsigned)delta;
}
// edge e: the wraps of its quad's vertices into its offset word
MCL_HD void p_body_wrap(const PView& V, int e) {
  const PI4 q = V.ev[e];
  if (!p_vertices_ok(V, q)) {
    p_error(V, MCL_ERR_DEGENERATE_INPUT, 2);
    return;
  }
  p_wrap_with(V, e, V.wv[q.x], V.wv[q.y], V.wv[q.z], V.wv[q.w]);
}

// the length, squared, of vertex v's current move on the torus (exact
// differences; float squares)
MCL_HD float p_moved2(const PView& V, int v) {
  const PF2 p = V.pos[v], q = V.pos_old[v];
  const float dx = p_toward(p.x, q.x, V.L), dy = p_toward(p.y, q.y, V.L);
  return fadd(fmul(dx, dx), fmul(dy, dy));
}
// the vertex of a turned face that goes back: the one that moved farthest
// (the smallest id among equals); sending it back ends the turn in most
// cases, and a face still turned marks another vertex in the next pass
MCL_HD int p_culprit(const PView& V, int a, int b, int c) {
  const float ma = p_moved2(V, a), mb = p_moved2(V, b), mc = p_moved2(V, c);
  int best = a;
  float bm = ma;
  if (mb > bm || (mb == bm && b < best)) { best = b; bm = mb; }
  if (mc > bm || (mc == bm && c < best)) { best = c; bm = mc; }
  return best;
}

// non-Delaunay edge e: its wings (en), a claim on both its faces for this
// round, and a place in the round's list
MCL_HD void p_claim_nd(const PView& V, int e, unsigned stamp) {
  const PI4 w = V.en[e];
  if (!p_halfedges_ok(V, w)) {
    p_error(V, MCL_ERR_DEGENERATE_INPUT, 3);
    return;
  }
  const unsigned long long key = p_key(e, stamp);
  p_max(V.claim + p_face_a(e, w), key);
  p_max(V.claim + p_face_b(e, w), key);
  V.cand[e] = stamp;
  V.clist[p_inc(&V.cnt->nondelaunay)] = e;
}

// edge e (record q with its vertices in range, offset word o, its quad's
// vertices at pa .. pd in their canonical positions): orientation of its two
// faces and, when both are positive, the incircle test; a non-Delaunay edge
// reads its wings (en) and claims both faces for this round and joins the
// round's list
MCL_HD void p_classify_with(const PView& V, int e, unsigned stamp, PI4 q, unsigned o, PF2 pa, PF2 pb, PF2 pc,
                            PF2 pd) {
  PF2 qb, qc, qd;
  if (!quad_frame(o, pb, pc, pd, V.L, qb, qc, qd)) {
    p_error(V, MCL_ERR_DEGENERATE_INPUT, 4);  // an offset outside -1..+1
    return;
  }
  PLocal lc;
  const int sa = orient2d(pa.x, pa.y, qb.x, qb.y, qc.x, qc.y, &lc, &lc.overflow);
  const int sb = orient2d(qb.x, qb.y, pa.x, pa.y, qd.x, qd.y, &lc, &lc.overflow);
  if (sa <= 0 || sb <= 0) {
    p_add(&V.cnt->inverted, (unsigned long long)((sa <= 0) + (sb <= 0)));
    if (sa <= 0) V.mark[p_culprit(V, q.x, q.y, q.z)] = 1;
    if (sb <= 0) V.mark[p_culprit(V, q.y, q.x, q.w)] = 1;
    p_flush(V, lc);
    return;
  }
  const bool nd =
      incircle_sos(pa.x, pa.y, qb.x, qb.y, qc.x, qc.y, qd.x, qd.y, q.x, q.y, q.z, q.w, &lc, &lc.overflow) > 0;
  p_flush(V, lc);
  if (nd) p_claim_nd(V, e, stamp);
}
// edge e: its record and positions, then p_classify_with
MCL_HD void p_body_classify(const PView& V, int e, unsigned stamp) {
  const PI4 q = V.ev[e];
  const unsigned o = V.eo[e];
  if (!p_vertices_ok(V, q)) {
    p_error(V, MCL_ERR_DEGENERATE_INPUT, 3);
    return;
  }
  p_classify_with(V, e, stamp, q, o, V.pos[q.x], V.pos[q.y], V.pos[q.z], V.pos[q.w]);
}

// edge e onto work-list k for the round with stamp `next`, once
MCL_HD void p_queue(const PView& V, int e, unsigned next, int k) {
  if (p_exch(V.qstamp + e, next) == next) return;
  int* wl = k ? V.wl1 : V.wl0;
  wl[p_inc(&V.cnt->lcount[k])] = e;
}

// the four wing edges of a flip onto work-list k for the round with stamp
// `next`, each once: the four marks first, then one reservation for those
// newly marked
MCL_HD void p_queue4(const PView& V, int e0, int e1, int e2, int e3, unsigned next, int k) {
  const int es[4] = {e0, e1, e2, e3};
  bool put[4];
  unsigned cnt = 0;
  for (int i = 0; i < 4; ++i) {
    put[i] = p_exch(V.qstamp + es[i], next) != next;
    cnt += put[i] ? 1u : 0u;
  }
  if (!cnt) return;
  int* wl = k ? V.wl1 : V.wl0;
  unsigned long long at = p_inc_n(&V.cnt->lcount[k], cnt);
  for (int i = 0; i < 4; ++i)
    if (put[i]) wl[at++] = es[i];
}

// one side of a wing half-edge h: its apex, next and prev, and its apex offset byte
MCL_HD void p_set_face(const PView& V, int h, int apex, int next, int prev, unsigned char apex_off) {
  const int e = h >> 1;
  PI4* q = V.ev + e;
  PI4* w = V.en + e;
  unsigned char* ob = reinterpret_cast<unsigned char*>(V.eo + e);
  if (h & 1) {
    q->w = apex;
    w->z = next;
    w->w = prev;
    ob[2] = apex_off;
  } else {
    q->z = apex;
    w->x = next;
    w->y = prev;
    ob[1] = apex_off;
  }
}

// edge e: flip when it holds the claims of both its faces (the planar
// engine's flip, plus the offsets); the four wing edges, whose quads changed,
// go onto work-list `next` for the next round, and so does a candidate that
// lost a claim
MCL_HD void p_body_flip(const PView& V, int e, unsigned stamp, int next) {
  if (V.cand[e] != stamp) return;
  const PI4 q = V.ev[e];
  const PI4 w = V.en[e];
  if (!p_vertices_ok(V, q) || !p_halfedges_ok(V, w)) {
    p_error(V, MCL_ERR_DEGENERATE_INPUT, 5);
    return;
  }
  const unsigned long long key = p_key(e, stamp);
  if (V.claim[p_face_a(e, w)] != key || V.claim[p_face_b(e, w)] != key) {
    // lost a face (possibly to another loser, so no flip may touch it): retry
    p_queue(V, e, stamp + 1, next);
    return;
  }
  const FlipOffsets f = flip_offsets(V.eo[e]);
  const int a = q.x, b = q.y, c = q.z, d = q.w;
  const int n0 = w.x, p0 = w.y, n1 = w.z, p1 = w.w;
  const int h0 = 2 * e, h1 = 2 * e + 1;
  V.ev[e] = PI4{d, c, a, b};
  V.en[e] = PI4{p0, n1, p1, n0};
  V.eo[e] = f.eo;
  p_set_face(V, p0, d, n1, h0, f.p0);
  p_set_face(V, n1, c, h0, p0, f.n1);
  p_set_face(V, p1, c, n0, h1, f.p1);
  p_set_face(V, n0, d, h1, p1, f.n0);
  p_add(&V.cnt->flips, 1);
  p_queue4(V, p0 >> 1, n1 >> 1, p1 >> 1, n0 >> 1, stamp + 1, next);
}

constexpr int kPeriodicMaxDeg = 4096;

MCL_HD int p_origin(const PView& V, int h) {
  const PI4 q = V.ev[h >> 1];
  return (h & 1) ? q.y : q.x;
}
// next outgoing half-edge clockwise around the origin: next(twin(h))
MCL_HD int p_rot(const PView& V, int h) {
  const PI4 w = V.en[(h ^ 1) >> 1];
  return ((h ^ 1) & 1) ? w.z : w.x;
}

// ---------------------------------------------------------------------------
// Removal and reinsertion of a vertex, one at a time (a single thread runs
// these for the few vertices that neither the step nor its sub-steps brought
// to their targets).  Faces are rewritten whole: p_make_face sets the three
// half-edges of a face from its vertices and their offsets in its first
// vertex's frame; vhe holds one outgoing half-edge per vertex and is kept up
// to date.

MCL_HD int p_next(const PView& V, int h) {
  const PI4 w = V.en[h >> 1];
  return (h & 1) ? w.z : w.x;
}
MCL_HD int p_prev(const PView& V, int h) {
  const PI4 w = V.en[h >> 1];
  return (h & 1) ? w.w : w.y;
}
MCL_HD int p_apex(const PView& V, int h) {
  const PI4 q = V.ev[h >> 1];
  return (h & 1) ? q.w : q.z;
}
MCL_HD Off p_tof(const PView& V, int h) { return eo_target(V.eo[h >> 1], h & 1); }
MCL_HD Off p_xof(const PView& V, int h) { return eo_apex(V.eo[h >> 1], h & 1); }

// one half-edge's whole record: origin, apex, next, prev, target offset t and
// apex offset x (both relative to the origin)
MCL_HD void p_set_half(const PView& V, int h, int origin, int apex, int next, int prev, Off t, Off x) {
  // field by field: the other side of the edge may be rewritten at the same
  // time by another thread (the parallel removal and reinsertion rounds);
  // byte 0 (the edge's offset) is the same value from either side
  const int e = h >> 1;
  unsigned char* ob = reinterpret_cast<unsigned char*>(V.eo + e);
  if (h & 1) {
    V.ev[e].y = origin;
    V.ev[e].w = apex;
    V.en[e].z = next;
    V.en[e].w = prev;
    ob[0] = (unsigned char)off_byte(off_neg(t));
    ob[2] = (unsigned char)off_byte(x);
  } else {
    V.ev[e].x = origin;
    V.ev[e].z = apex;
    V.en[e].x = next;
    V.en[e].y = prev;
    ob[0] = (unsigned char)off_byte(t);
    ob[1] = (unsigned char)off_byte(x);
  }
}

// face v0 -> v1 -> v2 of half-edges h0 (v0 -> v1), h1, h2, with v1 at O1 and
// v2 at O2 in v0's frame
MCL_HD void p_make_face(const PView& V, int h0, int h1, int h2, int v0, int v1, int v2, Off O1, Off O2) {
  p_set_half(V, h0, v0, v2, h1, h2, O1, O2);
  p_set_half(V, h1, v1, v0, h2, h0, off_sub(O2, O1), off_neg(O1));
  p_set_half(V, h2, v2, v1, h0, h1, off_neg(O2), off_sub(O1, O2));
}

MCL_HD int p_orient_at(const PView& V, PF2 a, PF2 b, PF2 c) {
  PLocal lc;
  const int s = orient2d(a.x, a.y, b.x, b.y, c.x, c.y, &lc, &lc.overflow);
  p_flush(V, lc);
  return s;
}

// flip of edge e done by one thread (the same rewrite as p_body_flip), with
// vhe kept; false when the flip would not leave both new faces positive
// (only checked when `check`)
MCL_HD bool p_flip_seq(const PView& V, int* vhe, int e, bool check) {
  const PI4 q = V.ev[e];
  const PI4 w = V.en[e];
  if (!p_vertices_ok(V, q) || !p_halfedges_ok(V, w)) {
    p_error(V, MCL_ERR_DEGENERATE_INPUT, 11);
    return false;
  }
  const unsigned o = V.eo[e];
  const Off B = eo_b(o), C = eo_c(o), D = off_add(B, eo_x1(o));
  if (!off_small(B) || !off_small(C) || !off_small(D)) {
    p_error(V, MCL_ERR_DEGENERATE_INPUT, 12);
    return false;
  }
  const int a = q.x, b = q.y, c = q.z, d = q.w;
  if (check) {
    const PF2 pa = V.pos[a], pb = off_translate(V.pos[b], B, V.L), pc = off_translate(V.pos[c], C, V.L),
              pd = off_translate(V.pos[d], D, V.L);
    if (p_orient_at(V, pd, pc, pa) <= 0 || p_orient_at(V, pc, pd, pb) <= 0) return false;
  }
  const int n0 = w.x, p0 = w.y, n1 = w.z, p1 = w.w, h0 = 2 * e, h1 = 2 * e + 1;
  p_make_face(V, h0, p0, n1, d, c, a, off_sub(C, D), off_neg(D));
  p_make_face(V, h1, p1, n0, c, d, b, off_sub(D, C), off_sub(B, C));
  if (vhe[a] == h0) vhe[a] = n1;
  if (vhe[b] == h1) vhe[b] = n0;
  p_add(&V.cnt->flips, 1);
  return true;
}

constexpr int kSeqStar = 64;  // largest star the one-thread removal takes apart

// Removes vertex v from the mesh (vhe[v] must be one of its outgoing
// half-edges): spoke flips down to degree 3, then its three faces merge into
// one.  The three freed edges go to freed[0..2], a half-edge of the merged
// face to *near, and every edge of the hole's new triangulation (and of its
// boundary) to hole[0..*nhole) for the flips that follow.  False (the mesh
// still valid) when the star is not one this can take apart.
MCL_HD bool p_remove_seq(const PView& V, int* vhe, int v, int* freed, int* near, int* hole, int* nhole) {
  const unsigned H = 2u * (unsigned)V.E;
  *nhole = 0;
  {
    // the hole's boundary: the link edges of v's star
    const int h0 = vhe[v];
    if ((unsigned)h0 >= H || p_origin(V, h0) != v) {
      p_error(V, MCL_ERR_DEGENERATE_INPUT, 13);
      return false;
    }
    int h = h0, deg = 0;
    do {
      if (deg == kSeqStar) return false;
      const int l = p_next(V, h);
      if ((unsigned)l >= H) {
        p_error(V, MCL_ERR_DEGENERATE_INPUT, 21);
        return false;
      }
      hole[(*nhole)++] = l >> 1;
      h = p_rot(V, h);
      ++deg;
    } while (h != h0 && (unsigned)h < H);
    if (h != h0) {
      p_error(V, MCL_ERR_DEGENERATE_INPUT, 14);
      return false;
    }
  }
  for (int guard = 0; guard < kSeqStar; ++guard) {
    const int h0 = vhe[v];
    if ((unsigned)h0 >= H || p_origin(V, h0) != v) {
      p_error(V, MCL_ERR_DEGENERATE_INPUT, 13);
      return false;
    }
    int deg = 0, h = h0;
    do {
      h = p_rot(V, h);
      ++deg;
    } while (h != h0 && deg < kPeriodicMaxDeg && (unsigned)h < H);
    if (h != h0) {
      p_error(V, MCL_ERR_DEGENERATE_INPUT, 14);
      return false;
    }
    if (deg == 3) break;
    if (deg < 3) return false;
    // a spoke whose flip keeps both new faces positive (one exists while the
    // star is a valid star of degree > 3)
    bool flipped = false;
    h = h0;
    for (int k = 0; k < deg && !flipped; ++k) {
      const int nh = p_rot(V, h);
      if (vhe[v] == h) vhe[v] = nh;  // h stops being v's after the flip
      if (p_flip_seq(V, vhe, h >> 1, true)) {
        flipped = true;
        hole[(*nhole)++] = h >> 1;  // now a diagonal of the hole
      } else {
        vhe[v] = h0;
        h = nh;
      }
    }
    if (!flipped) return false;
  }
  // degree 3: spokes s0, s1, s2; the link half-edges next(s_i) run between
  // the link vertices and become the merged face
  const int s0 = vhe[v], s1 = p_rot(V, s0), s2 = p_rot(V, s1);
  const int l[3] = {p_next(V, s0), p_next(V, s1), p_next(V, s2)};
  int lo[3], lt[3];
  Off lt_off[3];
  for (int k = 0; k < 3; ++k) {
    if ((unsigned)l[k] >= H) return false;
    lo[k] = p_origin(V, l[k]);
    lt[k] = p_origin(V, l[k] ^ 1);
    lt_off[k] = p_tof(V, l[k]);
  }
  if (lo[0] == lo[1] || lo[1] == lo[2] || lo[0] == lo[2]) return false;
  // order the link half-edges into a cycle: after l[i] comes the one leaving its target
  int ord[3] = {0, -1, -1};
  for (int k = 1; k < 3; ++k)
    for (int j = 0; j < 3; ++j)
      if (lo[j] == lt[ord[k - 1]]) ord[k] = j;
  if (ord[1] < 0 || ord[2] < 0 || lt[ord[2]] != lo[ord[0]]) return false;
  const int A = lo[ord[0]], Bv = lo[ord[1]], Cv = lo[ord[2]];
  const Off OB = lt_off[ord[0]], OC = off_add(OB, lt_off[ord[1]]);
  if (!off_small(OB) || !off_small(OC)) return false;
  freed[0] = s0 >> 1;
  freed[1] = s1 >> 1;
  freed[2] = s2 >> 1;
  p_make_face(V, l[ord[0]], l[ord[1]], l[ord[2]], A, Bv, Cv, OB, OC);
  vhe[A] = l[ord[0]];
  vhe[Bv] = l[ord[1]];
  vhe[Cv] = l[ord[2]];
  vhe[v] = -1;
  *near = l[ord[0]];
  return true;
}

// the copy of t nearest to p, and its offset in periods (exact: see p_toward)
MCL_HD PF2 p_nearest_copy(PF2 t, PF2 p, float L, Off& k) {
  PF2 q;
  q.x = fadd(p.x, p_toward(t.x, p.x, L));
  q.y = fadd(p.y, p_toward(t.y, p.y, L));
  k.x = q.x > t.x ? (fsub(q.x, t.x) > 0.5f * L ? 1 : 0) : (fsub(t.x, q.x) > 0.5f * L ? -1 : 0);
  k.y = q.y > t.y ? (fsub(q.y, t.y) > 0.5f * L ? 1 : 0) : (fsub(t.y, q.y) > 0.5f * L ? -1 : 0);
  return q;
}

// The face of canonical position t by the stochastic walk from half-edge h:
// *face = a half-edge of it, *vertex = t is one of its corners.  False (an
// error flagged) on a malformed mesh or a walk that does not end.
MCL_HD bool p_locate_face(const PView& V, PF2 t, int h, int* face, bool* vertex) {
  const unsigned H = 2u * (unsigned)V.E;
  for (int guard = 0; guard < (1 << 20); ++guard) {
    if ((unsigned)h >= H) {
      p_error(V, MCL_ERR_DEGENERATE_INPUT, 15);
      return false;
    }
    // stochastic walk: the first edge tested turns with the step, so the walk
    // ends in any triangulation, Delaunay or not
    const int a = p_origin(V, h), b = p_origin(V, h ^ 1), c = p_apex(V, h);
    if ((unsigned)a >= (unsigned)V.n || (unsigned)b >= (unsigned)V.n || (unsigned)c >= (unsigned)V.n) {
      p_error(V, MCL_ERR_DEGENERATE_INPUT, 16);
      return false;
    }
    const Off Ob = p_tof(V, h), Oc = p_xof(V, h);
    const PF2 pa = V.pos[a], pb = off_translate(V.pos[b], Ob, V.L), pc = off_translate(V.pos[c], Oc, V.L);
    Off K;
    const PF2 pt = p_nearest_copy(t, pa, V.L, K);
    const int o1 = p_orient_at(V, pa, pb, pt), o2 = p_orient_at(V, pb, pc, pt), o3 = p_orient_at(V, pc, pa, pt);
    const int cross[3] = {o1 < 0 ? h : -1, o2 < 0 ? p_next(V, h) : -1, o3 < 0 ? p_prev(V, h) : -1};
    int go = -1;
    for (int k = 0; k < 3 && go < 0; ++k) go = cross[(guard + k) % 3];
    if (go >= 0) {
      h = go ^ 1;
      continue;
    }
    *face = h;
    *vertex = (o1 == 0) + (o2 == 0) + (o3 == 0) >= 2;
    return true;
  }
  p_error(V, MCL_ERR_NO_CONVERGENCE, 17);
  return false;
}

// Splits the face of half-edge h, which holds t (inside or on one of its
// sides, as p_locate_face found it), by vertex v at t with the three free
// edges: 1 -> 3 inside, 2 -> 4 on a side; false when t is a corner.  The
// half-edges of the new star's link go to link[0..3] (count in *nlink).
MCL_HD bool p_split_at(const PView& V, int* vhe, int v, PF2 t, const int* f, int h, int* link, int* nlink) {
  const int a = p_origin(V, h), b = p_origin(V, h ^ 1), c = p_apex(V, h);
  const Off Ob = p_tof(V, h), Oc = p_xof(V, h);
  const PF2 pa = V.pos[a], pb = off_translate(V.pos[b], Ob, V.L), pc = off_translate(V.pos[c], Oc, V.L);
  Off K;
  const PF2 pt = p_nearest_copy(t, pa, V.L, K);
  const int o1 = p_orient_at(V, pa, pb, pt), o2 = p_orient_at(V, pb, pc, pt), o3 = p_orient_at(V, pc, pa, pt);
  const int zeros = (o1 == 0) + (o2 == 0) + (o3 == 0);
  if (zeros >= 2) return false;  // t is a vertex
  const Off Ov = K;              // v's copy in a's frame
  if (zeros == 0) {
    const int n = p_next(V, h), p = p_prev(V, h);
    p_make_face(V, h, 2 * f[1], 2 * f[0] + 1, a, b, v, Ob, Ov);
    p_make_face(V, n, 2 * f[2], 2 * f[1] + 1, b, c, v, off_sub(Oc, Ob), off_sub(Ov, Ob));
    p_make_face(V, p, 2 * f[0], 2 * f[2] + 1, c, a, v, off_neg(Oc), off_sub(Ov, Oc));
    vhe[v] = 2 * f[0] + 1;
    link[0] = h;
    link[1] = n;
    link[2] = p;
    *nlink = 3;
    return true;
  }
  // on one edge: make it g (a -> b) with v on the segment a b
  int g = h;
  if (o2 == 0) g = p_next(V, h);
  if (o3 == 0) g = p_prev(V, h);
  const int ga = p_origin(V, g), gb = p_origin(V, g ^ 1), gc = p_apex(V, g), gd = p_apex(V, g ^ 1);
  if ((unsigned)gd >= (unsigned)V.n) return false;
  // offsets in ga's frame
  const Off Gb = p_tof(V, g), Gc = p_xof(V, g), Gd = off_add(Gb, p_xof(V, g ^ 1));
  Off Ka;
  p_nearest_copy(t, off_translate(V.pos[ga], Off{0, 0}, V.L), V.L, Ka);
  const int ng = p_next(V, g), pg = p_prev(V, g), g1 = g ^ 1, ng1 = p_next(V, g1), pg1 = p_prev(V, g1);
  p_make_face(V, g, 2 * f[1] + 1, pg, ga, v, gc, Ka, Gc);
  p_make_face(V, 2 * f[0], ng, 2 * f[1], v, gb, gc, off_sub(Gb, Ka), off_sub(Gc, Ka));
  p_make_face(V, 2 * f[0] + 1, 2 * f[2] + 1, pg1, gb, v, gd, off_sub(Ka, Gb), off_sub(Gd, Gb));
  p_make_face(V, g1, ng1, 2 * f[2], v, ga, gd, off_neg(Ka), off_sub(Gd, Ka));
  vhe[v] = 2 * f[0];
  if (vhe[gb] == g1) vhe[gb] = 2 * f[0] + 1;
  link[0] = ng;
  link[1] = pg;
  link[2] = ng1;
  link[3] = pg1;
  *nlink = 4;
  return true;
}

// Inserts vertex v (not in the mesh) at canonical position t, using the
// three free edges, starting the point location walk at half-edge `near`.
// 1 -> 3 split inside a face, 2 -> 4 split on an edge; false when t is an
// existing vertex or the walk does not end.  Returns the half-edges of the
// new star's link in link[0..3] (count in *nlink) for the flips that follow.
MCL_HD bool p_insert_seq(const PView& V, int* vhe, int v, PF2 t, const int* f, int near, int* link, int* nlink) {
  int face = -1;
  bool vertex = false;
  if (!p_locate_face(V, t, near, &face, &vertex) || vertex) return false;
  return p_split_at(V, vhe, v, t, f, face, link, nlink);
}

constexpr int kSeqStack = 512;

// Lawson flips around a freshly inserted vertex, one thread: a stack of edges
// starting from the link of its star
MCL_HD bool p_lawson_seq(const PView& V, int* vhe, const int* link, int nlink) {
  int stack[kSeqStack];
  int top = 0;
  for (int k = 0; k < nlink; ++k) stack[top++] = link[k] >> 1;
  for (int guard = 0; top > 0 && guard < (1 << 20); ++guard) {
    const int e = stack[--top];
    const PI4 q = V.ev[e];
    PF2 qb, qc, qd;
    if (!p_vertices_ok(V, q) || !quad_frame(V.eo[e], V.pos[q.y], V.pos[q.z], V.pos[q.w], V.L, qb, qc, qd)) {
      p_error(V, MCL_ERR_DEGENERATE_INPUT, 18);
      return false;
    }
    const PF2 pa = V.pos[q.x];
    PLocal lc;
    const bool nd = orient2d(pa.x, pa.y, qb.x, qb.y, qc.x, qc.y, &lc, &lc.overflow) > 0 &&
                    orient2d(qb.x, qb.y, pa.x, pa.y, qd.x, qd.y, &lc, &lc.overflow) > 0 &&
                    incircle_sos(pa.x, pa.y, qb.x, qb.y, qc.x, qc.y, qd.x, qd.y, q.x, q.y, q.z, q.w, &lc,
                                 &lc.overflow) > 0;
    p_flush(V, lc);
    if (!nd) continue;
    const PI4 w = V.en[e];
    if (!p_flip_seq(V, vhe, e, false)) return false;
    if (top + 4 > kSeqStack) {
      p_error(V, MCL_ERR_CAPACITY, 19);
      return false;
    }
    stack[top++] = w.x >> 1;
    stack[top++] = w.y >> 1;
    stack[top++] = w.z >> 1;
    stack[top++] = w.w >> 1;
  }
  if (top != 0) p_error(V, MCL_ERR_NO_CONVERGENCE, 22);  // the flip guard ran out
  return top == 0;
}

// One thread: every listed vertex (list == null: every vertex, by ascending
// id) that is not at its target is removed and reinserted there (or, if its
// target is taken by another vertex, where it was), then the flips around it
// restore Delaunay; at most `limit` of them.
MCL_HD void p_body_reinsert(const PView& V, int* vhe, const int* list, int count, int limit) {
  int done = 0;
  for (int i = 0; i < count && done < limit && !V.cnt->error; ++i) {
    const int v = list ? list[i] : i;
    if ((unsigned)v >= (unsigned)V.n) continue;
    const PF2 here = V.pos[v], t = V.target[v];
    if (here.x == t.x && here.y == t.y) continue;
    ++done;
    int freed[3], near = -1, link[4], nlink = 0, hole[2 * kSeqStar], nhole = 0;
    if (!p_remove_seq(V, vhe, v, freed, &near, hole, &nhole)) {
      if (V.cnt->error) return;
      // refused (v stays where it was, counted as behind); spoke flips it
      // made first leave its star non-Delaunay: Lawson over the hole's sides,
      // the flipped spokes and v's remaining spokes
      if (nhole > 0) {
        int live[3 * kSeqStar], nlive = 0;
        for (int k = 0; k < nhole && nlive < 3 * kSeqStar; ++k) live[nlive++] = 2 * hole[k];
        const int h0 = vhe[v];
        if ((unsigned)h0 < 2u * (unsigned)V.E) {
          int h = h0;
          do {
            if (nlive < 3 * kSeqStar) live[nlive++] = h;
            h = p_rot(V, h);
          } while (h != h0 && (unsigned)h < 2u * (unsigned)V.E && nlive < 3 * kSeqStar);
        }
        if (!p_lawson_seq(V, vhe, live, nlive)) return;
      }
      continue;
    }
    // the hole was filled by arbitrary flips: make it Delaunay again (its
    // edges that died with v are skipped: they are free now)
    int live[2 * kSeqStar], nlive = 0;
    for (int k = 0; k < nhole; ++k)
      if (hole[k] != freed[0] && hole[k] != freed[1] && hole[k] != freed[2]) live[nlive++] = 2 * hole[k];
    if (!p_lawson_seq(V, vhe, live, nlive)) return;
    // the merged face may have been flipped away: start the walk from a
    // half-edge still leaving a link vertex
    near = vhe[p_origin(V, near)];
    bool ok = p_insert_seq(V, vhe, v, t, freed, near, link, &nlink);
    if (ok) {
      V.pos[v] = t;
      p_add(&V.cnt->reinserted, 1);
    } else {
      ok = p_insert_seq(V, vhe, v, here, freed, near, link, &nlink);
      if (!ok) {
        p_error(V, MCL_ERR_DEGENERATE_INPUT, 20);  // v could not go back either
        return;
      }
    }
    if (!p_lawson_seq(V, vhe, link, nlink)) return;
  }
}

// ---------------------------------------------------------------------------
// Removal and reinsertion in parallel rounds (the GPU step's last phase; the
// one-thread pass above is its serial counterpart).  The vertices still away
// from their targets go through removal rounds (each claims every face of its
// star; a winner, sharing no face with another, removes itself: spoke flips
// down to degree 3, then a merge) and then insertion rounds (each locates its
// target from a vertex that stays and claims the face, or the two faces of the
// side, holding it; a winner splits them).  A winner rewrites only its own
// faces and, field by field, its side of their edges, so winners of one round
// never touch the same field; every edge a round rewrote is queued once on a
// work-list (wl0, counted by *lq) from which flip rounds restore Delaunay.
// Per vertex: pf[3 v .. 3 v + 2] its three free edges, pa[v] a vertex that
// stays to start the walk from, ps[v] its state (kParPending ...).

constexpr int kParRounds = 256;  // removal or insertion rounds at most
enum : int { kParPending = 1, kParRemoved = 2, kParStays = 3, kParBack = 4, kParDone = 5 };

// the smallest half-edge of h's face: its claim slot
MCL_HD int p_face_min(const PView& V, int h) { return p_min(h, p_min(p_next(V, h), p_prev(V, h))); }
// claim key of vertex v in the round with stamp s: the smaller id wins (the
// order the one-thread pass takes them in)
MCL_HD unsigned long long p_vkey(int v, unsigned s) { return ((unsigned long long)s << 32) | (unsigned)(~(unsigned)v); }

// edge e onto the repair work-list, once for stamp s
MCL_HD void p_lqueue(const PView& V, unsigned long long* lq, int e, unsigned s) {
  if ((unsigned)e >= (unsigned)V.E) return;
  if (p_exch(V.qstamp + e, s) == s) return;
  V.wl0[p_inc(lq)] = e;
}

// v's star, by its outgoing half-edges from vhe[v]: f(h) for each; false (an
// error flagged) when the star does not close
template <typename F>
MCL_HD bool p_each_spoke(const PView& V, const int* vhe, int v, F f) {
  const unsigned H = 2u * (unsigned)V.E;
  const int h0 = vhe[v];
  if ((unsigned)h0 >= H || p_origin(V, h0) != v) {
    p_error(V, MCL_ERR_DEGENERATE_INPUT, 23);
    return false;
  }
  int h = h0, deg = 0;
  do {
    f(h);
    h = p_rot(V, h);
    ++deg;
  } while (h != h0 && (unsigned)h < H && deg < kPeriodicMaxDeg);
  if (h != h0) {
    p_error(V, MCL_ERR_DEGENERATE_INPUT, 24);
    return false;
  }
  return true;
}

// removal round, claims: every face of v's star
MCL_HD void p_body_claim_star(const PView& V, const int* vhe, int v, unsigned s) {
  const unsigned long long key = p_vkey(v, s);
  p_each_spoke(V, vhe, v, [&](int h) { p_max(V.claim + p_face_min(V, h), key); });
}

// removal round, verification (nothing is written meanwhile): v holds every
// claim of its star
MCL_HD bool p_body_holds_star(const PView& V, const int* vhe, int v, unsigned s) {
  const unsigned long long key = p_vkey(v, s);
  bool all = true;
  const bool ok = p_each_spoke(V, vhe, v, [&](int h) { all = all && V.claim[p_face_min(V, h)] == key; });
  return ok && all;
}

// removal round, a winner: v leaves the mesh (its free edges to pf, a
// neighbour that stays to pa, the hole's edges queued); a refused removal
// leaves v where it is (state kParStays) and queues the hole's edges and v's
// spokes, which its spoke flips may have left non-Delaunay
MCL_HD void p_body_remove_par(const PView& V, int* vhe, int v, int* pf, int* pa, int* ps, unsigned long long* lq,
                              unsigned s) {
  int freed[3], near = -1, hole[2 * kSeqStar], nhole = 0;
  // a neighbour that stays (not on the list), for the walk that reinserts v
  int stay = -1, any = -1;
  p_each_spoke(V, vhe, v, [&](int h) {
    const int w = p_origin(V, h ^ 1);
    if (any < 0) any = w;
    if (stay < 0 && ps[w] == 0) stay = w;
  });
  if (!p_remove_seq(V, vhe, v, freed, &near, hole, &nhole)) {
    ps[v] = kParStays;
    if (V.cnt->error) return;
    for (int k = 0; k < nhole; ++k) p_lqueue(V, lq, hole[k], s);
    p_each_spoke(V, vhe, v, [&](int h) { p_lqueue(V, lq, h >> 1, s); });
    return;
  }
  for (int k = 0; k < nhole; ++k)
    if (hole[k] != freed[0] && hole[k] != freed[1] && hole[k] != freed[2]) p_lqueue(V, lq, hole[k], s);
  pf[3 * v] = freed[0];
  pf[3 * v + 1] = freed[1];
  pf[3 * v + 2] = freed[2];
  pa[v] = stay >= 0 ? stay : any;
  ps[v] = kParRemoved;
}

// where v goes: its target, or (state kParBack: the target was taken) where it was
MCL_HD PF2 p_goal(const PView& V, int v, const int* ps) { return ps[v] == kParBack ? V.pos[v] : V.target[v]; }

// insertion round, location and claims (nothing is written but claims): the
// face of v's goal from the walk start (the face found last round, or a
// half-edge of v's neighbour that stays), into loc[v]; claims it, or the two
// faces of the side holding the goal; a goal on a corner (taken) is marked
// for the next round (-2 in loc)
MCL_HD void p_body_locate_par(const PView& V, const int* vhe, int v, const int* pa, int* loc, const int* ps,
                              unsigned s) {
  const unsigned H = 2u * (unsigned)V.E;
  int h = loc[v];
  if ((unsigned)h >= H) {
    const int a = pa[v];
    h = (unsigned)a < (unsigned)V.n ? vhe[a] : -1;
    for (int k = 1; (unsigned)h >= H && k <= V.n; ++k) h = vhe[(v + k) % V.n];  // any vertex in the mesh
  }
  int face = -1;
  bool vertex = false;
  if (!p_locate_face(V, p_goal(V, v, ps), h, &face, &vertex)) {
    loc[v] = -1;
    return;
  }
  if (vertex) {
    loc[v] = -2;
    return;
  }
  loc[v] = face;
  const unsigned long long key = p_vkey(v, s);
  p_max(V.claim + p_face_min(V, face), key);
  // a goal on a side also claims the face across it (the orientations of the
  // split decide which side; claiming across all three sides is enough and
  // costs two more claims at most)
  const PF2 t = p_goal(V, v, ps);
  const int a = p_origin(V, face), b = p_origin(V, face ^ 1), c = p_apex(V, face);
  const Off Ob = p_tof(V, face), Oc = p_xof(V, face);
  const PF2 qa = V.pos[a], qb = off_translate(V.pos[b], Ob, V.L), qc = off_translate(V.pos[c], Oc, V.L);
  Off K;
  const PF2 pt = p_nearest_copy(t, qa, V.L, K);
  const int sides[3] = {face, p_next(V, face), p_prev(V, face)};
  const int o[3] = {p_orient_at(V, qa, qb, pt), p_orient_at(V, qb, qc, pt), p_orient_at(V, qc, qa, pt)};
  for (int k = 0; k < 3; ++k)
    if (o[k] == 0) p_max(V.claim + p_face_min(V, sides[k] ^ 1), key);
}

// insertion round, verification (nothing is written meanwhile): v holds the
// claims of its face and of the face across a side holding its goal
MCL_HD bool p_body_holds_face(const PView& V, int v, const int* loc, const int* ps, unsigned s) {
  const int face = loc[v];
  if (face < 0) return false;
  const unsigned long long key = p_vkey(v, s);
  if (V.claim[p_face_min(V, face)] != key) return false;
  const PF2 t = p_goal(V, v, ps);
  const int a = p_origin(V, face), b = p_origin(V, face ^ 1), c = p_apex(V, face);
  const Off Ob = p_tof(V, face), Oc = p_xof(V, face);
  const PF2 qa = V.pos[a], qb = off_translate(V.pos[b], Ob, V.L), qc = off_translate(V.pos[c], Oc, V.L);
  Off K;
  const PF2 pt = p_nearest_copy(t, qa, V.L, K);
  const int sides[3] = {face, p_next(V, face), p_prev(V, face)};
  const int o[3] = {p_orient_at(V, qa, qb, pt), p_orient_at(V, qb, qc, pt), p_orient_at(V, qc, qa, pt)};
  for (int k = 0; k < 3; ++k)
    if (o[k] == 0 && V.claim[p_face_min(V, sides[k] ^ 1)] != key) return false;
  return true;
}

// insertion round, a winner: v splits its face (or the two faces of its side)
// at its goal; the new star's link and spokes queued
MCL_HD bool p_body_split_par(const PView& V, int* vhe, int v, const int* pf, const int* loc, int* ps,
                             unsigned long long* lq, unsigned s) {
  const int f[3] = {pf[3 * v], pf[3 * v + 1], pf[3 * v + 2]};
  const bool back = ps[v] == kParBack;
  const PF2 t = p_goal(V, v, ps);
  int link[4], nlink = 0;
  if (!p_split_at(V, vhe, v, t, f, loc[v], link, &nlink)) {
    p_error(V, MCL_ERR_DEGENERATE_INPUT, 25);  // located inside this face, the split must succeed
    return false;
  }
  if (!back) {
    V.pos[v] = t;
    p_add(&V.cnt->reinserted, 1);
  }
  ps[v] = kParDone;
  for (int k = 0; k < nlink; ++k) p_lqueue(V, lq, link[k] >> 1, s);
  for (int k = 0; k < 3; ++k) p_lqueue(V, lq, f[k], s);
  return true;
}

// ---------------------------------------------------------------------------
// Queries on a periodic mesh.

// half-edge h: a candidate for its origin's outgoing half-edge; the largest
// id wins (vhe starts at -1), so every run picks the same one
MCL_HD void p_body_vhe(const PView& V, int* vhe, int h) {
  const PI4 q = V.ev[h >> 1];
  const int o = (h & 1) ? q.y : q.x;
  if ((unsigned)o >= (unsigned)V.n) {
    p_error(V, MCL_ERR_DEGENERATE_INPUT, 6);
    return;
  }
#if defined(__CUDA_ARCH__)
  atomicMax(vhe + o, h);
#else
  if (h > vhe[o]) vhe[o] = h;
#endif
}

// neighbour key for the ring's start: smallest id, then smallest offset byte
MCL_HD long long p_ring_key(int id, unsigned off) { return ((long long)id << 8) | off; }

// vertex v: its neighbours clockwise, starting at the smallest (id, offset),
// at most max_ring - 1 of them; slot 0 holds the count (the reference's ring
// layout, include/kernels.cuh:54-84).  offs (may be null) receives, in the same
// layout, each neighbour's copy offset relative to v (an offset byte).
MCL_HD void p_body_ring(const PView& V, const int* vhe, int v, bool column, int max_ring, int* ring,
                        unsigned char* offs) {
  const int h0 = vhe[v];
  const unsigned H = 2u * (unsigned)V.E;
  if ((unsigned)h0 >= H || p_origin(V, h0) != v) {
    p_error(V, MCL_ERR_DEGENERATE_INPUT, 7);
    return;
  }
  const size_t stride = column ? (size_t)V.n : 1;
  int* row = column ? ring + v : ring + (size_t)v * max_ring;
  unsigned char* orow = offs ? (column ? offs + v : offs + (size_t)v * max_ring) : nullptr;
  int start = h0, deg = 0, h = h0;
  long long best = 0;
  do {
    const int nb = p_origin(V, h ^ 1);
    const unsigned ob = off_byte(eo_target(V.eo[h >> 1], h & 1));
    const long long key = p_ring_key(nb, ob);
    if (deg == 0 || key < best) {
      best = key;
      start = h;
    }
    h = p_rot(V, h);
    ++deg;
    if ((unsigned)h >= H) {
      p_error(V, MCL_ERR_DEGENERATE_INPUT, 8);
      return;
    }
  } while (h != h0 && deg < kPeriodicMaxDeg);
  if (h != h0) {
    p_error(V, MCL_ERR_DEGENERATE_INPUT, 9);
    return;
  }
  const int cap = max_ring - 1;
  const int cnt = deg < cap ? deg : cap;
  h = start;
  for (int k = 0; k < cnt; ++k) {
    row[(size_t)(k + 1) * stride] = p_origin(V, h ^ 1);
    if (orow) orow[(size_t)(k + 1) * stride] = (unsigned char)off_byte(eo_target(V.eo[h >> 1], h & 1));
    h = p_rot(V, h);
  }
  row[0] = cnt;
  if (orow) orow[0] = 0;
  if (deg > cap) p_add(&V.cnt->truncated, 1);
}

// vertex v: the ring neighbour nearest to v on the torus (smallest id among
// equals), by the reference's float squared distance (include/kernels.cuh:125-127)
// between v and the neighbour's copy; -1 for an empty ring.
MCL_HD void p_body_closest(const PView& V, int v, bool column, int max_ring, const int* ring,
                           const unsigned char* offs, int* out) {
  const int cnt = column ? ring[v] : ring[(size_t)v * max_ring];
  const PF2 p = V.pos[v];
  int best = -1;
  float bd = 0.f;
  for (int k = 0; k < cnt && k < max_ring - 1; ++k) {
    const size_t at = column ? (size_t)(k + 1) * V.n + v : (size_t)v * max_ring + k + 1;
    const int j = ring[at];
    if ((unsigned)j >= (unsigned)V.n) continue;
    const PF2 q = off_translate(V.pos[j], off_from_byte(offs[at]), V.L);
    const float dx = fsub(p.x, q.x), dy = fsub(p.y, q.y);
    const float d = fadd(fmul(dx, dx), fmul(dy, dy));
    if (best < 0 || d < bd || (d == bd && j < best)) {
      best = j;
      bd = d;
    }
  }
  out[v] = best;
}

constexpr int kPeriodicFrnnLocal = 256;

// vertex i: every other vertex with a copy within r of i (r < L / 2, so at
// most one copy of each), found by a search over the mesh from i through the
// vertices already found (the reference's getFRNN, include/kernels.cuh:169-219,
// on the torus); written by ascending id, slot 0 the count, at most
// max_frnn - 1 of them; offs (may be null) gets each one's copy offset byte.
MCL_HD void p_body_frnn(const PView& V, const int* vhe, int i, float r2, bool column, int max_frnn, int* out,
                        unsigned char* offs) {
  int fid[kPeriodicFrnnLocal];
  unsigned char foff[kPeriodicFrnnLocal];
  int nf = 0, top = 0;
  bool over = false;
  const unsigned H = 2u * (unsigned)V.E;
  const PF2 pi = V.pos[i];
  int cur = i;
  Off ocur{0, 0};
  for (int guard = 0; guard < (1 << 20); ++guard) {
    const int h0 = vhe[cur];
    if ((unsigned)h0 < H) {
      int h = h0, deg = 0;
      do {
        const int w = p_origin(V, h ^ 1);
        const Off ow = off_add(ocur, eo_target(V.eo[h >> 1], h & 1));
        if (w != i && (unsigned)w < (unsigned)V.n && off_small(ow)) {
          bool seen = false;
          for (int k = 0; k < nf; ++k)
            if (fid[k] == w) {
              seen = true;
              break;
            }
          if (!seen) {
            const PF2 q = off_translate(V.pos[w], ow, V.L);
            const float dx = fsub(pi.x, q.x), dy = fsub(pi.y, q.y);
            if (fadd(fmul(dx, dx), fmul(dy, dy)) <= r2) {
              if (nf < kPeriodicFrnnLocal) {
                fid[nf] = w;
                foff[nf] = (unsigned char)off_byte(ow);
                ++nf;
              } else {
                over = true;
              }
            }
          }
        }
        h = p_rot(V, h);
        ++deg;
        if ((unsigned)h >= H) {
          p_error(V, MCL_ERR_DEGENERATE_INPUT, 10);
          return;
        }
      } while (h != h0 && deg < kPeriodicMaxDeg);
    }
    if (top >= nf) break;
    cur = fid[top];
    ocur = off_from_byte(foff[top]);
    ++top;
  }
  for (int a = 1; a < nf; ++a) {  // insertion sort by id
    const int x = fid[a];
    const unsigned char xo = foff[a];
    int b = a - 1;
    while (b >= 0 && fid[b] > x) {
      fid[b + 1] = fid[b];
      foff[b + 1] = foff[b];
      --b;
    }
    fid[b + 1] = x;
    foff[b + 1] = xo;
  }
  const int cap = max_frnn - 1;
  const int cnt = nf < cap ? nf : cap;
  const size_t stride = column ? (size_t)V.n : 1;
  int* row = column ? out + i : out + (size_t)i * max_frnn;
  unsigned char* orow = offs ? (column ? offs + i : offs + (size_t)i * max_frnn) : nullptr;
  for (int k = 0; k < cnt; ++k) {
    row[(size_t)(k + 1) * stride] = fid[k];
    if (orow) orow[(size_t)(k + 1) * stride] = foff[k];
  }
  row[0] = cnt;
  if (orow) orow[0] = 0;
  if (over || nf > cap) p_add(&V.cnt->truncated, 1);
}

}  // namespace mcl
