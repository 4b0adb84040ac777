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
// rewrite the apex offset of a wing half-edge with a byte store, and a wrap of
// a vertex updates offsets with one signed atomic add per edge (the bias keeps
// every nibble in 0..15, so no borrow crosses a field).
//
// Exact translates: with positions in [2L, 3L), x + L stays in the binade
// [2L, 4L) and x - L lands in [L, 2L), whose grid is finer, so every
// translated coordinate the predicates see is an exact float and the
// FP32-filter / exact ladder applies unchanged.  The lifted-perturbation
// incircle (ids ascending) is invariant under translation, so the copies of a
// vertex are perturbed alike.
#pragma once

#include "predicates.cuh"

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
// the results for every role a wrapped vertex holds (in any order, with
// atomicAdd on the GPU) gives B' = B + w_b - w_a, C' = C + w_c - w_a,
// X1' = X1 + w_d - w_b.
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

}  // namespace mcl
