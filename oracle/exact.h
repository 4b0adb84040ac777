// Oracle exact geometric predicates (test infrastructure only).
//
// This file is part of the CPU oracle that checks the GPU engine; nothing in
// the shipped library includes it.  Signs are computed in two stages:
//   1. a double-precision evaluation with Shewchuk's stage-A forward error
//      bounds (Shewchuk 1997, "Adaptive Precision Floating-Point Arithmetic and
//      Fast Robust Geometric Predicates", constants ccwerrboundA and
//      iccerrboundA);
//   2. when the filter cannot decide, an exact evaluation with arbitrary
//      precision integers: every float input is m * 2^e, all inputs of one call
//      are rescaled to integers on a common exponent and the determinant is
//      evaluated with exact big-integer arithmetic.
// Stage 2 is a different method from the GPU's expansion arithmetic on purpose,
// so the two implementations check each other.
//
// Sign conventions follow the reference (include/Helpers_Triangulation.h:86-151):
//   orient2d(a,b,c) > 0  iff  a,b,c are counter-clockwise;
//   incircle(a,b,c,d) > 0 iff d lies inside the circle through CCW a,b,c.
#pragma once
#include <cstdint>

namespace oracle {

struct P2 { float x, y; };

// Exact sign of orient2d(a,b,c): -1, 0, +1.
int orient2d_exact(P2 a, P2 b, P2 c);
// Exact sign of incircle(a,b,c,d): -1, 0, +1.
int incircle_exact(P2 a, P2 b, P2 c, P2 d);
// Incircle with symbolic perturbation (never 0 for a quad whose two triangles
// have non-zero area).  Each point's paraboloid lift z = x^2+y^2 is raised by an
// infinitesimal delta(id), with delta(i) >> delta(j) whenever i < j.  When the
// exact 4x4 lifted determinant is 0 the sign is that of the first non-zero
// cofactor of the z column, taken in ascending vertex-id order:
//   C_a = +orient(b,c,d), C_b = -orient(a,c,d), C_c = +orient(a,b,d),
//   C_d = -orient(a,b,c).
int incircle_sos(P2 a, P2 b, P2 c, P2 d, int ia, int ib, int ic, int id);

// Reference-style FP64 predicates, restated from
// include/Helpers_Triangulation.h:86-122 (orient2d) and :136-151 (inCircle):
// double evaluation from float inputs, |det| < EPS(=1e-17f) -> 0.  These are
// what the reference's HostTriangulation uses (with abs bound to double).
int orient2d_ref(P2 a, P2 b, P2 c);
int incircle_ref(P2 a, P2 b, P2 c, P2 d);

// Counters of how often stage 2 was needed (for reporting).
struct ExactStats { uint64_t orient_calls, orient_exact, incircle_calls, incircle_exact, sos_used; };
ExactStats exact_stats();
void exact_stats_reset();

}  // namespace oracle
