// Geometric predicates for float32 points: a three-stage ladder.
//
//   stage 1  FP32 evaluation with a static forward-error filter;
//   stage 2  FP64 evaluation of the same expression with its bound;
//   stage 3  exact expansion arithmetic on the double images of the inputs.
//
// The filters are Shewchuk's stage-A bounds (J. R. Shewchuk, "Adaptive
// Precision Floating-Point Arithmetic and Fast Robust Geometric Predicates",
// Discrete Comput. Geom. 18, 1997, sec. 4): orient2d |det| >= (3+16e)e*detsum,
// incircle |det| > (10+96e)e*permanent, with e = 2^-24 for float and 2^-53 for
// double.  Both stages evaluate the expression in exactly the order the bound
// was derived for, with explicitly rounded operations (no FMA contraction).
// Stage 3 uses the paper's expansion algorithms (Two-Sum, Two-Product via FMA,
// Grow-Expansion, Scale-Expansion, Compress) with fixed-capacity arrays; a
// capacity overflow is reported through the `overflow` flag, never silently.
//
// Sign conventions are the reference's (include/Helpers_Triangulation.h:86-151):
// orient2d(a,b,c) > 0 iff a,b,c counter-clockwise; incircle(a,b,c,d) > 0 iff d
// lies inside the circle through counter-clockwise a,b,c.
//
// incircle_sos adds symbolic perturbation: each point's lift x^2+y^2 is raised
// by an infinitesimal that is larger for smaller vertex ids; an exactly
// cocircular quad is then decided by the first non-zero cofactor of the lift
// column of the 4x4 lifted determinant, in ascending id order:
//   C_a = +orient(b,c,d), C_b = -orient(a,c,d), C_c = +orient(a,b,d), C_d = -orient(a,b,c).
// This makes the Delaunay triangulation unique for every input, so the GPU's
// edge set can be compared bit for bit with the oracle's.
//
// Everything here compiles for host and device so the CPU test suite can run
// the same code against golden vectors.
#pragma once

#include <cstdint>
#include <cmath>

#ifdef __CUDACC__
#define MCL_HD __host__ __device__ __forceinline__
#define MCL_HD_NOINLINE static __host__ __device__ __noinline__
#else
#define MCL_HD inline
#define MCL_HD_NOINLINE static
#endif

namespace mcl {

#if defined(__CUDA_ARCH__)
MCL_HD float fadd(float a, float b) { return __fadd_rn(a, b); }
MCL_HD float fsub(float a, float b) { return __fsub_rn(a, b); }
MCL_HD float fmul(float a, float b) { return __fmul_rn(a, b); }
MCL_HD double dadd(double a, double b) { return __dadd_rn(a, b); }
MCL_HD double dsub(double a, double b) { return __dsub_rn(a, b); }
MCL_HD double dmul(double a, double b) { return __dmul_rn(a, b); }
MCL_HD double dfma(double a, double b, double c) { return __fma_rn(a, b, c); }
#else
// Host build is compiled with -ffp-contract=off, so these are single roundings.
MCL_HD float fadd(float a, float b) { return a + b; }
MCL_HD float fsub(float a, float b) { return a - b; }
MCL_HD float fmul(float a, float b) { return a * b; }
MCL_HD double dadd(double a, double b) { return a + b; }
MCL_HD double dsub(double a, double b) { return a - b; }
MCL_HD double dmul(double a, double b) { return a * b; }
MCL_HD double dfma(double a, double b, double c) { return std::fma(a, b, c); }
#endif

struct PredCounters {
  // incremented only on the slow stages (the fast stage is counted by callers)
  unsigned long long orient_fp64, orient_exact, incircle_fp64, incircle_exact, sos, overflow;
};

// ---------------------------------------------------------------------------
// Expansion arithmetic (nonoverlapping expansions, increasing magnitude).
constexpr int kExpCap = 64;

struct Exp {
  int n;
  double c[kExpCap];
};

MCL_HD void two_sum(double a, double b, double& x, double& y) {
  x = dadd(a, b);
  double bv = dsub(x, a);
  double av = dsub(x, bv);
  double br = dsub(b, bv);
  double ar = dsub(a, av);
  y = dadd(ar, br);
}

MCL_HD void fast_two_sum(double a, double b, double& x, double& y) {  // |a| >= |b|
  x = dadd(a, b);
  double bv = dsub(x, a);
  y = dsub(b, bv);
}

MCL_HD void two_prod(double a, double b, double& x, double& y) {
  x = dmul(a, b);
  y = dfma(a, b, -x);
}

// h = e + b  (Grow-Expansion with zero elimination); h may alias e.
MCL_HD bool grow(const Exp& e, double b, Exp& h) {
  double q = b, hh;
  int k = 0;
  const int n = e.n;
  for (int i = 0; i < n; ++i) {
    double qn;
    two_sum(q, e.c[i], qn, hh);
    q = qn;
    if (hh != 0.0) {
      if (k >= kExpCap) return false;
      h.c[k++] = hh;
    }
  }
  if (q != 0.0 || k == 0) {
    if (k >= kExpCap) return false;
    h.c[k++] = q;
  }
  h.n = k;
  return true;
}

// h = e + f by repeated Grow-Expansion; h must not alias f.
MCL_HD bool exp_add(const Exp& e, const Exp& f, Exp& h) {
  if (&h != &e) {
    h.n = e.n;
    for (int i = 0; i < e.n; ++i) h.c[i] = e.c[i];
  }
  for (int j = 0; j < f.n; ++j)
    if (!grow(h, f.c[j], h)) return false;
  return true;
}

MCL_HD void exp_neg(Exp& e) {
  for (int i = 0; i < e.n; ++i) e.c[i] = -e.c[i];
}

// h = e * b (Scale-Expansion with zero elimination); h must not alias e.
MCL_HD bool exp_scale(const Exp& e, double b, Exp& h) {
  int k = 0;
  double q, hh;
  if (e.n == 0 || b == 0.0) { h.n = 1; h.c[0] = 0.0; return true; }
  two_prod(e.c[0], b, q, hh);
  if (hh != 0.0) h.c[k++] = hh;
  for (int i = 1; i < e.n; ++i) {
    double p1, p0, s;
    two_prod(e.c[i], b, p1, p0);
    two_sum(q, p0, s, hh);
    if (hh != 0.0) { if (k >= kExpCap) return false; h.c[k++] = hh; }
    fast_two_sum(p1, s, q, hh);
    if (hh != 0.0) { if (k >= kExpCap) return false; h.c[k++] = hh; }
  }
  if (q != 0.0 || k == 0) { if (k >= kExpCap) return false; h.c[k++] = q; }
  h.n = k;
  return true;
}

// Compress (Shewchuk 1997, sec. 2.8) in place.
MCL_HD void exp_compress(Exp& e) {
  if (e.n <= 1) return;
  double g[kExpCap];
  int bottom = e.n - 1;
  double q = e.c[bottom];
  for (int i = e.n - 2; i >= 0; --i) {
    double qn, r;
    fast_two_sum(q, e.c[i], qn, r);
    if (r != 0.0) { g[bottom--] = qn; q = r; }
    else q = qn;
  }
  g[bottom] = q;
  int top = 0;
  q = g[bottom];
  for (int i = bottom + 1; i < e.n; ++i) {
    double qn, r;
    fast_two_sum(g[i], q, qn, r);
    if (r != 0.0) e.c[top++] = r;
    q = qn;
  }
  e.c[top++] = q;
  e.n = top;
}

// h = e * f, compressing the running sum after every partial product.
MCL_HD bool exp_mul(const Exp& e, const Exp& f, Exp& h, Exp& tmp) {
  h.n = 1;
  h.c[0] = 0.0;
  for (int j = 0; j < f.n; ++j) {
    if (!exp_scale(e, f.c[j], tmp)) return false;
    if (!exp_add(h, tmp, h)) return false;
    exp_compress(h);
  }
  return true;
}

MCL_HD int exp_sign(const Exp& e) {
  for (int i = e.n - 1; i >= 0; --i)
    if (e.c[i] != 0.0) return e.c[i] > 0 ? 1 : -1;
  return 0;
}

MCL_HD void exp_diff(double a, double b, Exp& h) {  // exact a - b
  double x, y;
  two_sum(a, -b, x, y);
  int k = 0;
  if (y != 0.0) h.c[k++] = y;
  if (x != 0.0 || k == 0) h.c[k++] = x;
  h.n = k;
}

// ---------------------------------------------------------------------------
// Exact stage.  Returns the sign; sets *overflow on capacity exhaustion.
MCL_HD_NOINLINE int orient2d_exact_exp(float ax, float ay, float bx, float by, float cx, float cy,
                                       int* overflow) {
  Exp acx, bcy, acy, bcx, l, r, t;
  exp_diff(ax, cx, acx);
  exp_diff(by, cy, bcy);
  exp_diff(ay, cy, acy);
  exp_diff(bx, cx, bcx);
  bool ok = exp_mul(acx, bcy, l, t) && exp_mul(acy, bcx, r, t);
  if (ok) {
    exp_neg(r);
    ok = exp_add(l, r, l);
  }
  if (!ok) { *overflow = 1; return 0; }
  return exp_sign(l);
}

MCL_HD_NOINLINE int incircle_exact_exp(float ax, float ay, float bx, float by, float cx, float cy,
                                       float dx, float dy, int* overflow) {
  Exp adx, ady, bdx, bdy, cdx, cdy, lift, cr, t1, t2, acc;
  exp_diff(ax, dx, adx);
  exp_diff(ay, dy, ady);
  exp_diff(bx, dx, bdx);
  exp_diff(by, dy, bdy);
  exp_diff(cx, dx, cdx);
  exp_diff(cy, dy, cdy);
  acc.n = 1;
  acc.c[0] = 0.0;
  // det = alift*(bdx*cdy - bdy*cdx) + blift*(cdx*ady - cdy*adx) + clift*(adx*bdy - ady*bdx)
  const Exp* X[3] = {&adx, &bdx, &cdx};
  const Exp* Y[3] = {&ady, &bdy, &cdy};
  for (int k = 0; k < 3; ++k) {
    const Exp& px = *X[k];
    const Exp& py = *Y[k];
    const Exp& qx = *X[(k + 1) % 3];
    const Exp& qy = *Y[(k + 1) % 3];
    const Exp& rx = *X[(k + 2) % 3];
    const Exp& ry = *Y[(k + 2) % 3];
    // lift = px^2 + py^2
    if (!exp_mul(px, px, lift, t2) || !exp_mul(py, py, t1, t2) || !exp_add(lift, t1, lift)) {
      *overflow = 1;
      return 0;
    }
    exp_compress(lift);
    // cross = qx*ry - qy*rx
    if (!exp_mul(qx, ry, cr, t2) || !exp_mul(qy, rx, t1, t2)) { *overflow = 1; return 0; }
    exp_neg(t1);
    if (!exp_add(cr, t1, cr)) { *overflow = 1; return 0; }
    exp_compress(cr);
    if (!exp_mul(lift, cr, t1, t2) || !exp_add(acc, t1, acc)) { *overflow = 1; return 0; }
    exp_compress(acc);
  }
  return exp_sign(acc);
}

// ---------------------------------------------------------------------------
// FP32 / FP64 filtered stages.
constexpr float kEpsF = 5.9604644775390625e-08f;          // 2^-24
constexpr double kEpsD = 1.1102230246251565404236316680908203125e-16;  // 2^-53
constexpr float kCcwErrF = (3.0f + 16.0f * kEpsF) * kEpsF;
constexpr float kIccErrF = (10.0f + 96.0f * kEpsF) * kEpsF;
constexpr double kCcwErrD = (3.0 + 16.0 * kEpsD) * kEpsD;
constexpr double kIccErrD = (10.0 + 96.0 * kEpsD) * kEpsD;
// Below these magnitudes the float / double bounds could be spoiled by underflow.
constexpr float kTinyF = 1e-30f;
constexpr double kTinyD = 1e-250;

// Returns 2 when undecided.
MCL_HD int orient2d_fp32(float ax, float ay, float bx, float by, float cx, float cy) {
  const float detleft = fmul(fsub(ax, cx), fsub(by, cy));
  const float detright = fmul(fsub(ay, cy), fsub(bx, cx));
  const float det = fsub(detleft, detright);
  float detsum;
  if (detleft > 0.0f) {
    if (detright <= 0.0f) return det > 0.0f ? 1 : (det < 0.0f ? -1 : 2);
    detsum = fadd(detleft, detright);
  } else if (detleft < 0.0f) {
    if (detright >= 0.0f) return det > 0.0f ? 1 : (det < 0.0f ? -1 : 2);
    detsum = fsub(-detleft, detright);
  } else {
    detsum = fabsf(detright);
  }
  if (!(detsum > kTinyF) || !(detsum < 1e37f)) return 2;
  const float err = fmul(kCcwErrF, detsum);
  if (det >= err || -det >= err) return det > 0.0f ? 1 : (det < 0.0f ? -1 : 2);
  return 2;
}

MCL_HD int orient2d_fp64(float ax, float ay, float bx, float by, float cx, float cy) {
  const double detleft = dmul(dsub(ax, cx), dsub(by, cy));
  const double detright = dmul(dsub(ay, cy), dsub(bx, cx));
  const double det = dsub(detleft, detright);
  double detsum;
  if (detleft > 0.0) {
    if (detright <= 0.0) return det > 0.0 ? 1 : (det < 0.0 ? -1 : 2);
    detsum = dadd(detleft, detright);
  } else if (detleft < 0.0) {
    if (detright >= 0.0) return det > 0.0 ? 1 : (det < 0.0 ? -1 : 2);
    detsum = dsub(-detleft, detright);
  } else {
    detsum = fabs(detright);
  }
  if (!(detsum > kTinyD)) return 2;
  const double err = dmul(kCcwErrD, detsum);
  if (det >= err || -det >= err) return det > 0.0 ? 1 : (det < 0.0 ? -1 : 2);
  return 2;
}

MCL_HD int incircle_fp32(float ax, float ay, float bx, float by, float cx, float cy, float dx,
                         float dy) {
  const float adx = fsub(ax, dx), bdx = fsub(bx, dx), cdx = fsub(cx, dx);
  const float ady = fsub(ay, dy), bdy = fsub(by, dy), cdy = fsub(cy, dy);
  const float bdxcdy = fmul(bdx, cdy), cdxbdy = fmul(cdx, bdy);
  const float alift = fadd(fmul(adx, adx), fmul(ady, ady));
  const float cdxady = fmul(cdx, ady), adxcdy = fmul(adx, cdy);
  const float blift = fadd(fmul(bdx, bdx), fmul(bdy, bdy));
  const float adxbdy = fmul(adx, bdy), bdxady = fmul(bdx, ady);
  const float clift = fadd(fmul(cdx, cdx), fmul(cdy, cdy));
  const float det = fadd(fadd(fmul(alift, fsub(bdxcdy, cdxbdy)), fmul(blift, fsub(cdxady, adxcdy))),
                         fmul(clift, fsub(adxbdy, bdxady)));
  const float perm = fadd(fadd(fmul(fadd(fabsf(bdxcdy), fabsf(cdxbdy)), alift),
                               fmul(fadd(fabsf(cdxady), fabsf(adxcdy)), blift)),
                          fmul(fadd(fabsf(adxbdy), fabsf(bdxady)), clift));
  if (!(perm > kTinyF) || !(perm < 1e37f)) return 2;
  const float err = fmul(kIccErrF, perm);
  if (det > err || -det > err) return det > 0.0f ? 1 : -1;
  return 2;
}

MCL_HD int incircle_fp64(float ax, float ay, float bx, float by, float cx, float cy, float dx,
                         float dy) {
  const double adx = dsub(ax, dx), bdx = dsub(bx, dx), cdx = dsub(cx, dx);
  const double ady = dsub(ay, dy), bdy = dsub(by, dy), cdy = dsub(cy, dy);
  const double bdxcdy = dmul(bdx, cdy), cdxbdy = dmul(cdx, bdy);
  const double alift = dadd(dmul(adx, adx), dmul(ady, ady));
  const double cdxady = dmul(cdx, ady), adxcdy = dmul(adx, cdy);
  const double blift = dadd(dmul(bdx, bdx), dmul(bdy, bdy));
  const double adxbdy = dmul(adx, bdy), bdxady = dmul(bdx, ady);
  const double clift = dadd(dmul(cdx, cdx), dmul(cdy, cdy));
  const double det = dadd(dadd(dmul(alift, dsub(bdxcdy, cdxbdy)), dmul(blift, dsub(cdxady, adxcdy))),
                          dmul(clift, dsub(adxbdy, bdxady)));
  const double perm = dadd(dadd(dmul(dadd(fabs(bdxcdy), fabs(cdxbdy)), alift),
                                dmul(dadd(fabs(cdxady), fabs(adxcdy)), blift)),
                           dmul(dadd(fabs(adxbdy), fabs(bdxady)), clift));
  if (!(perm > kTinyD)) return 2;
  const double err = dmul(kIccErrD, perm);
  if (det > err || -det > err) return det > 0.0 ? 1 : -1;
  return 2;
}

// ---------------------------------------------------------------------------
// Full ladders.  `cnt` may be null.
template <typename Counters>
MCL_HD int orient2d(float ax, float ay, float bx, float by, float cx, float cy, Counters* cnt,
                    int* overflow) {
  int s = orient2d_fp32(ax, ay, bx, by, cx, cy);
  if (s != 2) return s;
  if (cnt) cnt->orient_fp64++;
  s = orient2d_fp64(ax, ay, bx, by, cx, cy);
  if (s != 2) return s;
  if (cnt) cnt->orient_exact++;
  return orient2d_exact_exp(ax, ay, bx, by, cx, cy, overflow);
}

template <typename Counters>
MCL_HD int incircle(float ax, float ay, float bx, float by, float cx, float cy, float dx, float dy,
                    Counters* cnt, int* overflow) {
  int s = incircle_fp32(ax, ay, bx, by, cx, cy, dx, dy);
  if (s != 2) return s;
  if (cnt) cnt->incircle_fp64++;
  s = incircle_fp64(ax, ay, bx, by, cx, cy, dx, dy);
  if (s != 2) return s;
  if (cnt) cnt->incircle_exact++;
  return incircle_exact_exp(ax, ay, bx, by, cx, cy, dx, dy, overflow);
}

template <typename Counters>
MCL_HD int incircle_sos(float ax, float ay, float bx, float by, float cx, float cy, float dx,
                        float dy, int ia, int ib, int ic, int id, Counters* cnt, int* overflow) {
  int s = incircle(ax, ay, bx, by, cx, cy, dx, dy, cnt, overflow);
  if (s != 0) return s;
  if (cnt) cnt->sos++;
  // visit a, b, c, d in ascending id order
  int ids[4] = {ia, ib, ic, id};
  int ord[4] = {0, 1, 2, 3};
  for (int i = 1; i < 4; ++i)
    for (int j = i; j > 0 && ids[ord[j]] < ids[ord[j - 1]]; --j) {
      int tmp = ord[j]; ord[j] = ord[j - 1]; ord[j - 1] = tmp;
    }
  for (int k = 0; k < 4; ++k) {
    int c0 = 0;
    switch (ord[k]) {
      case 0: c0 = orient2d(bx, by, cx, cy, dx, dy, cnt, overflow); break;
      case 1: c0 = -orient2d(ax, ay, cx, cy, dx, dy, cnt, overflow); break;
      case 2: c0 = orient2d(ax, ay, bx, by, dx, dy, cnt, overflow); break;
      default: c0 = -orient2d(ax, ay, bx, by, cx, cy, cnt, overflow); break;
    }
    if (c0 != 0) return c0;
  }
  return 0;
}

}  // namespace mcl
