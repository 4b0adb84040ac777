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
#include <cstring>

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
// Exact stage.  Returns the sign, or kExpOverflow when the expansion capacity
// was exhausted.  (No pointer arguments: callers keep their state in registers.)
constexpr int kExpOverflow = 3;

MCL_HD_NOINLINE int orient2d_exact_exp(float ax, float ay, float bx, float by, float cx, float cy) {
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
  if (!ok) return kExpOverflow;
  return exp_sign(l);
}

MCL_HD_NOINLINE int incircle_exact_exp(float ax, float ay, float bx, float by, float cx, float cy,
                                       float dx, float dy) {
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
    if (!exp_mul(px, px, lift, t2) || !exp_mul(py, py, t1, t2) || !exp_add(lift, t1, lift)) return kExpOverflow;
    exp_compress(lift);
    // cross = qx*ry - qy*rx
    if (!exp_mul(qx, ry, cr, t2) || !exp_mul(qy, rx, t1, t2)) return kExpOverflow;
    exp_neg(t1);
    if (!exp_add(cr, t1, cr)) return kExpOverflow;
    exp_compress(cr);
    if (!exp_mul(lift, cr, t1, t2) || !exp_add(acc, t1, acc)) return kExpOverflow;
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
// Branch-free form of the stage-A test: |det| >= (3+16e)e (|detleft|+|detright|).
// (When detleft and detright differ in sign, |det| ~ detsum and the test
// passes, which is the case Shewchuk's early exits handle.)
MCL_HD int orient2d_fp32(float ax, float ay, float bx, float by, float cx, float cy) {
  const float detleft = fmul(fsub(ax, cx), fsub(by, cy));
  const float detright = fmul(fsub(ay, cy), fsub(bx, cx));
  const float det = fsub(detleft, detright);
  const float detsum = fadd(fabsf(detleft), fabsf(detright));
  const float err = fmul(kCcwErrF, detsum);
  const bool ok = (detsum > kTinyF) & (detsum < 1e37f);
  const int s = det > err ? 1 : (-det > err ? -1 : 2);
  return ok ? s : 2;
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
// Exact stage on integers.  Every float32 is an integer mantissa times a power
// of two; after stripping trailing zero bits and aligning all coordinates of a
// call to their smallest exponent, each coordinate is an integer of at most
// 62 bits whenever the exponents span no more than ~38 binary orders (all
// coordinates of one quad in practice, including the +-1e7 corners).  The
// determinants are then evaluated exactly in 64-, 128- and 256-bit integer
// arithmetic - no floating point, which on this GPU (FP64 at a small fraction
// of FP32 / INT32 throughput) is much faster than the FP64 stage.  Returns
// false when the coordinates do not fit; the caller then falls back to the
// FP64 filter and the expansion arithmetic.
typedef unsigned long long u64;
typedef unsigned __int128 u128;
typedef __int128 i128;

MCL_HD unsigned f32_bits(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  unsigned u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}

MCL_HD int ctz32(unsigned x) {
#if defined(__CUDA_ARCH__)
  return __ffs(x) - 1;
#else
  return __builtin_ctz(x);
#endif
}

MCL_HD int clz64(u64 x) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

template <int N>
MCL_HD bool to_fixed(const float (&v)[N], long long (&X)[N]) {
  int e[N];
  long long m[N];
  int emin = 1 << 30;
  for (int i = 0; i < N; ++i) {
    const unsigned b = f32_bits(v[i]);
    const unsigned ex = (b >> 23) & 0xFF;
    unsigned mant = b & 0x7FFFFF;
    int exp2;
    if (ex == 0xFF) return false;  // inf / nan
    if (ex == 0) exp2 = -149;
    else { mant |= 0x800000u; exp2 = (int)ex - 150; }
    if (mant == 0) { m[i] = 0; e[i] = 0; continue; }
    const int tz = ctz32(mant);
    mant >>= tz;
    exp2 += tz;
    m[i] = (b >> 31) ? -(long long)mant : (long long)mant;
    e[i] = exp2;
    if (exp2 < emin) emin = exp2;
  }
  for (int i = 0; i < N; ++i) {
    if (m[i] == 0) { X[i] = 0; continue; }
    const int sh = e[i] - emin;
    const u64 mag = (u64)(m[i] < 0 ? -m[i] : m[i]);
    if (sh > 61 || (64 - clz64(mag)) + sh > 61) return false;
    X[i] = m[i] * (long long)(1ll << sh);
  }
  return true;
}

MCL_HD int orient2d_int(float ax, float ay, float bx, float by, float cx, float cy) {
  const float v[6] = {ax, ay, bx, by, cx, cy};
  long long X[6];
  if (!to_fixed(v, X)) return 2;
  const long long acx = X[0] - X[4], bcy = X[3] - X[5], acy = X[1] - X[5], bcx = X[2] - X[4];
  const i128 l = (i128)acx * bcy, r = (i128)acy * bcx;
  return l > r ? 1 : (l < r ? -1 : 0);
}

struct U256 {
  u64 w[4];
};

MCL_HD void u256_add(U256& acc, const U256& x) {
  u64 carry = 0;
  for (int i = 0; i < 4; ++i) {
    const u128 t = (u128)acc.w[i] + x.w[i] + carry;
    acc.w[i] = (u64)t;
    carry = (u64)(t >> 64);
  }
}

MCL_HD U256 u128_mul(u128 a, u128 b) {
  const u64 a0 = (u64)a, a1 = (u64)(a >> 64), b0 = (u64)b, b1 = (u64)(b >> 64);
  U256 r;
  const u128 t = (u128)a0 * b0;
  r.w[0] = (u64)t;
  const u128 p01 = (u128)a0 * b1, p10 = (u128)a1 * b0, p11 = (u128)a1 * b1;
  u128 mid = (t >> 64) + (u64)p01;
  mid += (u64)p10;
  r.w[1] = (u64)mid;
  u128 hi = (mid >> 64) + (p01 >> 64) + (p10 >> 64) + (u64)p11;
  r.w[2] = (u64)hi;
  r.w[3] = (u64)((hi >> 64) + (p11 >> 64));
  return r;
}

MCL_HD int u256_cmp(const U256& a, const U256& b) {
  for (int i = 3; i >= 0; --i)
    if (a.w[i] != b.w[i]) return a.w[i] > b.w[i] ? 1 : -1;
  return 0;
}

MCL_HD int incircle_int(float ax, float ay, float bx, float by, float cx, float cy, float dx, float dy) {
  const float v[8] = {ax, ay, bx, by, cx, cy, dx, dy};
  long long X[8];
  if (!to_fixed(v, X)) return 2;
  const long long adx = X[0] - X[6], ady = X[1] - X[7];
  const long long bdx = X[2] - X[6], bdy = X[3] - X[7];
  const long long cdx = X[4] - X[6], cdy = X[5] - X[7];
  const u128 lift[3] = {(u128)((i128)adx * adx) + (u128)((i128)ady * ady),
                        (u128)((i128)bdx * bdx) + (u128)((i128)bdy * bdy),
                        (u128)((i128)cdx * cdx) + (u128)((i128)cdy * cdy)};
  const i128 cross[3] = {(i128)bdx * cdy - (i128)bdy * cdx, (i128)cdx * ady - (i128)cdy * adx,
                         (i128)adx * bdy - (i128)ady * bdx};
  U256 pos = {{0, 0, 0, 0}}, neg = {{0, 0, 0, 0}};
  for (int k = 0; k < 3; ++k) {
    if (cross[k] == 0 || lift[k] == 0) continue;
    const u128 mag = (u128)(cross[k] < 0 ? -cross[k] : cross[k]);
    const U256 t = u128_mul(lift[k], mag);
    if (cross[k] > 0) u256_add(pos, t);
    else u256_add(neg, t);
  }
  return u256_cmp(pos, neg);
}

// ---------------------------------------------------------------------------
// Full ladders.  Only the FP32 filter is inlined at the call site; the rest of
// the ladder is one out-of-line call that returns the sign packed with flags
// (so the hot loops keep a small register footprint and no local memory).
enum : int { kUsedFp64 = 1, kUsedExact = 2, kUsedSos = 4, kOverflow = 8 };
MCL_HD int pack_sign(int s, int flags) { return (s + 1) | (flags << 2); }
MCL_HD int unpack_sign(int r) { return (r & 3) - 1; }
MCL_HD int unpack_flags(int r) { return r >> 2; }

MCL_HD_NOINLINE int orient2d_slow(float ax, float ay, float bx, float by, float cx, float cy) {
  int s = orient2d_int(ax, ay, bx, by, cx, cy);
  if (s != 2) return pack_sign(s, kUsedFp64 | kUsedExact);
  s = orient2d_fp64(ax, ay, bx, by, cx, cy);
  if (s != 2) return pack_sign(s, kUsedFp64);
  s = orient2d_exact_exp(ax, ay, bx, by, cx, cy);
  if (s == kExpOverflow) return pack_sign(0, kUsedFp64 | kUsedExact | kOverflow);
  return pack_sign(s, kUsedFp64 | kUsedExact);
}

MCL_HD_NOINLINE int incircle_slow(float ax, float ay, float bx, float by, float cx, float cy, float dx, float dy) {
  int s = incircle_int(ax, ay, bx, by, cx, cy, dx, dy);
  if (s != 2) return pack_sign(s, kUsedFp64 | kUsedExact);
  s = incircle_fp64(ax, ay, bx, by, cx, cy, dx, dy);
  if (s != 2) return pack_sign(s, kUsedFp64);
  s = incircle_exact_exp(ax, ay, bx, by, cx, cy, dx, dy);
  if (s == kExpOverflow) return pack_sign(0, kUsedFp64 | kUsedExact | kOverflow);
  return pack_sign(s, kUsedFp64 | kUsedExact);
}

// Exactly cocircular: decide by the symbolic perturbation (ascending ids).
MCL_HD_NOINLINE int incircle_sos_tail(float ax, float ay, float bx, float by, float cx, float cy, float dx, float dy,
                                      int ia, int ib, int ic, int id, int flags) {
  flags |= kUsedSos;
  int ids[4] = {ia, ib, ic, id};
  int ord[4] = {0, 1, 2, 3};
  for (int i = 1; i < 4; ++i)
    for (int j = i; j > 0 && ids[ord[j]] < ids[ord[j - 1]]; --j) {
      int tmp = ord[j]; ord[j] = ord[j - 1]; ord[j - 1] = tmp;
    }
  for (int k = 0; k < 4; ++k) {
    int r;
    int neg = 0;
    switch (ord[k]) {
      case 0: r = orient2d_fp32(bx, by, cx, cy, dx, dy); if (r == 2) r = orient2d_slow(bx, by, cx, cy, dx, dy); else r = pack_sign(r, 0); break;
      case 1: r = orient2d_fp32(ax, ay, cx, cy, dx, dy); if (r == 2) r = orient2d_slow(ax, ay, cx, cy, dx, dy); else r = pack_sign(r, 0); neg = 1; break;
      case 2: r = orient2d_fp32(ax, ay, bx, by, dx, dy); if (r == 2) r = orient2d_slow(ax, ay, bx, by, dx, dy); else r = pack_sign(r, 0); break;
      default: r = orient2d_fp32(ax, ay, bx, by, cx, cy); if (r == 2) r = orient2d_slow(ax, ay, bx, by, cx, cy); else r = pack_sign(r, 0); neg = 1; break;
    }
    flags |= unpack_flags(r) & kOverflow;
    const int c0 = neg ? -unpack_sign(r) : unpack_sign(r);
    if (c0 != 0) return pack_sign(c0, flags);
  }
  return pack_sign(0, flags);
}

template <typename Counters>
MCL_HD void count_flags(int flags, Counters* cnt, int* overflow, bool incircle) {
  if (cnt) {
    if (incircle) {
      if (flags & kUsedFp64) cnt->incircle_fp64++;
      if (flags & kUsedExact) cnt->incircle_exact++;
    } else {
      if (flags & kUsedFp64) cnt->orient_fp64++;
      if (flags & kUsedExact) cnt->orient_exact++;
    }
    if (flags & kUsedSos) cnt->sos++;
  }
  if (flags & kOverflow) *overflow = 1;
}

template <typename Counters>
MCL_HD int orient2d(float ax, float ay, float bx, float by, float cx, float cy, Counters* cnt, int* overflow) {
  const int s = orient2d_fp32(ax, ay, bx, by, cx, cy);
  if (s != 2) return s;
  const int r = orient2d_slow(ax, ay, bx, by, cx, cy);
  count_flags(unpack_flags(r), cnt, overflow, false);
  return unpack_sign(r);
}

template <typename Counters>
MCL_HD int incircle(float ax, float ay, float bx, float by, float cx, float cy, float dx, float dy,
                    Counters* cnt, int* overflow) {
  const int s = incircle_fp32(ax, ay, bx, by, cx, cy, dx, dy);
  if (s != 2) return s;
  const int r = incircle_slow(ax, ay, bx, by, cx, cy, dx, dy);
  count_flags(unpack_flags(r), cnt, overflow, true);
  return unpack_sign(r);
}

template <typename Counters>
MCL_HD int incircle_sos(float ax, float ay, float bx, float by, float cx, float cy, float dx, float dy,
                        int ia, int ib, int ic, int id, Counters* cnt, int* overflow) {
  const int s = incircle_fp32(ax, ay, bx, by, cx, cy, dx, dy);
  if (s != 2) return s;
  int r = incircle_slow(ax, ay, bx, by, cx, cy, dx, dy);
  if (unpack_sign(r) == 0 && !(unpack_flags(r) & kOverflow))
    r = incircle_sos_tail(ax, ay, bx, by, cx, cy, dx, dy, ia, ib, ic, id, unpack_flags(r));
  const int f = unpack_flags(r);
  count_flags(f, cnt, overflow, true);
  return unpack_sign(r);
}

}  // namespace mcl
