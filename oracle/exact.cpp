// Oracle exact predicates: double filter + big-integer exact fallback.
// Test infrastructure only (see exact.h).
#include "exact.h"

#include <cmath>
#include <cstring>
#include <vector>
#include <algorithm>

namespace oracle {

namespace {

ExactStats g_stats = {0, 0, 0, 0, 0};

// ---------------------------------------------------------------------------
// Minimal signed big integer: sign-magnitude, 32-bit limbs, little endian.
struct Big {
  int sign = 0;                 // -1, 0, +1
  std::vector<uint32_t> mag;    // no leading zero limbs when sign != 0

  void trim() {
    while (!mag.empty() && mag.back() == 0) mag.pop_back();
    if (mag.empty()) sign = 0;
  }
};

int cmp_mag(const std::vector<uint32_t>& a, const std::vector<uint32_t>& b) {
  if (a.size() != b.size()) return a.size() < b.size() ? -1 : 1;
  for (size_t i = a.size(); i-- > 0;) {
    if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
  }
  return 0;
}

std::vector<uint32_t> add_mag(const std::vector<uint32_t>& a, const std::vector<uint32_t>& b) {
  std::vector<uint32_t> r(std::max(a.size(), b.size()) + 1, 0);
  uint64_t carry = 0;
  for (size_t i = 0; i < r.size(); ++i) {
    uint64_t s = carry;
    if (i < a.size()) s += a[i];
    if (i < b.size()) s += b[i];
    r[i] = (uint32_t)s;
    carry = s >> 32;
  }
  return r;
}

// requires |a| >= |b|
std::vector<uint32_t> sub_mag(const std::vector<uint32_t>& a, const std::vector<uint32_t>& b) {
  std::vector<uint32_t> r(a.size(), 0);
  int64_t borrow = 0;
  for (size_t i = 0; i < a.size(); ++i) {
    int64_t s = (int64_t)a[i] - borrow - (i < b.size() ? (int64_t)b[i] : 0);
    borrow = 0;
    if (s < 0) { s += ((int64_t)1 << 32); borrow = 1; }
    r[i] = (uint32_t)s;
  }
  return r;
}

Big add(const Big& a, const Big& b) {
  if (a.sign == 0) return b;
  if (b.sign == 0) return a;
  Big r;
  if (a.sign == b.sign) {
    r.sign = a.sign;
    r.mag = add_mag(a.mag, b.mag);
  } else {
    int c = cmp_mag(a.mag, b.mag);
    if (c == 0) return Big();
    if (c > 0) { r.sign = a.sign; r.mag = sub_mag(a.mag, b.mag); }
    else       { r.sign = b.sign; r.mag = sub_mag(b.mag, a.mag); }
  }
  r.trim();
  return r;
}

Big neg(Big a) { a.sign = -a.sign; return a; }
Big sub(const Big& a, const Big& b) { return add(a, neg(b)); }

Big mul(const Big& a, const Big& b) {
  if (a.sign == 0 || b.sign == 0) return Big();
  Big r;
  r.sign = a.sign * b.sign;
  r.mag.assign(a.mag.size() + b.mag.size() + 1, 0);
  for (size_t i = 0; i < a.mag.size(); ++i) {
    uint64_t carry = 0;
    for (size_t j = 0; j < b.mag.size(); ++j) {
      uint64_t cur = (uint64_t)r.mag[i + j] + (uint64_t)a.mag[i] * b.mag[j] + carry;
      r.mag[i + j] = (uint32_t)cur;
      carry = cur >> 32;
    }
    size_t k = i + b.mag.size();
    while (carry) {
      uint64_t cur = (uint64_t)r.mag[k] + carry;
      r.mag[k] = (uint32_t)cur;
      carry = cur >> 32;
      ++k;
    }
  }
  r.trim();
  return r;
}

// value = m * 2^shift with m >= 0, shift >= 0
Big from_shifted(uint32_t m, int shift, int sign) {
  Big r;
  if (m == 0) return r;
  r.sign = sign;
  int limb = shift / 32, bit = shift % 32;
  r.mag.assign(limb + 2, 0);
  uint64_t v = (uint64_t)m << bit;
  r.mag[limb] = (uint32_t)v;
  r.mag[limb + 1] = (uint32_t)(v >> 32);
  r.trim();
  return r;
}

// Decompose a finite float into (sign, integer mantissa, exponent): f = s*m*2^e.
void decompose(float f, int& s, uint32_t& m, int& e) {
  uint32_t bits;
  std::memcpy(&bits, &f, 4);
  s = (bits >> 31) ? -1 : 1;
  uint32_t ex = (bits >> 23) & 0xFF;
  uint32_t fr = bits & 0x7FFFFF;
  if (ex == 0) { m = fr; e = -149; }
  else { m = fr | 0x800000u; e = (int)ex - 150; }
  if (m == 0) { s = 0; }
}

// Convert n floats into exact big integers on a common exponent.
void to_common(const float* v, int n, Big* out) {
  int s[8]; uint32_t m[8]; int e[8];
  int emin = 1 << 30;
  for (int i = 0; i < n; ++i) {
    decompose(v[i], s[i], m[i], e[i]);
    if (m[i] != 0) emin = std::min(emin, e[i]);
  }
  for (int i = 0; i < n; ++i) {
    out[i] = (m[i] == 0) ? Big() : from_shifted(m[i], e[i] - emin, s[i]);
  }
}

int orient_big(P2 a, P2 b, P2 c) {
  float v[6] = {a.x, a.y, b.x, b.y, c.x, c.y};
  Big B[6];
  to_common(v, 6, B);
  Big l = mul(sub(B[2], B[0]), sub(B[5], B[1]));
  Big r = mul(sub(B[3], B[1]), sub(B[4], B[0]));
  return sub(l, r).sign;
}

int incircle_big(P2 a, P2 b, P2 c, P2 d) {
  float v[8] = {a.x, a.y, b.x, b.y, c.x, c.y, d.x, d.y};
  Big B[8];
  to_common(v, 8, B);
  Big adx = sub(B[0], B[6]), ady = sub(B[1], B[7]);
  Big bdx = sub(B[2], B[6]), bdy = sub(B[3], B[7]);
  Big cdx = sub(B[4], B[6]), cdy = sub(B[5], B[7]);
  Big alift = add(mul(adx, adx), mul(ady, ady));
  Big blift = add(mul(bdx, bdx), mul(bdy, bdy));
  Big clift = add(mul(cdx, cdx), mul(cdy, cdy));
  Big bc = sub(mul(bdx, cdy), mul(bdy, cdx));
  Big ca = sub(mul(cdx, ady), mul(cdy, adx));
  Big ab = sub(mul(adx, bdy), mul(ady, bdx));
  Big det = add(add(mul(alift, bc), mul(blift, ca)), mul(clift, ab));
  return det.sign;
}

const double kEps = 1.1102230246251565e-16;  // 2^-53
const double kCcwErrA = (3.0 + 16.0 * kEps) * kEps;
const double kIccErrA = (10.0 + 96.0 * kEps) * kEps;

}  // namespace

int orient2d_exact(P2 a, P2 b, P2 c) {
  ++g_stats.orient_calls;
  double detleft = ((double)a.x - (double)c.x) * ((double)b.y - (double)c.y);
  double detright = ((double)a.y - (double)c.y) * ((double)b.x - (double)c.x);
  double det = detleft - detright;
  double detsum;
  if (detleft > 0.0) {
    if (detright <= 0.0) return det > 0 ? 1 : (det < 0 ? -1 : 0);
    detsum = detleft + detright;
  } else if (detleft < 0.0) {
    if (detright >= 0.0) return det > 0 ? 1 : (det < 0 ? -1 : 0);
    detsum = -detleft - detright;
  } else {
    // detleft == 0: det = -detright exactly when the products are exact;
    // fall through to the exact path for safety.
    detsum = std::fabs(detright);
    if (detsum == 0.0) { ++g_stats.orient_exact; return orient_big(a, b, c); }
  }
  double err = kCcwErrA * detsum;
  if (det >= err || -det >= err) {
    if (det != 0.0) return det > 0 ? 1 : -1;
  }
  ++g_stats.orient_exact;
  return orient_big(a, b, c);
}

int incircle_exact(P2 a, P2 b, P2 c, P2 d) {
  ++g_stats.incircle_calls;
  double adx = (double)a.x - (double)d.x, ady = (double)a.y - (double)d.y;
  double bdx = (double)b.x - (double)d.x, bdy = (double)b.y - (double)d.y;
  double cdx = (double)c.x - (double)d.x, cdy = (double)c.y - (double)d.y;
  double bdxcdy = bdx * cdy, cdxbdy = cdx * bdy;
  double alift = adx * adx + ady * ady;
  double cdxady = cdx * ady, adxcdy = adx * cdy;
  double blift = bdx * bdx + bdy * bdy;
  double adxbdy = adx * bdy, bdxady = bdx * ady;
  double clift = cdx * cdx + cdy * cdy;
  double det = alift * (bdxcdy - cdxbdy) + blift * (cdxady - adxcdy) + clift * (adxbdy - bdxady);
  double perm = (std::fabs(bdxcdy) + std::fabs(cdxbdy)) * alift +
                (std::fabs(cdxady) + std::fabs(adxcdy)) * blift +
                (std::fabs(adxbdy) + std::fabs(bdxady)) * clift;
  double err = kIccErrA * perm;
  // Guard against underflow of the bound for extremely close points.
  if (perm > 1e-250 && (det > err || -det > err)) return det > 0 ? 1 : -1;
  ++g_stats.incircle_exact;
  return incircle_big(a, b, c, d);
}

int incircle_sos(P2 a, P2 b, P2 c, P2 d, int ia, int ib, int ic, int id) {
  int s = incircle_exact(a, b, c, d);
  if (s != 0) return s;
  ++g_stats.sos_used;
  struct Item { int id; int which; } items[4] = {{ia, 0}, {ib, 1}, {ic, 2}, {id, 3}};
  std::sort(items, items + 4, [](const Item& x, const Item& y) { return x.id < y.id; });
  for (int k = 0; k < 4; ++k) {
    int c0 = 0;
    switch (items[k].which) {
      case 0: c0 = orient2d_exact(b, c, d); break;
      case 1: c0 = -orient2d_exact(a, c, d); break;
      case 2: c0 = orient2d_exact(a, b, d); break;
      case 3: c0 = -orient2d_exact(a, b, c); break;
    }
    if (c0 != 0) return c0;
  }
  return 0;  // all four points collinear
}

int orient2d_ref(P2 a, P2 b, P2 c) {
  // Helpers_Triangulation.h:86-122, with abs() bound to the double overload.
  const double EPS = (double)0.00000000000000001f;
  double l = ((double)b.x - (double)a.x) * ((double)c.y - (double)a.y);
  double r = ((double)b.y - (double)a.y) * ((double)c.x - (double)a.x);
  double det = l - r;
  return (std::fabs(det) < EPS ? 0 : (det > 0 ? 1 : -1));
}

int incircle_ref(P2 a, P2 b, P2 c, P2 d) {
  // Helpers_Triangulation.h:136-151: lifted 3x3 determinant in double.
  const double EPS = (double)0.00000000000000001f;
  const double a00 = (double)(a.x - d.x);  // float subtraction, as in the reference
  const double a01 = (double)(a.y - d.y);
  const double a02 = a00 * a00 + a01 * a01;
  const double a10 = (double)(b.x - d.x);
  const double a11 = (double)(b.y - d.y);
  const double a12 = a10 * a10 + a11 * a11;
  const double a20 = (double)(c.x - d.x);
  const double a21 = (double)(c.y - d.y);
  const double a22 = a20 * a20 + a21 * a21;
  double det = (a00 * (a11 * a22 - a12 * a21) - a01 * (a10 * a22 - a12 * a20) +
                a02 * (a10 * a21 - a11 * a20));
  return (std::fabs(det) < EPS ? 0 : (det > 0 ? 1 : -1));
}

ExactStats exact_stats() { return g_stats; }
void exact_stats_reset() { g_stats = {0, 0, 0, 0, 0}; }

}  // namespace oracle
