// Minimal stand-in for libmorton's 2-D encoder used by the reference's
// HostTriangulation::addDelaunayPoints: interleave the low 32 bits of the two
// coordinates, x into the even bits.  Written for the oracle check build.
#pragma once
#include <cstdint>

namespace libmorton {
template <typename M, typename C>
inline M m2D_e_LUT(const C x, const C y) {
  auto spread = [](uint64_t w) {
    w &= 0xFFFFFFFFull;
    w = (w | (w << 16)) & 0x0000FFFF0000FFFFull;
    w = (w | (w << 8)) & 0x00FF00FF00FF00FFull;
    w = (w | (w << 4)) & 0x0F0F0F0F0F0F0F0Full;
    w = (w | (w << 2)) & 0x3333333333333333ull;
    w = (w | (w << 1)) & 0x5555555555555555ull;
    return w;
  };
  return (M)(spread((uint64_t)x) | (spread((uint64_t)y) << 1));
}
}  // namespace libmorton
