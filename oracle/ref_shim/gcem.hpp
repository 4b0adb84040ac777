// Minimal constexpr floor/sqrt for the reference's unused filter constants
// (include/Common_Triangulation.h:16-17).  Written for the oracle check build.
#pragma once
namespace gcem {
constexpr double floor(double x) {
  return (double)(long long)x - ((double)(long long)x > x ? 1.0 : 0.0);
}
constexpr double sqrt_iter(double x, double g, int n) {
  return n == 0 ? g : sqrt_iter(x, 0.5 * (g + x / g), n - 1);
}
constexpr double sqrt(double x) { return x <= 0 ? 0.0 : sqrt_iter(x, x > 1 ? x : 1.0, 200); }
constexpr double abs(double x) { return x < 0 ? -x : x; }
}  // namespace gcem
