// Minimal stand-in for the glm vector types the reference's host code uses
// (vec2 / dvec2 / ivec2 arithmetic, dot, length, clamp).  Written for building
// the reference's HostTriangulation as an oracle check; not a copy of glm.
#pragma once
#include <cmath>

namespace glm {

template <typename T>
struct tvec2 {
  T x, y;
  tvec2() : x(0), y(0) {}
  explicit tvec2(T s) : x(s), y(s) {}
  tvec2(T a, T b) : x(a), y(b) {}
  template <typename U>
  tvec2(const tvec2<U>& o) : x((T)o.x), y((T)o.y) {}
  tvec2& operator+=(const tvec2& o) { x += o.x; y += o.y; return *this; }
  tvec2& operator-=(const tvec2& o) { x -= o.x; y -= o.y; return *this; }
};

template <typename T> tvec2<T> operator+(const tvec2<T>& a, const tvec2<T>& b) { return {a.x + b.x, a.y + b.y}; }
template <typename T> tvec2<T> operator-(const tvec2<T>& a, const tvec2<T>& b) { return {a.x - b.x, a.y - b.y}; }
template <typename T> tvec2<T> operator*(const tvec2<T>& a, T s) { return {a.x * s, a.y * s}; }
template <typename T> tvec2<T> operator*(T s, const tvec2<T>& a) { return {a.x * s, a.y * s}; }
template <typename T> tvec2<T> operator/(const tvec2<T>& a, T s) { return {a.x / s, a.y / s}; }

template <typename T> T dot(const tvec2<T>& a, const tvec2<T>& b) { return a.x * b.x + a.y * b.y; }
template <typename T> T length(const tvec2<T>& a) { return std::sqrt(dot(a, a)); }
template <typename T> T clamp(T v, T lo, T hi) { return v < lo ? lo : (v > hi ? hi : v); }

using vec2 = tvec2<float>;
using dvec2 = tvec2<double>;
using ivec2 = tvec2<int>;

}  // namespace glm
