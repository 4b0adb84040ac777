// Vector types of the drop-in headers.  The reference's call surface takes
// glm::vec2 / glm::ivec2; when glm is available it is used as is, otherwise a
// minimal layout-compatible stand-in (two floats / two ints) is declared.
#pragma once

#if __has_include(<glm/glm.hpp>)
#include <glm/glm.hpp>
#else
#include <cmath>
#ifndef __CUDACC__
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#endif
namespace glm {
struct vec2 {
  float x, y;
  __host__ __device__ vec2() : x(0), y(0) {}
  __host__ __device__ explicit vec2(float s) : x(s), y(s) {}
  __host__ __device__ vec2(float a, float b) : x(a), y(b) {}
  __host__ __device__ vec2& operator+=(const vec2& o) { x += o.x; y += o.y; return *this; }
};
__host__ __device__ inline vec2 operator+(vec2 a, vec2 b) { return vec2(a.x + b.x, a.y + b.y); }
__host__ __device__ inline vec2 operator-(vec2 a, vec2 b) { return vec2(a.x - b.x, a.y - b.y); }
__host__ __device__ inline vec2 operator*(vec2 a, float s) { return vec2(a.x * s, a.y * s); }
__host__ __device__ inline float dot(vec2 a, vec2 b) { return a.x * b.x + a.y * b.y; }
struct ivec2 {
  int x, y;
  __host__ __device__ ivec2() : x(0), y(0) {}
  __host__ __device__ explicit ivec2(int s) : x(s), y(s) {}
  __host__ __device__ ivec2(int a, int b) : x(a), y(b) {}
};
}  // namespace glm
#endif

static_assert(sizeof(glm::vec2) == 8, "glm::vec2 must be two packed floats");
