// Minimal, project-written stand-in for the few GLM types and functions that
// the reference's simulation.cpp / pressure_solver.cpp / db2dgrid.hpp touch.
// GLM is not installed in this image; this header exists only so that the
// reference's own sources compile unmodified into the test oracle.
#pragma once
#include <cmath>

namespace glm {

struct ivec2;

struct vec2 {
  float x, y;
  vec2() : x(0), y(0) {}
  vec2(float s) : x(s), y(s) {}
  vec2(float a, float b) : x(a), y(b) {}
  template <class V, class = decltype(V{}.z)> explicit vec2(const V &v) : x(v.x), y(v.y) {}
};

struct ivec2 {
  int x, y;
  ivec2() : x(0), y(0) {}
  ivec2(int a, int b) : x(a), y(b) {}
  ivec2(const vec2 &v) : x((int)v.x), y((int)v.y) {}
  operator vec2() const { return vec2((float)x, (float)y); }
};

struct vec3 {
  float x, y, z;
  vec3() : x(0), y(0), z(0) {}
  vec3(float a, float b, float c) : x(a), y(b), z(c) {}
};

struct vec4 {
  float x, y, z, w;
};

struct mat4 {
  float m[16];
  mat4() {}
  explicit mat4(float) {}
};

inline vec2 operator+(vec2 a, vec2 b) { return {a.x + b.x, a.y + b.y}; }
inline vec2 operator-(vec2 a, vec2 b) { return {a.x - b.x, a.y - b.y}; }
inline vec2 operator*(vec2 a, vec2 b) { return {a.x * b.x, a.y * b.y}; }
inline vec2 operator/(vec2 a, vec2 b) { return {a.x / b.x, a.y / b.y}; }
inline vec2 operator+(vec2 a, float s) { return {a.x + s, a.y + s}; }
inline vec2 operator-(vec2 a, float s) { return {a.x - s, a.y - s}; }
inline vec2 operator*(vec2 a, float s) { return {a.x * s, a.y * s}; }
inline vec2 operator/(vec2 a, float s) { return {a.x / s, a.y / s}; }
inline vec2 operator*(float s, vec2 a) { return {a.x * s, a.y * s}; }
inline ivec2 operator+(ivec2 a, ivec2 b) { return {a.x + b.x, a.y + b.y}; }
inline ivec2 operator-(ivec2 a, ivec2 b) { return {a.x - b.x, a.y - b.y}; }

inline float min(float a, float b) { return b < a ? b : a; }
inline float max(float a, float b) { return a < b ? b : a; }
inline ivec2 min(ivec2 a, ivec2 b) { return {b.x < a.x ? b.x : a.x, b.y < a.y ? b.y : a.y}; }
inline ivec2 max(ivec2 a, ivec2 b) { return {a.x < b.x ? b.x : a.x, a.y < b.y ? b.y : a.y}; }
inline vec2 clamp(vec2 v, vec2 lo, vec2 hi) {
  return {min(max(v.x, lo.x), hi.x), min(max(v.y, lo.y), hi.y)};
}
inline vec2 fract(vec2 v) { return {v.x - std::floor(v.x), v.y - std::floor(v.y)}; }
inline float mix(float a, float b, float t) { return a + t * (b - a); }

}  // namespace glm
