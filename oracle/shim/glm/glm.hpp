// Test infrastructure (oracle): a minimal glm stand-in, written for this
// project, that supplies exactly what the reference's src/ray-tracing/Bvh.h,
// GpuModels.h and RtScene.h use from glm (vec3, vec4, component-wise
// min/max, +, -, cross, length). The glm submodule is empty in the reference
// tree. min/max follow glm's scalar rule min(x,y) = (y < x) ? y : x and
// max(x,y) = (x < y) ? y : x, which fixes the order of -0/+0 and NaN.
#pragma once
#include <cmath>
#include <cfloat>
#include <cstdlib>

namespace glm {
struct vec3 {
  float x, y, z;
  vec3() : x(0), y(0), z(0) {}
  vec3(float a, float b, float c) : x(a), y(b), z(c) {}
  explicit vec3(double s) : x((float)s), y((float)s), z((float)s) {}
  explicit vec3(float s) : x(s), y(s), z(s) {}
  float &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  const float &operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
struct vec4 {
  float x, y, z, w;
  vec4() : x(0), y(0), z(0), w(0) {}
  vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
  vec4(double a, double b, double c, double d)
      : x((float)a), y((float)b), z((float)c), w((float)d) {}
  vec4(double a, int b, int c, double d)
      : x((float)a), y((float)b), z((float)c), w((float)d) {}
  float &operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};
inline float min(float a, float b) { return (b < a) ? b : a; }
inline float max(float a, float b) { return (a < b) ? b : a; }
inline vec3 min(const vec3 &a, const vec3 &b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline vec3 max(const vec3 &a, const vec3 &b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline vec3 operator+(const vec3 &a, const vec3 &b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3 &a, const vec3 &b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 cross(const vec3 &a, const vec3 &b) {
  return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float length(const vec3 &a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
}  // namespace glm
