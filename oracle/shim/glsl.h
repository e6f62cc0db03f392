// Test infrastructure (oracle) — NOT part of the product.
//
// A small GLSL 4.50 compatibility layer in C++ so that the reference's
// compute shader, mechanically rewritten by oracle/glsl2cpp.py, compiles and
// runs on the host. Only what that shader uses is defined. Every built-in
// follows the GLSL specification's definition in fp32 (min(x, y) = y < x ?
// y : x, normalize(v) = v / length(v), reflect, refract, ...); the file is
// compiled with -ffp-contract=off so no step is fused. Images are RGBA8
// (the shader's `rgba8` format): imageStore rounds each channel to 8 bits.
#pragma once
#include <cmath>
#include <cstdint>
#include <vector>

typedef uint32_t uint;

struct vec2 {
  float x, y;
  vec2() : x(0), y(0) {}
  vec2(float a, float b) : x(a), y(b) {}
  explicit vec2(float s) : x(s), y(s) {}
  vec2 xy() const { return *this; }
};
struct vec3 {
  float x, y, z;
  vec3() : x(0), y(0), z(0) {}
  vec3(float a, float b, float c) : x(a), y(b), z(c) {}
  explicit vec3(float s) : x(s), y(s), z(s) {}
  vec3 zxy() const { return vec3(z, x, y); }
  vec3 xyz() const { return *this; }
  vec2 xy() const { return vec2(x, y); }
  int length() const { return 3; }  // GLSL: the number of components
};
struct vec4 {
  float x, y, z, w;
  vec4() : x(0), y(0), z(0), w(0) {}
  vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
  vec4(vec3 v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
  vec3 xyz() const { return vec3(x, y, z); }
  vec3 rgb() const { return vec3(x, y, z); }
  vec4 rgba() const { return *this; }
};
struct ivec2 {
  int x, y;
  ivec2(int a, int b) : x(a), y(b) {}
  explicit ivec2(vec2 v) : x((int)v.x), y((int)v.y) {}
};
// gl_GlobalInvocationID: .xy converts to vec2 as GLSL does where a uvec2 meets
// a vec2 in arithmetic (the only use in the shader).
struct uvec3 {
  uint x, y, z;
  vec2 xy() const { return vec2((float)x, (float)y); }
};

inline vec2 operator/(vec2 a, vec2 b) { return vec2(a.x / b.x, a.y / b.y); }
inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(vec3 a, vec3 b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(vec3 a, vec3 b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator/(vec3 a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 &operator+=(vec3 &a, vec3 b) { return a = a + b; }
inline vec3 &operator*=(vec3 &a, vec3 b) { return a = a * b; }
inline vec3 &operator*=(vec3 &a, float s) { return a = a * s; }
inline vec4 operator+(vec4 a, vec4 b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator*(vec4 a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline vec4 operator/(vec4 a, float s) { return vec4(a.x / s, a.y / s, a.z / s, a.w / s); }

inline float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 cross(vec3 a, vec3 b) {
  return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float length(vec3 a) { return std::sqrt(dot(a, a)); }
inline vec3 normalize(vec3 a) { return a / length(a); }
inline float min(float x, float y) { return (y < x) ? y : x; }
inline float max(float x, float y) { return (x < y) ? y : x; }
inline vec3 min(vec3 a, vec3 b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline vec3 max(vec3 a, vec3 b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float abs(float x) { return std::fabs(x); }
inline float floor(float x) { return std::floor(x); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float sin(float x) { return std::sin(x); }
inline float cos(float x) { return std::cos(x); }
inline float tan(float x) { return std::tan(x); }
inline vec3 reflect(vec3 I, vec3 N) { return I - 2.0f * dot(N, I) * N; }
inline vec3 refract(vec3 I, vec3 N, float eta) {
  float d = dot(N, I);
  float k = 1.0f - eta * eta * (1.0f - d * d);
  if (k < 0.0f) return vec3(0.0f);
  return eta * I - (eta * d + std::sqrt(k)) * N;
}

// Runtime-sized storage-buffer array: length() is the bound element count.
template <typename T> struct GlslArray {
  const T *data = nullptr;
  int n = 0;
  const T &operator[](int i) const { return data[i]; }
  int length() const { return n; }
};

// An rgba8 storage image.
struct image2D {
  int w = 0, h = 0;
  std::vector<uint8_t> px;  // w * h * 4
};
inline uint8_t unorm8(float v) {
  float c = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);  // NaN -> 0
  if (!(c == c)) c = 0.0f;
  return (uint8_t)std::floor(c * 255.0f + 0.5f);
}
inline vec2 glsl_imageSize(const image2D &im) { return vec2((float)im.w, (float)im.h); }
inline vec4 imageLoad(const image2D &im, ivec2 p) {
  const uint8_t *q = &im.px[4 * ((size_t)p.y * im.w + p.x)];
  return vec4(q[0] / 255.0f, q[1] / 255.0f, q[2] / 255.0f, q[3] / 255.0f);
}
inline void imageStore(image2D &im, ivec2 p, vec4 v) {
  uint8_t *q = &im.px[4 * ((size_t)p.y * im.w + p.x)];
  q[0] = unorm8(v.x);
  q[1] = unorm8(v.y);
  q[2] = unorm8(v.z);
  q[3] = unorm8(v.w);
}

extern thread_local uvec3 gl_GlobalInvocationID;
