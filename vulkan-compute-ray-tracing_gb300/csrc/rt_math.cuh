// Device math with a fixed evaluation order.
//
// Every helper spells its operations with round-to-nearest intrinsics
// (__fadd_rn, __fmul_rn, ...), which the compiler never fuses into FMAs, so
// each result is the IEEE fp32 value of the GLSL expression evaluated left to
// right — the same value a host compiler produces for the same expression
// with contraction disabled. This is what makes the closest-hit index and t
// bit-exact against an fp32 host evaluation of the reference shader
// (resources/shaders/source/ray-trace-compute.comp).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rtgb {

struct f3 {
  float x, y, z;
};

__device__ __forceinline__ f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 ld3(const float *p) { return f3{p[0], p[1], p[2]}; }
__device__ __forceinline__ f3 add3(f3 a, f3 b) {
  return f3{__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)};
}
__device__ __forceinline__ f3 sub3(f3 a, f3 b) {
  return f3{__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)};
}
__device__ __forceinline__ f3 mul3(float s, f3 a) {
  return f3{__fmul_rn(s, a.x), __fmul_rn(s, a.y), __fmul_rn(s, a.z)};
}
__device__ __forceinline__ f3 mulv3(f3 a, f3 b) {
  return f3{__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z)};
}
__device__ __forceinline__ f3 divs3(f3 a, float s) {
  return f3{__fdiv_rn(a.x, s), __fdiv_rn(a.y, s), __fdiv_rn(a.z, s)};
}
__device__ __forceinline__ f3 neg3(f3 a) { return f3{-a.x, -a.y, -a.z}; }
// dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z
__device__ __forceinline__ float dot3(f3 a, f3 b) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
// GLSL cross(a, b) = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y)
__device__ __forceinline__ f3 cross3(f3 a, f3 b) {
  return f3{__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(b.y, a.z)),
            __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(b.z, a.x)),
            __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(b.x, a.y))};
}
__device__ __forceinline__ float length3(f3 a) { return __fsqrt_rn(dot3(a, a)); }
// normalize(v) = v / length(v), one IEEE division per component.
__device__ __forceinline__ f3 normalize3(f3 a) { return divs3(a, length3(a)); }

// Two fp32 values in one 64-bit register pair, for the packed arithmetic of
// sm_100 and later (add/mul/fma .f32x2): one instruction computes both
// halves, each rounded exactly as the scalar operation with the same
// rounding mode would round it.
struct f2 {
  unsigned long long v;
};
__device__ __forceinline__ f2 pk2(float lo, float hi) {
  f2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ float lo2(f2 a) { return __uint_as_float((uint32_t)a.v); }
__device__ __forceinline__ float hi2(f2 a) { return __uint_as_float((uint32_t)(a.v >> 32)); }
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
  f2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d.v) : "l"(a.v), "l"(b.v), "l"(c.v));
  return d;
}
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
  f2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
  return d;
}

// GLSL min/max in the specification's wording.
__device__ __forceinline__ float gmin(float x, float y) { return (y < x) ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return (x < y) ? y : x; }
__device__ __forceinline__ float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
// reflect(I, N) = I - 2*dot(N, I)*N
__device__ __forceinline__ f3 reflect3(f3 I, f3 N) {
  float s = __fmul_rn(2.0f, dot3(N, I));
  return sub3(I, mul3(s, N));
}
// refract(I, N, eta): k = 1 - eta*eta*(1 - dot(N,I)^2); 0 if k < 0,
// else eta*I - (eta*dot(N,I) + sqrt(k))*N
__device__ __forceinline__ f3 refract3(f3 I, f3 N, float eta) {
  float d = dot3(N, I);
  float k = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(eta, eta), __fsub_rn(1.0f, __fmul_rn(d, d))));
  if (k < 0.0f) return mk3(0.0f, 0.0f, 0.0f);
  float s = __fadd_rn(__fmul_rn(eta, d), __fsqrt_rn(k));
  return sub3(mul3(eta, I), mul3(s, N));
}

// random.glsl:4-22: state = state*747796405 + 1; RXS-M-XS output;
// float(word) / 4294967295.0f (the divisor rounds to 2^32 in fp32).
struct Rng {
  uint32_t s;
  __device__ __forceinline__ float next() {
    s = s * 747796405u + 1u;
    uint32_t w = ((s >> ((s >> 28) + 4u)) ^ s) * 277803737u;
    w = (w >> 22) ^ w;
    return __fdiv_rn(__uint2float_rn(w), 4294967296.0f);
  }
};

}  // namespace rtgb
