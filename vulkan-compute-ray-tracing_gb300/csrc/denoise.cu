// smartDeNoise as a CUDA pass over an RGBA32F image: the filter the
// reference's post-process shader defines (post-process-shader.frag:26-68,
// after BrutPitt's glslSmartDeNoise) and leaves switched off in main()
// (frag:73 blends it 50/50 with the unfiltered pixel in the commented line).
//
// Per pixel: a circular kernel of radius round(kSigma * sigma); for each
// column x in [-radius, radius] the rows run y = -pt, -pt + 1, ... <= pt with
// pt = sqrt(radius^2 - x^2), so most taps fall between two texel rows. Each
// tap is weighted by a spatial Gaussian exp(-|d|^2 / (2 sigma^2)) / (pi 2
// sigma^2) and a range Gaussian of its RGBA distance to the centre pixel,
// exp(-|dC|^2 / (2 threshold^2)) / (sqrt(2 pi) threshold); the result is the
// weighted mean. Taps are fetched the way the reference's sampler does
// (linear filter, REPEAT wrap: src/memory/Image.cpp:353-357), here in texel
// space: position (px + x, py + y), bilinear between the four texels around
// it, indices wrapped modulo the image size. Every operation is a separately
// rounded fp32 step in shader order, as in the oracle's restatement; only
// expf/sqrtf come from CUDA's library.
#include <cuda_runtime.h>

#include "rt_internal.h"
#include "rt_math.cuh"

namespace rtgb {
namespace {

struct DenoiseParams {
  float radius, rad_q, inv_sigma_q2, inv_sigma_q2pi, inv_thr_q2, inv_thr_sqrt2pi, mix;
};

__device__ __forceinline__ float4 texel(const float4 *__restrict__ img, int x, int y, int W, int H) {
  x %= W;
  y %= H;
  if (x < 0) x += W;
  if (y < 0) y += H;
  return __ldg(img + (size_t)y * W + x);
}

__device__ __forceinline__ float lerp_rn(float a, float b, float w) {
  return __fadd_rn(__fmul_rn(__fsub_rn(1.0f, w), a), __fmul_rn(w, b));
}

__device__ __forceinline__ float4 lerp4(float4 a, float4 b, float w) {
  return make_float4(lerp_rn(a.x, b.x, w), lerp_rn(a.y, b.y, w), lerp_rn(a.z, b.z, w), lerp_rn(a.w, b.w, w));
}

__global__ void k_denoise(const float4 *__restrict__ in, int W, int H, DenoiseParams p, float4 *__restrict__ out) {
  const int px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y * blockDim.y + threadIdx.y;
  if (px >= W || py >= H) return;
  const float4 c = in[(size_t)py * W + px];
  float z = 0.0f;
  float4 a = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  for (float x = -p.radius; x <= p.radius; x = __fadd_rn(x, 1.0f)) {
    const float pt = __fsqrt_rn(__fsub_rn(p.rad_q, __fmul_rn(x, x)));
    for (float y = -pt; y <= pt; y = __fadd_rn(y, 1.0f)) {
      const float dd = __fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y));
      const float blur = __fmul_rn(expf(__fmul_rn(-dd, p.inv_sigma_q2)), p.inv_sigma_q2pi);
      // Bilinear tap at texel-space position (px + x, py + y).
      const float s = __fadd_rn((float)px, x), t = __fadd_rn((float)py, y);
      const float fs = floorf(s), ft = floorf(t);
      const float al = __fsub_rn(s, fs), be = __fsub_rn(t, ft);
      const int i0 = (int)fs, j0 = (int)ft;
      const float4 w = lerp4(lerp4(texel(in, i0, j0, W, H), texel(in, i0 + 1, j0, W, H), al),
                             lerp4(texel(in, i0, j0 + 1, W, H), texel(in, i0 + 1, j0 + 1, W, H), al), be);
      const float dx = __fsub_rn(w.x, c.x), dy = __fsub_rn(w.y, c.y), dz = __fsub_rn(w.z, c.z),
                  dw = __fsub_rn(w.w, c.w);
      const float dc2 = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)),
                                  __fmul_rn(dw, dw));
      const float delta =
          __fmul_rn(__fmul_rn(expf(__fmul_rn(-dc2, p.inv_thr_q2)), p.inv_thr_sqrt2pi), blur);
      z = __fadd_rn(z, delta);
      a.x = __fadd_rn(a.x, __fmul_rn(delta, w.x));
      a.y = __fadd_rn(a.y, __fmul_rn(delta, w.y));
      a.z = __fadd_rn(a.z, __fmul_rn(delta, w.z));
      a.w = __fadd_rn(a.w, __fmul_rn(delta, w.w));
    }
  }
  const float4 f = make_float4(__fdiv_rn(a.x, z), __fdiv_rn(a.y, z), __fdiv_rn(a.z, z), __fdiv_rn(a.w, z));
  out[(size_t)py * W + px] = lerp4(c, f, p.mix);
}

}  // namespace

cudaError_t launch_denoise(const float *in, uint32_t W, uint32_t H, float sigma, float ksigma, float threshold,
                           float mix, float *out, cudaStream_t st) {
  if (W == 0 || H == 0) return cudaSuccess;
  // frag:29-36, each constant as one fp32 expression.
  const float kInvPi = 0.31830988618379067154f, kInvSqrt2Pi = 0.39894228040143267794f;
  DenoiseParams p;
  p.radius = roundf(ksigma * sigma);
  p.rad_q = p.radius * p.radius;
  p.inv_sigma_q2 = 0.5f / (sigma * sigma);
  p.inv_sigma_q2pi = kInvPi * p.inv_sigma_q2;
  p.inv_thr_q2 = 0.5f / (threshold * threshold);
  p.inv_thr_sqrt2pi = kInvSqrt2Pi / threshold;
  p.mix = mix;
  dim3 block(16, 16), grid((W + 15) / 16, (H + 15) / 16);
  k_denoise<<<grid, block, 0, st>>>(reinterpret_cast<const float4 *>(in), (int)W, (int)H, p,
                                     reinterpret_cast<float4 *>(out));
  return cudaGetLastError();
}

}  // namespace rtgb
