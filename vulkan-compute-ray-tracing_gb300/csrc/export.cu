// Display epilogue: the reference's post-process fragment shader
// (resources/shaders/source/post-process-shader.frag:62-68) turns the
// accumulated image into the displayed one with pow(rgb, 1/2.2) and alpha 1;
// the swapchain then stores 8 bits per channel. Here that is one pass over
// the RGBA32F image into an RGBA8 device buffer. The smartDeNoise filter the
// shader defines (disabled there, frag:73) is a separate pass, denoise.cu.
#include <cuda_runtime.h>

#include "rt_internal.h"

namespace rtgb {
namespace {

__device__ __forceinline__ uint8_t to_unorm8(float x) {
  x = fminf(fmaxf(x, 0.0f), 1.0f);  // NaN -> 0
  return (uint8_t)__float2int_rn(x * 255.0f);
}

__global__ void k_export(const float4 *__restrict__ in, uint32_t n, float inv_gamma, uchar4 *__restrict__ out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 c = in[i];
  float r = c.x > 0.0f ? powf(c.x, inv_gamma) : 0.0f;
  float g = c.y > 0.0f ? powf(c.y, inv_gamma) : 0.0f;
  float b = c.z > 0.0f ? powf(c.z, inv_gamma) : 0.0f;
  out[i] = make_uchar4(to_unorm8(r), to_unorm8(g), to_unorm8(b), 255);
}

}  // namespace

cudaError_t launch_export(const float *in, uint32_t n, float gamma, uint8_t *out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_export<<<(n + 255) / 256, 256, 0, st>>>(reinterpret_cast<const float4 *>(in), n, 1.0f / gamma,
                                             reinterpret_cast<uchar4 *>(out));
  return cudaGetLastError();
}

}  // namespace rtgb
