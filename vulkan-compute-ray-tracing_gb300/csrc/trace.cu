// Closest-hit ray casting: one thread per ray, rays fetched by warps from a
// global work counter (persistent launch sized to the SM count), so warps
// that finish early pick up new rays instead of idling behind long ones.
#include <cuda_runtime.h>

#include "rt_internal.h"
#include "shade.cuh"
#include "traverse.cuh"

namespace rtgb {
namespace {

constexpr int kTraceBlock = 128;
constexpr int kBatch = 32;  // rays a warp takes per fetch

template <int STACK>
__global__ void __launch_bounds__(kTraceBlock) k_trace(DevScene sc, const float4 *__restrict__ rays, uint32_t n,
                                                       int4 *__restrict__ hits, uint32_t *__restrict__ counter,
                                                       uint32_t *err) {
  const uint32_t lane = threadIdx.x & 31;
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(counter, kBatch);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n) return;
    uint32_t i = base + lane;
    if (i < n) {
      float4 r0 = __ldg(rays + 2ull * i), r1 = __ldg(rays + 2ull * i + 1);
      TraceRay r = make_ray(mk3(r0.x, r0.y, r0.z), mk3(r1.x, r1.y, r1.z), r0.w);
      float closest = r1.w, u = 0.0f, v = 0.0f;
      int k = traverse_closest<STACK>(sc, r, closest, u, v, err);
      int4 h;
      if (k >= 0) {
        h = make_int4(__ldg(sc.leaf_tri + k), __float_as_int(closest), __float_as_int(u), __float_as_int(v));
      } else {
        h = make_int4(-1, 0, 0, 0);
      }
      hits[i] = h;
    }
  }
}

// RT_COMPAT_STACK16: the shader's literal traversal, one thread per ray.
__global__ void __launch_bounds__(kTraceBlock) k_trace_literal16(DevScene sc, const float4 *__restrict__ rays,
                                                                 uint32_t n, int4 *__restrict__ hits) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 r0 = __ldg(rays + 2ull * i), r1 = __ldg(rays + 2ull * i + 1);
  float closest = r1.w, u = 0.0f, v = 0.0f;
  int t = traverse_literal16(sc, mk3(r0.x, r0.y, r0.z), mk3(r1.x, r1.y, r1.z), r0.w, closest, u, v);
  hits[i] = t >= 0 ? make_int4(t, __float_as_int(closest), __float_as_int(u), __float_as_int(v))
                   : make_int4(-1, 0, 0, 0);
}

int g_num_sms = 0;

}  // namespace

cudaError_t launch_trace_literal16(const DevScene &sc, const rt_ray *rays, uint32_t n, rt_hit *hits,
                                   cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_trace_literal16<<<(n + kTraceBlock - 1) / kTraceBlock, kTraceBlock, 0, st>>>(
      sc, reinterpret_cast<const float4 *>(rays), n, reinterpret_cast<int4 *>(hits));
  return cudaGetLastError();
}

cudaError_t launch_trace(const DevScene &sc, const rt_ray *rays, uint32_t n, rt_hit *hits, uint32_t *counter,
                         uint32_t *err, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  if (g_num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
  }
  // The work counter is private to this launch; reset it in stream order.
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  int blocks_per_sm = 0;
  if (sc.depth <= 32) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_trace<32>, kTraceBlock, 0);
  } else {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_trace<64>, kTraceBlock, 0);
  }
  if (blocks_per_sm < 1) blocks_per_sm = 1;
  uint32_t want = (n + kTraceBlock - 1) / kTraceBlock;
  uint32_t grid = (uint32_t)(g_num_sms * blocks_per_sm);
  if (grid > want) grid = want;
  if (sc.depth <= 32) {
    k_trace<32><<<grid, kTraceBlock, 0, st>>>(sc, reinterpret_cast<const float4 *>(rays), n,
                                              reinterpret_cast<int4 *>(hits), counter, err);
  } else {
    k_trace<64><<<grid, kTraceBlock, 0, st>>>(sc, reinterpret_cast<const float4 *>(rays), n,
                                              reinterpret_cast<int4 *>(hits), counter, err);
  }
  return cudaGetLastError();
}

}  // namespace rtgb
