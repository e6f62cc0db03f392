// Megakernel render: one thread per pixel runs the whole bounce loop of
// ray-trace-compute.comp:main (352-380) for every sample of the call.
// Threads are laid out as 8 x 4 pixel tiles per warp so camera rays of a warp
// are coherent. The number of traced segments (camera + secondary rays) is
// reduced per warp and added to a 64-bit counter for throughput reporting.
#include <cuda_runtime.h>

#include "rt_internal.h"
#include "shade.cuh"

namespace rtgb {
namespace {

constexpr int kTileX = 8, kTileY = 16;  // 128 threads; each warp covers 8 x 4 pixels

__device__ __forceinline__ void count_segments(uint32_t seg, unsigned long long *counter) {
  uint32_t lane = threadIdx.x + threadIdx.y * blockDim.x;
  lane &= 31;
  for (int o = 16; o > 0; o >>= 1) seg += __shfl_down_sync(0xffffffffu, seg, o);
  if (lane == 0 && counter) atomicAdd(counter, (unsigned long long)seg);
}

template <int STACK>
__global__ void __launch_bounds__(kTileX *kTileY) k_render(DevScene sc, rt_camera cam, rt_render_params p,
                                                           float4 *accum, unsigned long long *segments,
                                                           uint32_t *err) {
  uint32_t x = blockIdx.x * kTileX + threadIdx.x;
  uint32_t y = blockIdx.y * kTileY + threadIdx.y;
  uint32_t seg = 0;
  if (x < p.width && y < p.height) {
    PathState ps = path_state(sc, p.flags);
    seg = render_pixel<STACK>(sc, ps, cam, p, x, y, accum, err);
  }
  count_segments(seg, segments);
}

}  // namespace

cudaError_t launch_render(const DevScene &sc, const rt_camera &cam, const rt_render_params &p, float *accum,
                          unsigned long long *segments, uint32_t *err, cudaStream_t st) {
  if (p.width == 0 || p.height == 0 || p.spp == 0) return cudaSuccess;
  dim3 block(kTileX, kTileY);
  dim3 grid((p.width + kTileX - 1) / kTileX, (p.height + kTileY - 1) / kTileY);
  if (sc.depth <= 32) {
    k_render<32><<<grid, block, 0, st>>>(sc, cam, p, reinterpret_cast<float4 *>(accum), segments, err);
  } else {
    k_render<64><<<grid, block, 0, st>>>(sc, cam, p, reinterpret_cast<float4 *>(accum), segments, err);
  }
  return cudaGetLastError();
}

}  // namespace rtgb
