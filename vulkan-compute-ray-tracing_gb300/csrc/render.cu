// Megakernel render: one thread per pixel runs the whole bounce loop of
// ray-trace-compute.comp:main (352-380) for every sample of the call.
// Threads are laid out as 8 x 4 pixel tiles per warp so camera rays of a warp
// are coherent: a warp traces its camera segment as one packet, once per
// call (render_pixel). The number of traced segments (camera + secondary rays) is
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
  __shared__ int s_stack[kTileX * kTileY / 32][STACK];
  const uint32_t warp = (threadIdx.y * kTileX + threadIdx.x) >> 5;
  uint32_t x = blockIdx.x * kTileX + threadIdx.x;
  uint32_t y = blockIdx.y * kTileY + threadIdx.y;
  const bool active = x < p.width && y < p.height;
  PathState ps = path_state(sc, p.flags);
  uint32_t seg = render_pixel<STACK>(sc, ps, cam, p, x, y, active, accum, err, s_stack[warp]);
  count_segments(seg, segments);
}

// Many renders in one persistent launch: every job is cut into 8 x 16 pixel
// tiles numbered consecutively across jobs (job j owns tiles
// [tile_begin_j, tile_begin_j+1)); blocks claim tiles from a global counter
// until none are left, so small and large jobs share the GPU without a
// launch per job and no SM idles while another job still has tiles.
template <int STACK>
__global__ void __launch_bounds__(kTileX *kTileY) k_render_batch(const BatchJob *__restrict__ jobs, uint32_t njobs,
                                                                 uint32_t total_tiles, uint32_t *counter,
                                                                 unsigned long long *segments, uint32_t *err) {
  __shared__ uint32_t s_tile;
  __shared__ int s_stack[kTileX * kTileY / 32][STACK];
  const uint32_t warp = (threadIdx.y * kTileX + threadIdx.x) >> 5;
  const bool leader = threadIdx.x == 0 && threadIdx.y == 0;
  for (;;) {
    if (leader) s_tile = atomicAdd(counter, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    __syncthreads();
    if (tile >= total_tiles) return;
    uint32_t lo = 0, hi = njobs;
    while (hi - lo > 1) {
      uint32_t m = (lo + hi) >> 1;
      if (jobs[m].tile_begin <= tile) lo = m; else hi = m;
    }
    const BatchJob &J = jobs[lo];
    const DevScene sc = J.sc;
    const rt_render_params p = J.p;
    const uint32_t local = tile - J.tile_begin;
    const uint32_t x = (local % J.tiles_x) * kTileX + threadIdx.x;
    const uint32_t y = (local / J.tiles_x) * kTileY + threadIdx.y;
    const bool active = x < p.width && y < p.height;
    PathState ps = path_state(sc, p.flags);
    uint32_t seg =
        render_pixel<STACK>(sc, ps, J.cam, p, x, y, active, reinterpret_cast<float4 *>(J.accum), err, s_stack[warp]);
    count_segments(seg, segments);
  }
}

__global__ void k_batch_advance(BatchJob *jobs, uint32_t njobs) {
  uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < njobs) jobs[j].p.sample_index += jobs[j].p.spp;
}

int g_render_sms = 0;

}  // namespace

cudaError_t launch_batch_advance(BatchJob *d_jobs, uint32_t n_jobs, cudaStream_t st) {
  if (n_jobs == 0) return cudaSuccess;
  k_batch_advance<<<(n_jobs + 255) / 256, 256, 0, st>>>(d_jobs, n_jobs);
  return cudaGetLastError();
}

uint32_t batch_tiles_x(uint32_t width) { return (width + kTileX - 1) / kTileX; }
uint32_t batch_tiles(uint32_t width, uint32_t height) {
  return batch_tiles_x(width) * ((height + kTileY - 1) / kTileY);
}

cudaError_t launch_render_batch(const BatchJob *d_jobs, uint32_t n_jobs, uint32_t total_tiles, uint32_t max_depth,
                                uint32_t *counter, unsigned long long *segments, uint32_t *err, cudaStream_t st) {
  if (n_jobs == 0 || total_tiles == 0) return cudaSuccess;
  if (g_render_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_render_sms, cudaDevAttrMultiProcessorCount, dev);
  }
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  int bps = 0;
  dim3 block(kTileX, kTileY);
  if (max_depth <= 32)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_render_batch<32>, kTileX * kTileY, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_render_batch<64>, kTileX * kTileY, 0);
  uint32_t grid = (uint32_t)(g_render_sms * (bps > 0 ? bps : 1));
  if (grid > total_tiles) grid = total_tiles;
  if (max_depth <= 32)
    k_render_batch<32><<<grid, block, 0, st>>>(d_jobs, n_jobs, total_tiles, counter, segments, err);
  else
    k_render_batch<64><<<grid, block, 0, st>>>(d_jobs, n_jobs, total_tiles, counter, segments, err);
  return cudaGetLastError();
}

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
