// Autotuner for the context's launch-shape knobs (rtAutotuneTrace,
// rtAutotuneRender in rt_api.h). Every knob it touches leaves results
// unchanged (hits and images are identical in every shape), so tuning is a
// pure timing search on the caller's own workload:
//   closest hit  coordinate descent over trace.block (threads per block,
//                64/128/256), trace.stack (traversal stack entries 16/32/64,
//                each raised to the smallest size that holds the tree),
//                trace.wide, trace.wide_minblocks, trace.wide_visits, trace.defer, trace.spec,
//                trace.minblocks, trace.packet_minblocks, trace.sort and
//                trace.beam,
//                each candidate timed with CUDA events over `reps` casts
//                after one warm-up cast;
//   render       megakernel against wavefront at growing square image sizes
//                on the scene's camera; render.wavefront_pixels becomes the
//                smallest size from which the wavefront wins.
// The reference fixes the launch shape at compile time (local_size 32x32,
// ray-trace-compute.comp:3) and the stack at 16 entries (comp:262).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "rt_internal.h"
#include "rtgb/rt_api.h"

using namespace rtgb;

namespace {

// Milliseconds per cast of the batch with the context's current settings.
rt_status time_trace(rt_ctx *ctx, rt_scene_id scene, const rt_ray *rays, uint32_t n, rt_hit *hits, uint32_t reps,
                     float *ms) {
  cudaStream_t st = ctx_stream(ctx);
  rt_status s = rtTraceClosestEx(ctx, scene, rays, n, hits, 0, nullptr);
  if (s != RT_SUCCESS) return s;
  cudaEvent_t a = nullptr, b = nullptr;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
    if (a) cudaEventDestroy(a);
    return RT_ERR_CUDA;
  }
  cudaEventRecord(a, st);
  for (uint32_t r = 0; r < reps && s == RT_SUCCESS; r++) s = rtTraceClosestEx(ctx, scene, rays, n, hits, 0, nullptr);
  cudaEventRecord(b, st);
  cudaError_t e = cudaEventSynchronize(b);
  float total = 0.0f;
  if (e == cudaSuccess) cudaEventElapsedTime(&total, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (s != RT_SUCCESS) return s;
  if (e != cudaSuccess) return RT_ERR_CUDA;
  *ms = total / (float)reps;
  return rtSynchronize(ctx, nullptr);
}

rt_status time_render(rt_ctx *ctx, rt_scene_id scene, uint32_t side, uint32_t spp, uint32_t bounces, float *accum,
                      float *ms) {
  cudaStream_t st = ctx_stream(ctx);
  rt_render_params p{side, side, spp, bounces, 0, 0, {0, 0}};
  rt_status s = rtRender(ctx, scene, &p, accum, nullptr);
  if (s != RT_SUCCESS) return s;
  cudaEvent_t a = nullptr, b = nullptr;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
    if (a) cudaEventDestroy(a);
    return RT_ERR_CUDA;
  }
  cudaEventRecord(a, st);
  for (int r = 0; r < 2 && s == RT_SUCCESS; r++) {
    p.sample_index = spp * (r + 1);
    s = rtRender(ctx, scene, &p, accum, nullptr);
  }
  cudaEventRecord(b, st);
  cudaError_t e = cudaEventSynchronize(b);
  float total = 0.0f;
  if (e == cudaSuccess) cudaEventElapsedTime(&total, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (s != RT_SUCCESS) return s;
  if (e != cudaSuccess) return RT_ERR_CUDA;
  *ms = total / 2.0f;
  return rtSynchronize(ctx, nullptr);
}

}  // namespace

extern "C" {

rt_status rtAutotuneTrace(rt_ctx *ctx, rt_scene_id scene, const rt_ray *d_rays, uint32_t n, rt_hit *d_hits,
                          uint32_t reps, double *start_grays, double *best_grays) {
  if (!ctx || !d_rays || !d_hits || n == 0 || reps == 0 || reps > 1000) return RT_ERR_INVALID_ARGUMENT;
  struct Knob {
    const char *key;
    std::vector<int64_t> values;
  };
  const Knob knobs[] = {{"trace.block", {128, 64, 256}},
                        {"trace.stack", {0, 32, 64}},
                        {"trace.wide", {1, 0}},
                        {"trace.wide_minblocks", {8, 7, 6, 5}},
                        {"trace.wide_visits", {3, 2, 1}},
                        {"trace.defer", {1, 0}},
                        {"trace.spec", {1, 0}},
                        {"trace.minblocks", {16, 12, 10}},
                        {"trace.packet_minblocks", {16, 12, 10}},
                        {"trace.sort", {1, 0}},
                        {"trace.beam", {0, 2, 1}}};
  float best = 0.0f;
  rt_status s = time_trace(ctx, scene, d_rays, n, d_hits, reps, &best);
  if (s != RT_SUCCESS) return s;
  if (start_grays) *start_grays = (double)n / best / 1e6;
  for (const Knob &k : knobs) {
    int64_t keep = 0;
    if ((s = rtGetTuning(ctx, k.key, &keep)) != RT_SUCCESS) return s;
    int64_t choice = keep;
    for (int64_t v : k.values) {
      if (v == keep) continue;
      if ((s = rtSetTuning(ctx, k.key, v)) != RT_SUCCESS) return s;
      float ms = 0.0f;
      if ((s = time_trace(ctx, scene, d_rays, n, d_hits, reps, &ms)) != RT_SUCCESS) {
        rtSetTuning(ctx, k.key, keep);
        return s;
      }
      if (ms < best) {
        best = ms;
        choice = v;
      }
    }
    if ((s = rtSetTuning(ctx, k.key, choice)) != RT_SUCCESS) return s;
  }
  if (best_grays) *best_grays = (double)n / best / 1e6;
  return RT_SUCCESS;
}

rt_status rtAutotuneRender(rt_ctx *ctx, rt_scene_id scene, uint32_t spp, uint32_t max_bounces,
                           uint32_t max_side, uint64_t *wavefront_pixels) {
  if (!ctx || spp == 0 || max_bounces == 0 || max_side < 256 || max_side > 4096) return RT_ERR_INVALID_ARGUMENT;
  int64_t old_mode = 2, old_px = 0;
  rt_status s = rtGetTuning(ctx, "render.mode", &old_mode);
  if (s == RT_SUCCESS) s = rtGetTuning(ctx, "render.wavefront_pixels", &old_px);
  if (s != RT_SUCCESS) return s;
  float *accum = nullptr;
  cudaError_t e = cudaMalloc((void **)&accum, 16ull * max_side * max_side);
  if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? RT_ERR_OUT_OF_MEMORY : RT_ERR_CUDA;
  // Smallest size from which the wavefront wins; 2^31 when it never does.
  int64_t threshold = 1ll << 31;
  for (uint32_t side = 256; side <= max_side && s == RT_SUCCESS; side *= 2) {
    float ms[2] = {0.0f, 0.0f};
    for (int mode = 0; mode < 2 && s == RT_SUCCESS; mode++) {
      s = rtSetTuning(ctx, "render.mode", mode);
      if (s == RT_SUCCESS) s = time_render(ctx, scene, side, spp, max_bounces, accum, &ms[mode]);
    }
    if (s == RT_SUCCESS && ms[1] < ms[0]) {
      threshold = (int64_t)side * side;
      break;
    }
  }
  cudaFree(accum);
  rtSetTuning(ctx, "render.mode", old_mode);
  if (s != RT_SUCCESS) return s;
  s = rtSetTuning(ctx, "render.wavefront_pixels", threshold);
  if (s == RT_SUCCESS && wavefront_pixels) *wavefront_pixels = (uint64_t)threshold;
  (void)old_px;
  return s;
}

}  // extern "C"
