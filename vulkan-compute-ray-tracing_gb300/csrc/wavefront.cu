// Wavefront render: the bounce loop of ray-trace-compute.comp:314-338 split
// into kernels over queues of live paths.
//
//   raygen      one path per pixel for sample s (colour 1, the pixel's RNG
//               seed, the normalised camera ray) -> queue 0
//   per bounce  [Morton reorder of the queue's rays, render.sort] -> extend (closest
//               triangle per ray) -> shade (record, spheres, scatter, colour;
//               surviving paths are compacted into the other queue)
//   accumulate  the running mean of comp:375-377 for sample s
//
// Every floating-point step is the megakernel's (shade.cuh); only the order
// in which paths are processed changes, so images are identical to the
// megakernel's. What the split buys: finished paths leave the queue instead
// of idling lanes, the casting kernel runs without the shading code's
// registers, and each bounce's rays reach the 8-wide caster, whose warps
// refill from the queue (in the order shading queued them, or in Morton
// order when render.sort is set). Queue lengths stay on the device;
// kernels are sized for the queue's capacity and read the live count, so a
// render is a fixed launch sequence (no host synchronisation, capturable in
// a CUDA graph).
#include <cuda_runtime.h>

#include "rt_internal.h"
#include "shade.cuh"

namespace rtgb {
namespace {

constexpr int kWfBlock = 128;

struct WfBufs {
  rt_ray *rays[2];
  uint32_t *slots[2];
  int2 *hits;
  int2 *cam_hits;  // bounce-0 hits of the call's first sample, reused by the others
  float4 *color;
  uint32_t *rng;
  uint32_t *counts;  // [0], [1]: queue lengths; [2] listed chunks, [3] wide-caster counter
  uint32_t *list;    // chunks of the queue left to the 8-wide caster
  void *sort;
};

size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

WfBufs carve(void *scratch, uint32_t cap) {
  char *p = static_cast<char *>(scratch);
  WfBufs b;
  for (int i = 0; i < 2; i++) {
    b.rays[i] = reinterpret_cast<rt_ray *>(p);
    p += a256(sizeof(rt_ray) * (size_t)cap);
    b.slots[i] = reinterpret_cast<uint32_t *>(p);
    p += a256(4ull * cap);
  }
  b.hits = reinterpret_cast<int2 *>(p);
  p += a256(8ull * cap);
  b.cam_hits = reinterpret_cast<int2 *>(p);
  p += a256(8ull * cap);
  b.color = reinterpret_cast<float4 *>(p);
  p += a256(16ull * cap);
  b.rng = reinterpret_cast<uint32_t *>(p);
  p += a256(4ull * cap);
  b.counts = reinterpret_cast<uint32_t *>(p);
  p += 256;
  b.list = reinterpret_cast<uint32_t *>(p);
  p += a256(4ull * ((cap + 31) / 32));
  b.sort = p;
  return b;
}

// Sample index of this pass: s, or *d_s + s when the index lives on the
// device (batched jobs advanced by a captured graph).
__device__ __forceinline__ uint32_t sample_of(uint32_t s, const uint32_t *d_s) { return d_s ? *d_s + s : s; }

__global__ void k_wf_raygen(rt_camera cam, uint32_t W, uint32_t H, uint32_t s, const uint32_t *d_s, rt_ray *rays,
                            uint32_t *slots, float4 *color, uint32_t *rng, uint32_t *count) {
  s = sample_of(s, d_s);
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p == 0) *count = W * H;
  if (p >= W * H) return;
  uint32_t x = p % W, y = p / W;
  f3 d = normalize3(camera_dir(cam, x, y, W, H));
  rays[p] = rt_ray{{cam.origin[0], cam.origin[1], cam.origin[2]}, kTmin, {d.x, d.y, d.z}, kTmax};
  slots[p] = p;
  color[p] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
  rng[p] = (600u * x + y) * (s + 1u);
}

// Closest triangle per queued ray. A warp whose 32 rays are coherent (the
// camera rays of bounce 0 in pixel order, or any bundle sharing an origin)
// traverses them as one packet; other warps list their chunk for the 8-wide
// caster (list != NULL) or run each lane's ray with postponed leaves. All
// return every ray's own closest hit.
template <int STACK>
__global__ void __launch_bounds__(kWfBlock, 12) k_wf_extend(DevScene sc, const float4 *__restrict__ rays,
                                                            uint32_t cap, const uint32_t *count,
                                                            const uint32_t *__restrict__ perm,
                                                            int2 *__restrict__ hits, uint32_t *counter,
                                                            uint32_t *err, uint32_t *__restrict__ list,
                                                            uint32_t *__restrict__ list_count) {
  __shared__ int s_stack[kWfBlock / 32][STACK];
  const uint32_t n = min(cap, *count);
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(counter, 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n) return;
    uint32_t i = base + lane;
    const bool active = i < n;
    f3 o = mk3(0.0f, 0.0f, 0.0f), d = mk3(1.0f, 0.0f, 0.0f);
    float tmin = 0.0f, closest = 0.0f;
    if (active) {
      if (perm) i = __ldg(perm + i);
      float4 r0 = __ldg(rays + 2ull * i), r1 = __ldg(rays + 2ull * i + 1);
      o = mk3(r0.x, r0.y, r0.z);
      d = mk3(r1.x, r1.y, r1.z);
      tmin = r0.w;
      closest = r1.w;
    }
    TraceRay r = make_ray(o, d, tmin);
    float u = 0.0f, v = 0.0f;
    int k;
    const int oct = warp_octant(active, r);
    if (warp_is_coherent(active, r)) {
#define RTGB_CALL(O) k = traverse_packet<STACK, O>(sc, r, active, closest, u, v, s_stack[warp], err)
      RTGB_OCT_DISPATCH(oct, RTGB_CALL)
#undef RTGB_CALL
    } else if (list) {
      if (lane == 0) list[atomicAdd(list_count, 1u)] = base;
      continue;
    } else {
#define RTGB_CALL(O) k = traverse_spec<STACK, O>(sc, r, active, closest, u, v, err)
      RTGB_OCT_DISPATCH(oct, RTGB_CALL)
#undef RTGB_CALL
    }
    if (active) hits[i] = make_int2(k, __float_as_int(closest));
  }
}

__global__ void __launch_bounds__(kWfBlock) k_wf_shade(DevScene sc, uint32_t flags, const rt_ray *__restrict__ rays_in,
                                                       const uint32_t *__restrict__ slots_in, const uint32_t *count_in,
                                                       const int2 *__restrict__ hits, float4 *color, uint32_t *rng,
                                                       rt_ray *rays_out, uint32_t *slots_out, uint32_t *count_out,
                                                       int last, unsigned long long *segments) {
  const uint32_t n = *count_in;
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q == 0 && segments) atomicAdd(segments, (unsigned long long)n);
  bool push = false;
  HitRec rec;
  f3 nd;
  uint32_t s = 0;
  if (q < n) {
    PathState ps = path_state(sc, flags);
    s = slots_in[q];
    const rt_ray ray = rays_in[q];
    f3 o = ld3(ray.o), d = ld3(ray.d);
    int2 h = hits[q];
    float4 c4 = color[s];
    f3 c = mk3(c4.x, c4.y, c4.z);
    if (!resolve_hit(sc, ps, o, d, h.x, __int_as_float(h.y), rec)) {
      c = mul3(0.0f, c);
    } else {
      Rng g{rng[s]};
      f3 albedo;
      bool emits = scatter(sc, ps, d, rec, g, albedo, nd);
      c = mulv3(c, albedo);
      rng[s] = g.s;
      push = !emits && !last;
    }
    color[s] = make_float4(c.x, c.y, c.z, 0.0f);
  }
  // Warp-aggregated append of the surviving paths.
  const uint32_t lane = threadIdx.x & 31;
  uint32_t mask = __ballot_sync(0xffffffffu, push);
  if (mask) {
    uint32_t base = 0;
    uint32_t leader = __ffs(mask) - 1;
    if (lane == leader) base = atomicAdd(count_out, (uint32_t)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (push) {
      uint32_t pos = base + __popc(mask & ((1u << lane) - 1u));
      rays_out[pos] = rt_ray{{rec.p.x, rec.p.y, rec.p.z}, kTmin, {nd.x, nd.y, nd.z}, kTmax};
      slots_out[pos] = s;
    }
  }
}

__global__ void k_wf_accumulate(uint32_t W, uint32_t H, uint32_t s, const uint32_t *d_s, uint32_t flags,
                                const float4 *__restrict__ color, float4 *accum) {
  s = sample_of(s, d_s);
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= W * H) return;
  float4 c = color[p];
  float4 acc = accum[p];
  float sf = (float)s;
  float keep = gmin(sf, 1.0f);
  float den = __fadd_rn(sf, 1.0f);
  acc.x = __fdiv_rn(__fadd_rn(c.x, __fmul_rn(__fmul_rn(acc.x, keep), sf)), den);
  acc.y = __fdiv_rn(__fadd_rn(c.y, __fmul_rn(__fmul_rn(acc.y, keep), sf)), den);
  acc.z = __fdiv_rn(__fadd_rn(c.z, __fmul_rn(__fmul_rn(acc.z, keep), sf)), den);
  acc.w = __fdiv_rn(__fadd_rn(1.0f, __fmul_rn(__fmul_rn(acc.w, keep), sf)), den);
  if (flags & RT_COMPAT_UNORM8) {
    acc.x = unorm8(acc.x);
    acc.y = unorm8(acc.y);
    acc.z = unorm8(acc.z);
    acc.w = unorm8(acc.w);
  }
  accum[p] = acc;
}

int g_sms = 0;

}  // namespace

size_t wavefront_scratch_bytes(uint32_t cap) {
  return 2 * (a256(sizeof(rt_ray) * (size_t)cap) + a256(4ull * cap)) + 2 * a256(8ull * cap) + a256(16ull * cap) +
         a256(4ull * cap) + 256 + a256(4ull * ((cap + 31) / 32)) + a256(raysort_scratch_bytes(cap));
}

cudaError_t launch_render_wavefront(const DevScene &sc, const rt_camera &cam, const rt_render_params &p, float *accum,
                                    unsigned long long *segments, uint32_t *counter, uint32_t *err, void *scratch,
                                    bool sort, bool wide, cudaStream_t st, const uint32_t *d_sample_index) {
  const uint32_t W = p.width, H = p.height, cap = W * H;
  if (cap == 0 || p.spp == 0) return cudaSuccess;
  const bool use_wide = wide && wide_ok(sc);
  if (g_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
  }
  WfBufs b = carve(scratch, cap);
  const uint32_t grid = (cap + kWfBlock - 1) / kWfBlock;
  int bps = 0;
  if (sc.depth <= 32)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_wf_extend<32>, kWfBlock, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_wf_extend<64>, kWfBlock, 0);
  uint32_t egrid = (uint32_t)(g_sms * (bps > 0 ? bps : 1));
  if (egrid > grid) egrid = grid;
  cudaError_t e = cudaSuccess;
  for (uint32_t k = 0; k < p.spp; k++) {
    const uint32_t s = d_sample_index ? k : p.sample_index + k;
    k_wf_raygen<<<grid, kWfBlock, 0, st>>>(cam, W, H, s, d_sample_index, b.rays[0], b.slots[0], b.color, b.rng,
                                           b.counts);
    for (uint32_t bounce = 0; bounce < p.max_bounces; bounce++) {
      const int in = bounce & 1, out = in ^ 1;
      if ((e = cudaMemsetAsync(b.counts + out, 0, 4, st)) != cudaSuccess) return e;
      // Camera rays carry no jitter: bounce 0 is the same for every sample
      // of the call (queue slot = pixel), so later samples reuse its hits.
      if (bounce == 0 && k > 0) {
        k_wf_shade<<<grid, kWfBlock, 0, st>>>(sc, p.flags, b.rays[in], b.slots[in], b.counts + in, b.cam_hits,
                                              b.color, b.rng, b.rays[out], b.slots[out], b.counts + out,
                                              bounce + 1 == p.max_bounces, nullptr);
        continue;
      }
      uint32_t *perm = nullptr;
      if (sort && (e = launch_raysort(b.rays[in], cap, b.counts + in, b.sort, &perm, st)) != cudaSuccess) return e;
      if ((e = cudaMemsetAsync(counter, 0, 4, st)) != cudaSuccess) return e;
      const float4 *r4 = reinterpret_cast<const float4 *>(b.rays[in]);
      uint32_t *list = use_wide ? b.list : nullptr;
      if (use_wide && (e = cudaMemsetAsync(b.counts + 2, 0, 8, st)) != cudaSuccess) return e;
      if (sc.depth <= 32)
        k_wf_extend<32><<<egrid, kWfBlock, 0, st>>>(sc, r4, cap, b.counts + in, perm, b.hits, counter, err, list,
                                                    b.counts + 2);
      else
        k_wf_extend<64><<<egrid, kWfBlock, 0, st>>>(sc, r4, cap, b.counts + in, perm, b.hits, counter, err, list,
                                                    b.counts + 2);
      if (use_wide &&
          (e = launch_wide_leaf(sc, b.rays[in], cap, b.counts + in, perm, b.list, b.counts + 2, b.hits,
                                b.counts + 3, err, 6, 4, st)) != cudaSuccess)
        return e;
      if (bounce == 0 && p.spp > 1 &&
          (e = cudaMemcpyAsync(b.cam_hits, b.hits, 8ull * cap, cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
        return e;
      k_wf_shade<<<grid, kWfBlock, 0, st>>>(sc, p.flags, b.rays[in], b.slots[in], b.counts + in, b.hits, b.color,
                                            b.rng, b.rays[out], b.slots[out], b.counts + out,
                                            bounce + 1 == p.max_bounces, segments);
    }
    k_wf_accumulate<<<grid, kWfBlock, 0, st>>>(W, H, s, d_sample_index, p.flags, b.color,
                                               reinterpret_cast<float4 *>(accum));
  }
  return cudaGetLastError();
}

}  // namespace rtgb
