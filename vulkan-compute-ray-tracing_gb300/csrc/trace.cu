// Closest-hit ray casting: one thread per ray, rays fetched by warps from a
// global work counter (persistent launch sized to the SM count), so warps
// that finish early pick up new rays instead of idling behind long ones.
//
// The hit is chosen with the reference's fp32 arithmetic (traverse.cuh).
// Unless RT_HIT_FP32 is set, t, u, v of the chosen triangle are then
// recomputed once in fp64 with the same triIntersect formula
// (ray-trace-compute.comp:157-173) and rounded to fp32, which removes the
// cancellation error the fp32 formula shows at grazing angles.
#include <cuda_runtime.h>

#include <climits>

#include "rt_internal.h"
#include "shade.cuh"
#include "traverse.cuh"

namespace rtgb {
namespace {

constexpr int kTraceBlock = 128;


struct d3 {
  double x, y, z;
};
__device__ __forceinline__ d3 dsub(d3 a, d3 b) { return d3{__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z)}; }
__device__ __forceinline__ double ddot(d3 a, d3 b) {
  return __dadd_rn(__dadd_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)), __dmul_rn(a.z, b.z));
}
__device__ __forceinline__ d3 dcross(d3 a, d3 b) {
  return d3{__dsub_rn(__dmul_rn(a.y, b.z), __dmul_rn(b.y, a.z)), __dsub_rn(__dmul_rn(a.z, b.x), __dmul_rn(b.z, a.x)),
            __dsub_rn(__dmul_rn(a.x, b.y), __dmul_rn(b.x, a.y))};
}

// triIntersect in fp64 on the original vertices (fp32 inputs widened).
__device__ __forceinline__ void refine_fp64(const rt_triangle *__restrict__ tris, int tri, f3 o, f3 d, float &t,
                                            float &u, float &v) {
  const float4 *T = reinterpret_cast<const float4 *>(tris + tri);
  float4 a4 = __ldg(T), b4 = __ldg(T + 1), c4 = __ldg(T + 2);
  d3 v0{a4.x, a4.y, a4.z}, v1{b4.x, b4.y, b4.z}, v2{c4.x, c4.y, c4.z};
  d3 ro{o.x, o.y, o.z}, rd{d.x, d.y, d.z};
  d3 a = dsub(v0, v1), b = dsub(v2, v0), p = dsub(v0, ro);
  d3 n = dcross(b, a);
  d3 q = dcross(p, rd);
  double idet = __ddiv_rn(1.0, ddot(rd, n));
  u = __double2float_rn(__dmul_rn(ddot(q, b), idet));
  v = __double2float_rn(__dmul_rn(ddot(q, a), idet));
  t = __double2float_rn(__dmul_rn(ddot(n, p), idet));
}

constexpr int kDone = INT_MIN;  // no node left: the ray is finished

// Persistent warps with per-lane refill: each lane owns one ray at a time;
// when at least `refill` lanes of a warp have finished, the warp claims that
// many new rays with one atomic and the idle lanes start on them, so a warp
// never waits for its slowest ray with most lanes idle. Traversal runs as
// while-while: descend inner nodes until every active lane holds a leaf,
// then test those triangles together.
template <int STACK, bool REFINE>
__global__ void __launch_bounds__(kTraceBlock) k_trace(DevScene sc, const float4 *__restrict__ rays, uint32_t n,
                                                       int4 *__restrict__ hits, uint32_t *__restrict__ counter,
                                                       uint32_t *err, int refill, const uint32_t *__restrict__ perm) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t lt_mask = (1u << lane) - 1u;
  const float4 *__restrict__ bvh = sc.bvh2;
  int stack[STACK];
  int sp = 0, node = kDone, best = -1;
  int64_t ray_id = -1;
  float closest = 0.0f, bu = 0.0f, bv = 0.0f;
  TraceRay r;
  r.tmin = 0.0f;
  bool exhausted = false;
  for (;;) {
    const uint32_t idle = __ballot_sync(0xffffffffu, ray_id < 0);
    if (!exhausted && __popc(idle) >= refill) {
      const uint32_t cnt = __popc(idle);
      const uint32_t leader = __ffs(idle) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(counter, cnt);
      base = __shfl_sync(0xffffffffu, base, leader);
      if (base + cnt >= n) exhausted = true;
      if (ray_id < 0) {
        uint32_t my = base + __popc(idle & lt_mask);
        if (my < n) {
          if (perm) my = __ldg(perm + my);
          float4 r0 = __ldg(rays + 2ull * my), r1 = __ldg(rays + 2ull * my + 1);
          r = make_ray(mk3(r0.x, r0.y, r0.z), mk3(r1.x, r1.y, r1.z), r0.w);
          closest = r1.w;
          best = -1;
          sp = 0;
          ray_id = my;
          float root = slab_enter(r, sc.root_lo[0], sc.root_hi[0], sc.root_lo[1], sc.root_hi[1], sc.root_lo[2],
                                  sc.root_hi[2], closest);
          node = root < __int_as_float(0x7f800000) ? sc.root_ref : kDone;
        }
      }
    }
    // Leave only when no lane holds a ray after this round's fetch.
    if (exhausted && __all_sync(0xffffffffu, ray_id < 0)) return;
    if (ray_id >= 0) {
      // Inner nodes until this lane holds a leaf or runs out of work.
      while (node >= 0) {
        const float4 *N = bvh + 4ll * node;
        float4 a = __ldg(N), b = __ldg(N + 1), c = __ldg(N + 2), d = __ldg(N + 3);
        float t0 = slab_enter(r, a.x, a.y, a.z, a.w, c.x, c.y, closest);
        float t1 = slab_enter(r, b.x, b.y, b.z, b.w, c.z, c.w, closest);
        int r0 = __float_as_int(d.x), r1 = __float_as_int(d.y);
        bool h0 = t0 < __int_as_float(0x7f800000), h1 = t1 < __int_as_float(0x7f800000);
        if (h0 && h1) {
          int nearc = r0, farc = r1;
          if (t1 < t0) {
            nearc = r1;
            farc = r0;
          }
          if (sp >= STACK) {
            atomicOr(err, KERR_STACK_OVERFLOW);
            node = kDone;
            break;
          }
          stack[sp++] = farc;
          node = nearc;
        } else if (h0) {
          node = r0;
        } else if (h1) {
          node = r1;
        } else {
          node = sp > 0 ? stack[--sp] : kDone;
        }
      }
      if (node != kDone) {
        test_triangle(sc.tpre, sc.leaf_tri, ~node, r, closest, best, bu, bv);
        node = sp > 0 ? stack[--sp] : kDone;
      }
      if (node == kDone) {
        int4 h;
        if (best >= 0) {
          int tri = __ldg(sc.leaf_tri + best);
          float t = closest, u = bu, v = bv;
          if (REFINE) refine_fp64(sc.tris, tri, r.o, r.d, t, u, v);
          h = make_int4(tri, __float_as_int(t), __float_as_int(u), __float_as_int(v));
        } else {
          h = make_int4(-1, 0, 0, 0);
        }
        hits[ray_id] = h;
        ray_id = -1;
      }
    }
  }
}

// Whole-warp batches: a warp claims 32 consecutive rays (consecutive in
// Morton order when the batch was reordered). If they share an origin and
// point the same way (a camera tile), the warp traverses them as one packet
// (traverse_packet: every lane busy, ~1.5x the nodes of a single ray);
// otherwise each lane runs its own ray to completion in a tight loop.
template <int STACK, bool REFINE, bool SMEM>
__global__ void __launch_bounds__(kTraceBlock, SMEM ? 8 : 16) k_trace_batch(DevScene sc, const float4 *__restrict__ rays,
                                                             uint32_t n, int4 *__restrict__ hits,
                                                             uint32_t *__restrict__ counter, uint32_t *err,
                                                             const uint32_t *__restrict__ perm, int packet) {
  __shared__ int s_stack[kTraceBlock / 32][STACK];
  // Per-lane traversal stacks in shared memory, one column per thread.
  __shared__ int s_lane[SMEM ? STACK * kTraceBlock : 1];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(counter, 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n) return;
    uint32_t i = base + lane;
    const bool active = i < n;
    f3 o = mk3(0.0f, 0.0f, 0.0f), d = mk3(1.0f, 0.0f, 0.0f);
    float tmin = 0.0f, tmax = 0.0f;
    if (active) {
      if (perm) i = __ldg(perm + i);
      float4 r0 = __ldg(rays + 2ull * i), r1 = __ldg(rays + 2ull * i + 1);
      o = mk3(r0.x, r0.y, r0.z);
      d = mk3(r1.x, r1.y, r1.z);
      tmin = r0.w;
      tmax = r1.w;
    }
    TraceRay r = make_ray(o, d, tmin);
    float closest = tmax, u = 0.0f, v = 0.0f;
    int k;
    if (packet && warp_is_coherent(active, r))
      k = traverse_packet<STACK>(sc, r, active, closest, u, v, s_stack[warp], err);
    else if (SMEM)
      k = active ? traverse_closest_on<STACK>(sc, r, closest, u, v, err, s_lane + threadIdx.x, kTraceBlock) : -1;
    else
      k = active ? traverse_closest<STACK>(sc, r, closest, u, v, err) : -1;
    if (active) {
      int4 h;
      if (k >= 0) {
        int tri = __ldg(sc.leaf_tri + k);
        if (REFINE) refine_fp64(sc.tris, tri, o, d, closest, u, v);
        h = make_int4(tri, __float_as_int(closest), __float_as_int(u), __float_as_int(v));
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

template <int STACK, bool REFINE>
cudaError_t launch_variant(const DevScene &sc, const rt_ray *rays, uint32_t n, rt_hit *hits, uint32_t *counter,
                           uint32_t *err, const TraceOpts &opts, const uint32_t *perm, cudaStream_t st) {
  const bool batch = opts.refill >= 32;
  int blocks_per_sm = 0;
  if (batch && opts.smem)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_trace_batch<STACK, REFINE, true>, kTraceBlock, 0);
  else if (batch)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_trace_batch<STACK, REFINE, false>, kTraceBlock, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_trace<STACK, REFINE>, kTraceBlock, 0);
  if (blocks_per_sm < 1) blocks_per_sm = 1;
  uint32_t want = (n + kTraceBlock - 1) / kTraceBlock;
  uint32_t grid = (uint32_t)(g_num_sms * blocks_per_sm);
  if (grid > want) grid = want;
  if (batch && opts.smem)
    k_trace_batch<STACK, REFINE, true><<<grid, kTraceBlock, 0, st>>>(sc, reinterpret_cast<const float4 *>(rays), n,
                                                                     reinterpret_cast<int4 *>(hits), counter, err,
                                                                     perm, opts.packet);
  else if (batch)
    k_trace_batch<STACK, REFINE, false><<<grid, kTraceBlock, 0, st>>>(sc, reinterpret_cast<const float4 *>(rays), n,
                                                                      reinterpret_cast<int4 *>(hits), counter, err,
                                                                      perm, opts.packet);
  else
    k_trace<STACK, REFINE><<<grid, kTraceBlock, 0, st>>>(sc, reinterpret_cast<const float4 *>(rays), n,
                                                         reinterpret_cast<int4 *>(hits), counter, err, opts.refill,
                                                         perm);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_trace(const DevScene &sc, const rt_ray *rays, uint32_t n, rt_hit *hits, uint32_t *counter,
                         uint32_t *err, bool refine, const TraceOpts &opts, cudaStream_t st, const uint32_t *perm) {
  if (n == 0) return cudaSuccess;
  if (g_num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
  }
  // The work counter is private to this launch; reset it in stream order.
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  if (sc.depth <= 32)
    return refine ? launch_variant<32, true>(sc, rays, n, hits, counter, err, opts, perm, st)
                  : launch_variant<32, false>(sc, rays, n, hits, counter, err, opts, perm, st);
  return refine ? launch_variant<64, true>(sc, rays, n, hits, counter, err, opts, perm, st)
                : launch_variant<64, false>(sc, rays, n, hits, counter, err, opts, perm, st);
}

cudaError_t launch_trace_literal16(const DevScene &sc, const rt_ray *rays, uint32_t n, rt_hit *hits,
                                   cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_trace_literal16<<<(n + kTraceBlock - 1) / kTraceBlock, kTraceBlock, 0, st>>>(
      sc, reinterpret_cast<const float4 *>(rays), n, reinterpret_cast<int4 *>(hits));
  return cudaGetLastError();
}

}  // namespace rtgb
