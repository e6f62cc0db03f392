// Closest-hit ray casting. Persistent launches sized to the SM count fetch
// work from a global counter. The default whole-warp cast runs two kernels
// per batch: k_trace_packets takes 32 consecutive rays (Morton order) per
// warp and traverses coherent ones as a packet, listing the rest, and
// k_trace_wide casts the listed chunks one ray per lane over the 8-wide
// tree with a shared leaf pool (k_trace_lanes: the same over the binary
// layout with postponed leaves). With trace.beam, k_trace_beams takes the
// first kernel's place for sorted batches: one-origin batches are cast per
// Morton cell as beams (beam.cuh), others in 32-ray chunks as above.
// k_trace is the per-lane refill form (a warp claims new rays as lanes
// finish), k_trace_literal16 the shader's literal traversal.
//
// The hit is chosen with the reference's fp32 arithmetic (traverse.cuh).
// Unless RT_HIT_FP32 is set, t, u, v of the chosen triangle are then
// recomputed once in fp64 with the same triIntersect formula
// (ray-trace-compute.comp:157-173) and rounded to fp32, which removes the
// cancellation error the fp32 formula shows at grazing angles.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>

#include "rt_internal.h"
#include "shade.cuh"
#include "beam.cuh"
#include "traverse.cuh"
#include "wide.cuh"

namespace rtgb {
namespace {

constexpr int kTraceBlock = 128;

// Register budget of a persistent caster compiled for MINB resident blocks
// of 128 threads per SM (the register file holds 65,536 words; allocation
// is in steps of 8 per thread). The casters take their block size at launch
// (64, 128 or 256 threads, "trace.block") with per-warp shared memory
// sized dynamically, so the budget is set per thread with __maxnreg__.
template <int MINB>
__host__ __device__ constexpr int regs_for() {
  return (65536 / (128 * MINB)) / 8 * 8;
}


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
template <int STACK>
__global__ void __launch_bounds__(kTraceBlock) k_trace(DevScene sc, const float4 *__restrict__ rays, uint32_t n,
                                                       int4 *__restrict__ hits, uint32_t *__restrict__ counter,
                                                       uint32_t *err, int refill, const uint32_t *__restrict__ perm,
                                                       bool refine) {
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
        float4 a, b, c, d;
        load_node(N, a, b, c, d);
        const bool h0 = slab_hit_child(r, a, b, closest);
        const bool h1 = slab_hit_child(r, c, d, closest);
        int r0 = __float_as_int(b.z), r1 = __float_as_int(d.z);
        if (h0 && h1) {
          const bool f1 = child1_first(b, ray_octant(r));
          const int nearc = f1 ? r1 : r0, farc = f1 ? r0 : r1;
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
          const int tri = __ldg(sc.leaf_tri + best);
          float t = closest, u = bu, v = bv;
          if (refine) refine_fp64(sc.tris, tri, r.o, r.d, t, u, v);
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
// (traverse_packet: every lane busy, ~1.5x the nodes of a single ray).
// Other chunks are listed for k_trace_lanes, which runs each lane's ray with
// postponed leaves, or (no list) each lane runs its own ray in place.
__device__ __forceinline__ void load_ray(const float4 *__restrict__ rays, uint32_t i, f3 &o, f3 &d, float &tmin,
                                         float &tmax) {
  float4 r0 = __ldg(rays + 2ull * i), r1 = __ldg(rays + 2ull * i + 1);
  o = mk3(r0.x, r0.y, r0.z);
  d = mk3(r1.x, r1.y, r1.z);
  tmin = r0.w;
  tmax = r1.w;
}

__device__ __forceinline__ void store_hit(const DevScene &sc, int4 *__restrict__ hits, uint32_t i, int k, f3 o, f3 d,
                                          float closest, float u, float v, bool refine) {
  int4 h = make_int4(-1, 0, 0, 0);
  if (k >= 0) {
    const int tri = __ldg(sc.leaf_tri + k);
    if (refine) refine_fp64(sc.tris, tri, o, d, closest, u, v);
    h = make_int4(tri, __float_as_int(closest), __float_as_int(u), __float_as_int(v));
  }
  hits[i] = h;
}

// One whole-warp chunk: 32 consecutive rays from `base` (in the cast
// order). If they are coherent (warp_is_coherent) the warp traces them as
// one packet, otherwise it lists the chunk for k_trace_lanes (or, without a
// list, traces it per lane in place). Warp-converged call.
template <int STACK>
__device__ __forceinline__ void cast_chunk(const DevScene &sc, const float4 *__restrict__ rays, uint32_t n,
                                           int4 *__restrict__ hits, uint32_t *err, const uint32_t *__restrict__ perm,
                                           uint32_t *__restrict__ list, uint32_t *__restrict__ list_count,
                                           bool refine, uint32_t base, uint32_t lane, int *s_stack) {
  uint32_t i = base + lane;
  const bool active = i < n;
  f3 o = mk3(0.0f, 0.0f, 0.0f), d = mk3(1.0f, 0.0f, 0.0f);
  float tmin = 0.0f, tmax = 0.0f;
  if (active) {
    if (perm) i = __ldg(perm + i);
    load_ray(rays, i, o, d, tmin, tmax);
  }
  TraceRay r = make_ray(o, d, tmin);
  float closest = tmax, u = 0.0f, v = 0.0f;
  int k;
  if (warp_is_coherent(active, r)) {
    const int oct = warp_octant(active, r);
#define RTGB_CALL(O) k = traverse_packet<STACK, O>(sc, r, active, closest, u, v, s_stack, err)
    RTGB_OCT_DISPATCH(oct, RTGB_CALL)
#undef RTGB_CALL
  } else if (list) {
    if (lane == 0) list[atomicAdd(list_count, 1u)] = base;
    return;
  } else {
    k = active ? traverse_closest<STACK>(sc, r, closest, u, v, err) : -1;
  }
  if (active) store_hit(sc, hits, i, k, o, d, closest, u, v, refine);
}

// First kernel of a whole-warp cast: each warp takes 32 consecutive rays (in
// the cast order) at a time (cast_chunk). The postponed-leaf traversal
// lives in the other kernel: compiled into this one it cost the packet path
// 8% (measured), while the in-place per-lane path costs nothing.
template <int STACK, int MINB>
__global__ void __maxnreg__(regs_for<MINB>()) k_trace_packets(DevScene sc, const float4 *__restrict__ rays,
                                                                   uint32_t n, int4 *__restrict__ hits,
                                                                   uint32_t *__restrict__ counter, uint32_t *err,
                                                                   const uint32_t *__restrict__ perm,
                                                                   uint32_t *__restrict__ list,
                                                                   uint32_t *__restrict__ list_count, bool refine) {
  extern __shared__ int s_dyn_stack[];  // STACK entries per warp
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int *const s_stack = s_dyn_stack + warp * STACK;
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(counter, 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n) return;
    cast_chunk<STACK>(sc, rays, n, hits, err, perm, list, list_count, refine, base, lane, s_stack);
  }
}

// Per-lane cast of whole-warp chunks: the chunks k_trace_packets listed
// (list != nullptr) or every chunk of the batch. `spec` selects the
// postponed-leaf traversal (traverse_spec); results are identical.
template <int STACK, int MINB>
__global__ void __maxnreg__(regs_for<MINB>()) k_trace_lanes(DevScene sc, const float4 *__restrict__ rays,
                                                                   uint32_t n, int4 *__restrict__ hits,
                                                                   uint32_t *__restrict__ counter, uint32_t *err,
                                                                   const uint32_t *__restrict__ perm,
                                                                   const uint32_t *__restrict__ list,
                                                                   const uint32_t *__restrict__ list_count, int spec,
                                                                   bool refine) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t chunks = list ? min(*list_count, (n + 31) / 32) : (n + 31) / 32;
  for (;;) {
    uint32_t c = 0;
    if (lane == 0) c = atomicAdd(counter, 1u);
    c = __shfl_sync(0xffffffffu, c, 0);
    if (c >= chunks) return;
    const uint32_t base = list ? __ldg(list + c) : c * 32u;
    uint32_t i = base + lane;
    const bool active = i < n;
    f3 o = mk3(0.0f, 0.0f, 0.0f), d = mk3(1.0f, 0.0f, 0.0f);
    float tmin = 0.0f, tmax = 0.0f;
    if (active) {
      if (perm) i = __ldg(perm + i);
      load_ray(rays, i, o, d, tmin, tmax);
    }
    TraceRay r = make_ray(o, d, tmin);
    float closest = tmax, u = 0.0f, v = 0.0f;
    int k;
    if (spec) {
      const int oct = warp_octant(active, r);
#define RTGB_CALL(O) k = traverse_spec<STACK, O>(sc, r, active, closest, u, v, err)
      RTGB_OCT_DISPATCH(oct, RTGB_CALL)
#undef RTGB_CALL
    } else {
      k = active ? traverse_closest<STACK>(sc, r, closest, u, v, err) : -1;
    }
    if (active) store_hit(sc, hits, i, k, o, d, closest, u, v, refine);
  }
}

// Beam cast (beam.cuh). With the ray sort's cell tiles and a batch of one
// origin (the sort's sampled origin extent is zero), each block casts one
// cell tile at a time, up to 256 rays. A tile whose rays share the origin
// and whose directions fit a narrow cone around one axis walks the tree
// once as a beam, in rounds: expansion steps by the whole block until the
// round holds `round_leaves` leaves, then every warp tests them. Any other tile, or one
// whose beam was abandoned, is cast warp by warp in place (packet, or per
// lane). Other batches are cast in 32-ray chunks, as k_trace_packets casts
// them.
template <int STACK, int MINB>
__global__ void __launch_bounds__(kBeamRays, MINB)
    k_trace_beams(DevScene sc, const float4 *__restrict__ rays, uint32_t n, int4 *__restrict__ hits,
                  uint32_t *__restrict__ counter, uint32_t *err, const uint32_t *__restrict__ perm,
                  uint32_t *__restrict__ list, uint32_t *__restrict__ list_count,
                  const uint32_t *__restrict__ cell_tiles, const uint32_t *__restrict__ cell_count,
                  const uint32_t *__restrict__ ext, int round_leaves, bool refine) {
  __shared__ BeamShared s;
  extern __shared__ int s_dyn_stack[];  // STACK entries per warp (packet casts)
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int *const s_stack = s_dyn_stack + warp * STACK;
  const float INF = __int_as_float(0x7f800000);
  const bool one_origin = __ldg(ext + 0) == __ldg(ext + 5) && __ldg(ext + 1) == __ldg(ext + 6) &&
                          __ldg(ext + 2) == __ldg(ext + 7);
  if (!one_origin) {
    for (;;) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(counter, 32u);
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base >= n) return;
      cast_chunk<STACK>(sc, rays, n, hits, err, perm, list, list_count, refine, base, lane, s_stack);
    }
  }
  const uint32_t ntiles = __ldg(cell_count);
  for (;;) {
    __syncthreads();  // every thread is done with the previous tile's state
    if (tid == 0) s.tile = atomicAdd(counter, 1u);
    __syncthreads();
    const uint32_t t = s.tile;
    if (t >= ntiles) return;
    const uint32_t beg = __ldg(cell_tiles + 2 * t), end = __ldg(cell_tiles + 2 * t + 1);
    uint32_t i = beg + tid;
    const bool active = i < end && i < n;
    f3 o = mk3(0.0f, 0.0f, 0.0f), d = mk3(1.0f, 0.0f, 0.0f);
    float tmin = 0.0f, tmax = 0.0f;
    if (active) {
      i = __ldg(perm + i);
      load_ray(rays, i, o, d, tmin, tmax);
    }
    const TraceRay r = make_ray(o, d, tmin);
    // The tile's origin, dominant axis and near-first octant from its
    // first ray (thread 0's: every tile holds at least one ray).
    if (tid == 0) {
      s.o[0] = o.x, s.o[1] = o.y, s.o[2] = o.z;
      const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
      const int za = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
      s.za = za;
      s.sz = (za == 0 ? d.x : (za == 1 ? d.y : d.z)) >= 0.0f ? 1.0f : -1.0f;
      s.oct = ray_octant(r);
      s.u_lo = s.v_lo = 0xffffffffu;
      s.u_hi = s.v_hi = 0u;
      s.md[0] = s.md[1] = 0u;
    }
    __syncthreads();
    // Every ray: the same origin, in front along the tile's axis within
    // 2:1 of it, and (u, v) = (d_u, d_v) / d_z folded into the tile's and
    // the warp's bounds.
    bool ok = true;
    uint32_t ulo = 0xffffffffu, uhi = 0u, vlo = 0xffffffffu, vhi = 0u;
    const int za = s.za;
    const float sz = s.sz;
    if (active) {
      const float dz = sz * (za == 0 ? d.x : (za == 1 ? d.y : d.z));
      const float du = za == 0 ? d.y : (za == 1 ? d.z : d.x);
      const float dv = za == 0 ? d.z : (za == 1 ? d.x : d.y);
      ok = o.x == s.o[0] && o.y == s.o[1] && o.z == s.o[2] && dz > 0.0f && fabsf(du) <= 2.0f * dz &&
           fabsf(dv) <= 2.0f * dz;
      if (ok) {
        ulo = uhi = beam_ord(__fdiv_rn(du, dz));
        vlo = vhi = beam_ord(__fdiv_rn(dv, dz));
      }
    }
    ulo = __reduce_min_sync(0xffffffffu, ulo);
    uhi = __reduce_max_sync(0xffffffffu, uhi);
    vlo = __reduce_min_sync(0xffffffffu, vlo);
    vhi = __reduce_max_sync(0xffffffffu, vhi);
    if (lane == 0) {
      atomicMin(&s.u_lo, ulo);
      atomicMax(&s.u_hi, uhi);
      atomicMin(&s.v_lo, vlo);
      atomicMax(&s.v_hi, vhi);
    }
    ok = __syncthreads_and(ok);
    if (tid == 0) {
      // Bounds widened by 1e-5 (the quotients carry one rounding).
      const float umin = beam_unord(s.u_lo) - 1e-5f, umax = beam_unord(s.u_hi) + 1e-5f;
      const float vmin = beam_unord(s.v_lo) - 1e-5f, vmax = beam_unord(s.v_hi) + 1e-5f;
      s.lim[0] = umin, s.lim[1] = umax, s.lim[2] = vmin, s.lim[3] = vmax;
      // A one-triangle tree (the root a leaf) goes to the packets.
      s.ok = ok && sc.root_ref >= 0 && umax - umin <= kBeamMaxSpan && vmax - vmin <= kBeamMaxSpan;
      s.stack[0] = sc.root_ref;
    }
    __syncthreads();
    float closest = tmax, bu = 0.0f, bv = 0.0f;
    int best = -1;
    bool beam = s.ok != 0;
    if (beam) {
      Cone tcone;
      tcone.o[0] = s.o[0], tcone.o[1] = s.o[1], tcone.o[2] = s.o[2];
      tcone.umin = s.lim[0], tcone.umax = s.lim[1], tcone.vmin = s.lim[2], tcone.vmax = s.lim[3];
      tcone.sz = sz;
      tcone.za = za;
      // The warp's own cone (empty, inverted bounds, for a warp without rays).
      Cone wcone = tcone;
      wcone.umin = beam_unord(ulo) - 1e-5f, wcone.umax = beam_unord(uhi) + 1e-5f;
      wcone.vmin = beam_unord(vlo) - 1e-5f, wcone.vmax = beam_unord(vhi) + 1e-5f;
      const int woct = warp_octant(active, r);
      const float dn = active ? __fsqrt_rn(dot3(d, d)) : 0.0f;
      // Frontier size, round size, depth bound: the same in every thread.
      int sp = 1, nl = 0, round = 0;
      float maxd = INF;
      uint32_t steps = 0;
      for (;;) {
        if (sp > 0 && nl < round_leaves) {
          if (++steps > sc.ntris + 16u) {
            if (tid == 0) atomicOr(err, KERR_TIMEOUT);
            beam = false;
            break;
          }
          const float md2 = maxd * maxd;
          const bool stepped = za == 0   ? beam_step<0>(s, tcone, sc, lane, warp, sp, nl, md2, err)
                               : za == 1 ? beam_step<1>(s, tcone, sc, lane, warp, sp, nl, md2, err)
                                         : beam_step<2>(s, tcone, sc, lane, warp, sp, nl, md2, err);
          if (!stepped) {
            beam = false;
            break;
          }
          continue;
        }
        if (nl == 0) break;  // frontier and round empty
        // Farthest closest hit of the warp's rays, as a distance (unknown
        // values count as infinite). The 1% margin exceeds the fp32
        // triangle t's own error except at grazing angles below ~1e-5 rad,
        // where a hit's t may undershoot its distance.
        uint32_t wm = 0u;
        if (active) {
          const float x = closest * dn * 1.01f;
          wm = x >= 0.0f ? __float_as_uint(x) : (x < 0.0f ? 0u : 0x7f800000u);
        }
        const float wmd = __uint_as_float(__reduce_max_sync(0xffffffffu, wm));
#define RTGB_CALL(O) beam_test_round<O>(s, nl, wcone, wmd * wmd, lane, sc, r, active, closest, best, bu, bv)
        RTGB_OCT_DISPATCH(woct, RTGB_CALL)
#undef RTGB_CALL
        wm = 0u;
        if (active) {
          const float x = closest * dn * 1.01f;
          wm = x >= 0.0f ? __float_as_uint(x) : (x < 0.0f ? 0u : 0x7f800000u);
        }
        wm = __reduce_max_sync(0xffffffffu, wm);
        // This round's slot collects the maxima; the other one, read after
        // the previous round, is cleared for the next.
        if (tid == 0) s.md[(round + 1) & 1] = 0u;
        if (lane == 0) atomicMax(&s.md[round & 1], wm);
        __syncthreads();
        maxd = __uint_as_float(s.md[round & 1]);
        round++;
        nl = 0;
      }
    }
    if (beam) {
      if (active) store_hit(sc, hits, i, best, o, d, closest, bu, bv, refine);
      continue;
    }
    // Warp by warp, in place, from the start.
    closest = tmax;
    bu = bv = 0.0f;
    int k;
    if (warp_is_coherent(active, r)) {
      const int oct = warp_octant(active, r);
#define RTGB_CALL(O) k = traverse_packet<STACK, O>(sc, r, active, closest, bu, bv, s_stack, err)
      RTGB_OCT_DISPATCH(oct, RTGB_CALL)
#undef RTGB_CALL
    } else {
      k = active ? traverse_closest<STACK>(sc, r, closest, bu, bv, err) : -1;
    }
    if (active) store_hit(sc, hits, i, k, o, d, closest, bu, bv, refine);
  }
}

// Ordered keys for (t, triangle) pairs: ord_f maps fp32 to uint32 so that
// unsigned order equals float order (-0 is first mapped to +0 by the
// callers, which compare it equal to +0 as floats do).
__device__ __forceinline__ uint32_t ord_f(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord_inv(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// triIntersect of test_triangle on one precomputed record, without the
// acceptance rule: true when tmin < t <= closest and the hit lies inside.
__device__ __forceinline__ bool tri_candidate(const float4 *__restrict__ tpre, int k, f3 o, f3 d, float tmin,
                                              float closest, float &t, float &u, float &v) {
  const float4 *T = tpre + 3ll * k;
  const float4 t0 = __ldg(T), t1 = __ldg(T + 1), t2 = __ldg(T + 2);
  const f3 v0 = mk3(t0.x, t0.y, t0.z), n = mk3(t0.w, t1.x, t1.y);
  const f3 a = mk3(t1.z, t1.w, t2.x), b = mk3(t2.y, t2.z, t2.w);
  const f3 p = sub3(v0, o);
  const float idet = __frcp_rn(dot3(d, n));  // correctly rounded 1/x: the value of the IEEE division 1.0f / x
  t = __fmul_rn(dot3(n, p), idet);
  if (!(t > tmin && t <= closest)) return false;
  const f3 q = cross3(p, d);
  u = __fmul_rn(dot3(q, b), idet);
  v = __fmul_rn(dot3(q, a), idet);
  return !(u < 0.0f || u > 1.0f || v < 0.0f || __fadd_rn(u, v) > 1.0f);
}

// Leaf pool entries per warp (power of two): at most 31 are left after the
// leaf rounds of an iteration, and each of its VISITS node steps adds at
// most 8 per lane (31 + 3 * 256 < 1024).
template <int VISITS>
__host__ __device__ constexpr int pool_entries() {
  return VISITS == 1 ? 512 : 1024;
}
constexpr int kFinish = 64;  // finished-ray ring per warp (power of two, >= 64)
template <int VISITS>
__host__ __device__ constexpr int wide_warp_smem() {
  return 64 * 16 + 32 * 8 + 32 * 16 + pool_entries<VISITS>() * 4 + kFinish * 4 + 16;
}

// One ray per lane over bvh8 (Ylitie et al., HPG 2017, with explicit child
// refs). A step tests the lane's 96-byte quantized node (wide.cuh:
// wide_node_test: three 256-bit loads, eight slot tests with packed FMAs;
// empty slots hold an inverted box and a harmless leaf ref, so no per-slot
// mask test is needed). The node's slots were assigned by octant
// (bvh8.cu), so the entered inner children, kept as the bits s ^ o of a rank
// mask (o: the sign bits of the ray's direction), come out roughly
// near-first by taking the lowest set bit — no distance sort. The child
// with the smallest entry distance is visited next; the node and its other
// rank bits form a group on the lane's stack (one entry per level at most),
// and the next child of a group is fetched by re-reading one ref word of its
// node. On the bench mesh this order visits 8% more nodes than a full sort,
// at a fraction of its instructions.
// Leaves that are hit go to the warp's FIFO leaf pool in shared memory as
// (leaf, lane) entries, each lane reserving its run with one shared atomic;
// whenever 32 are pooled, or a lane has run out of
// nodes with entries still pooled, the 32 lanes test one pooled triangle
// each against the owning lane's ray (kept in shared memory), so triangle
// tests run with every lane busy whatever the rays' phases. Each ray's
// closest hit is one 64-bit key (ordered t, triangle index) lowered with a
// shared-memory atomicMin: a candidate wins when t is smaller, or equal with
// a lower triangle index — the acceptance rule of test_triangle,
// independent of the order in which leaves are tested. The winner of a
// round stores its t, u, v. A ray is done when it has no node, no group
// left, and the pool has moved past its last entry. Idle lanes claim new
// rays (slots of the listed chunks, or of the whole batch) once `refill` of
// them are idle. The pruning of every slot is bit for bit the generic
// min/max slab test's (for lo <= hi the FMA is monotonic in the byte), so
// only the visiting order differs from a sorted traversal.
// LEAF_OUT: hits are int2 (leaf k, fp32 t) for the wavefront's shading (k =
// -1 and the ray's tmax when nothing is hit), and the batch size is the
// device word *d_n (capped at n); otherwise int4 rt_hit records.
template <int GSTACK, int MINB, bool LEAF_OUT, int VISITS>
__global__ void __maxnreg__(regs_for<MINB>()) k_trace_wide(DevScene sc, const float4 *__restrict__ rays,
                                                               uint32_t n, const uint32_t *d_n,
                                                               void *__restrict__ hits_out,
                                                               uint32_t *__restrict__ counter, uint32_t *err,
                                                               const uint32_t *__restrict__ perm,
                                                               const uint32_t *__restrict__ list,
                                                               const uint32_t *__restrict__ list_count,
                                                               int refill, bool refine) {
  // Per warp (wide_warp_smem bytes, dynamic): the lanes' rays (32 x 2
  // float4), closest-hit keys (32 x u64), winning t/u/v/leaf (32 x float4),
  // the leaf pool (kPool x u32), the ring of finished rays waiting for
  // their fp64 re-evaluation (kFinish x u32) and the pool's tail (16 bytes).
  extern __shared__ float4 s_wide[];
  uint32_t lane;
  asm("mov.u32 %0, %%laneid;" : "=r"(lane));
  const uint32_t warp = threadIdx.x >> 5;
  const uint32_t lt_mask = (1u << lane) - 1u;
  constexpr int kPool = pool_entries<VISITS>();
  float4 *const wbase = s_wide + warp * (wide_warp_smem<VISITS>() / 16);
  float4(*ray_s)[2] = reinterpret_cast<float4(*)[2]>(wbase);
  volatile unsigned long long *key_v = reinterpret_cast<unsigned long long *>(wbase + 64);
  unsigned long long *key_a = reinterpret_cast<unsigned long long *>(wbase + 64);
  float4 *hit_s = wbase + 80;
  uint32_t *pool = reinterpret_cast<uint32_t *>(wbase + 112);
  uint32_t *finish = pool + kPool;
  // The pool's tail: lanes reserve their entries with one shared atomic.
  volatile uint32_t *pool_tail = finish + kFinish;
  if (lane == 0) *pool_tail = 0u;
  __syncwarp();
  uint32_t fhead = 0, ftail = 0;
  // fp64 re-evaluation of 32 queued finished rays (or the `cnt` left at the
  // end), one per lane: converged, so the few fp64 operations of each ray
  // overlap the other warps' work instead of occupying the pipe for one lane.
  auto refine_round = [&](uint32_t cnt) {
    if (lane < cnt) {
      const uint32_t i = finish[(fhead + lane) & (kFinish - 1)];
      int4 h = static_cast<int4 *>(hits_out)[i];
      const float4 r0 = __ldg(rays + 2ull * i), r1 = __ldg(rays + 2ull * i + 1);
      float t, u, v;
      refine_fp64(sc.tris, h.x, mk3(r0.x, r0.y, r0.z), mk3(r1.x, r1.y, r1.z), t, u, v);
      static_cast<int4 *>(hits_out)[i] = make_int4(h.x, __float_as_int(t), __float_as_int(u), __float_as_int(v));
    }
    fhead += cnt;
  };
  const float INF = __int_as_float(0x7f800000);
  if (d_n) n = min(n, *d_n);
  const uint32_t total = list ? min(*list_count, (n + 31) / 32) * 32u : n;
  const float4 *__restrict__ bvh8 = sc.bvh8;
  const int32_t *__restrict__ words8 = reinterpret_cast<const int32_t *>(sc.bvh8);
  const uint32_t n8 = sc.n8;
  const uint32_t step_cap = sc.n8 + 16u;

  uint32_t gstack[GSTACK];
  TraceRay r = make_ray(mk3(0.0f, 0.0f, 0.0f), mk3(1.0f, 0.0f, 0.0f), 0.0f);
  int node = -1, gsp = 0, ray_i = -1, finish_i = 0;
  uint32_t gnode = 0, gmask = 0, oct = 0;
  uint32_t steps = 0, mlp1 = 0, head = 0, tail = 0;
  bool exhausted = false;
  for (;;) {
    // A ray with no node, no group left and its last pooled leaf tested.
    bool queued = false;
    if (ray_i >= 0 && node < 0 && gmask == 0 && gsp == 0 && (int)(head - mlp1) >= 0) {
      const unsigned long long key = key_v[lane];
      const float tmax = ray_s[lane][1].w;
      const bool got = (uint32_t)(key >> 32) != ord_f(__fadd_rn(tmax, 0.0f));
      const float4 w = hit_s[lane];
      if (LEAF_OUT) {
        static_cast<int2 *>(hits_out)[ray_i] =
            got ? make_int2(__float_as_int(w.w), __float_as_int(w.x)) : make_int2(-1, __float_as_int(tmax));
      } else {
        int4 h = make_int4(-1, 0, 0, 0);
        if (got) h = make_int4((int)(uint32_t)key, __float_as_int(w.x), __float_as_int(w.y), __float_as_int(w.z));
        static_cast<int4 *>(hits_out)[ray_i] = h;
        queued = got && refine;
      }
      if (queued) finish_i = ray_i;
      ray_i = -1;
    }
    if (!LEAF_OUT && refine) {
      const uint32_t qm = __ballot_sync(0xffffffffu, queued);
      if (qm) {
        if (queued) finish[(ftail + __popc(qm & lt_mask)) & (kFinish - 1)] = (uint32_t)finish_i;
        ftail += __popc(qm);
        if (ftail - fhead >= 32u) {
          __syncwarp();
          refine_round(32u);
        }
      }
    }
    // Idle lanes claim new rays.
    const uint32_t idle = __ballot_sync(0xffffffffu, ray_i < 0);
    if (!exhausted && __popc(idle) >= refill) {
      const uint32_t cnt = __popc(idle), leader = __ffs(idle) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(counter, cnt);
      base = __shfl_sync(0xffffffffu, base, leader);
      if (base + cnt >= total) exhausted = true;
      if (ray_i < 0) {
        const uint32_t slot = base + __popc(idle & lt_mask);
        if (slot < total) {
          const uint32_t ray = list ? __ldg(list + (slot >> 5)) + (slot & 31u) : slot;
          if (ray < n) {
            const uint32_t i = perm ? __ldg(perm + ray) : ray;
            const float4 r0 = __ldg(rays + 2ull * i), r1 = __ldg(rays + 2ull * i + 1);
            ray_s[lane][0] = r0;
            ray_s[lane][1] = r1;
            key_v[lane] = (unsigned long long)ord_f(__fadd_rn(r1.w, 0.0f)) << 32;
            r = make_ray(mk3(r0.x, r0.y, r0.z), mk3(r1.x, r1.y, r1.z), r0.w);
            oct = (uint32_t)ray_octant(r);
            ray_i = (int)i;
            gsp = 0;
            gmask = 0;
            steps = 0;
            mlp1 = head;
            const float root = slab_enter(r, sc.root_lo[0], sc.root_hi[0], sc.root_lo[1], sc.root_hi[1],
                                          sc.root_lo[2], sc.root_hi[2], r1.w);
            node = root < INF ? sc.root8 : -1;
          }
        }
      }
    }
    if (exhausted && __all_sync(0xffffffffu, ray_i < 0)) {
      if (!LEAF_OUT && refine && ftail != fhead) {
        __syncwarp();
        refine_round(ftail - fhead);
      }
      return;
    }
    __syncwarp();

#pragma unroll 1
    for (int visit = 0; visit < VISITS; visit++) {
      if (visit > 0 && !__any_sync(0xffffffffu, ray_i >= 0 && node >= 0)) break;
      // One node per lane that holds one.
      uint32_t leafmask = 0;
      int32_t ref[8];
      if (ray_i >= 0 && node >= 0) {
        if ((uint32_t)node >= n8 || ++steps > step_cap) {
          atomicOr(err, (uint32_t)node >= n8 ? KERR_BAD_INDEX : KERR_TIMEOUT);
          node = -1;
          gmask = 0;
          gsp = 0;
        } else {
          const float closest = ord_inv((uint32_t)(key_v[lane] >> 32));
          const int node_idx = node;
          WideStep ws;
          wide_node_test(bvh8, node, r, oct, closest, ws);
  #pragma unroll
          for (int k = 0; k < 8; k++) ref[k] = ws.ref[k];
          leafmask = ws.leafmask;
          const uint32_t hin = ws.hin, nearest = ws.nearest;
          uint32_t ibits = rank_bits(hin, oct);
          node = -1;
          if (ibits) {
            if (gmask) {
              if (gsp >= GSTACK) {
                atomicOr(err, KERR_STACK_OVERFLOW);
                gsp = 0;
                gmask = 0;
                ibits = 0;
              } else {
                gstack[gsp++] = (gnode << 8) | gmask;
              }
            }
          }
          if (ibits) {
            // The nearest entered child next; the others later, in rank order.
            gnode = (uint32_t)node_idx;
            gmask = ibits & ~(1u << (nearest ^ oct));
            node = pick8(ref, nearest);
          }
        }
      }
      // The next entered child of the innermost group, when the lane has no node.
      if (ray_i >= 0 && node < 0 && (gmask != 0 || gsp > 0)) {
        if (gmask == 0) {
          const uint32_t e = gstack[--gsp];
          gnode = e >> 8;
          gmask = e & 0xffu;
        }
        const uint32_t rk = (uint32_t)(__ffs(gmask) - 1);
        gmask &= gmask - 1u;
        node = __ldg(words8 + 24ll * gnode + 16 + (rk ^ oct));
      }

      // Pool this step's leaves: each lane reserves its run of entries with
      // one shared-memory atomic (the pool's order does not matter).
      const uint32_t c = __popc(leafmask);
      if (c) {
        uint32_t pos = atomicAdd(const_cast<uint32_t *>(pool_tail), c);
  #pragma unroll
        for (int s = 0; s < 8; s++) {
          if (!((leafmask >> s) & 1u)) continue;
          // Leaf refs were range-checked when the bvh8 was built (k_encode8).
          pool[pos & (kPool - 1)] = ((uint32_t)~ref[s] << 5) | lane;
          pos++;
        }
        mlp1 = pos;
      }
      __syncwarp();
      tail = *pool_tail;
    }

    // Leaf rounds: 32 pooled leaves at a time, oldest first.
    for (;;) {
      const bool waiting = ray_i >= 0 && node < 0 && gmask == 0 && gsp == 0 && (int)(head - mlp1) < 0;
      if (!__any_sync(0xffffffffu, waiting) && tail - head < 32u) break;
      const uint32_t cnt = min(tail - head, 32u);
      bool acc = false;
      unsigned long long cand = 0;
      uint32_t owner = 0;
      int k = 0;
      float ct = 0.0f, cu = 0.0f, cv = 0.0f;
      if (lane < cnt) {
        const uint32_t e = pool[(head + lane) & (kPool - 1)];
        owner = e & 31u;
        k = (int)(e >> 5);
        const float4 q0 = ray_s[owner][0], q1 = ray_s[owner][1];
        const unsigned long long cur = key_v[owner];
        if (tri_candidate(sc.tpre, k, mk3(q0.x, q0.y, q0.z), mk3(q1.x, q1.y, q1.z), q0.w,
                          ord_inv((uint32_t)(cur >> 32)), ct, cu, cv)) {
          const unsigned long long key =
              ((unsigned long long)ord_f(__fadd_rn(ct, 0.0f)) << 32) | (uint32_t)__ldg(sc.leaf_tri + k);
          if (key < cur) {
            acc = true;
            cand = key;
            atomicMin(key_a + owner, key);
          }
        }
      }
      __syncwarp();
      if (acc && key_v[owner] == cand) hit_s[owner] = make_float4(ct, cu, cv, __int_as_float(k));
      __syncwarp();
      head += cnt;
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

template <typename K>
uint32_t persistent_grid(K kernel, uint32_t n, int block = kTraceBlock, size_t smem = 0) {
  int blocks_per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, kernel, block, smem);
  if (blocks_per_sm < 1) blocks_per_sm = 1;
  uint32_t want = (n + block - 1) / block;
  uint32_t grid = (uint32_t)(g_num_sms * blocks_per_sm);
  return grid > want ? want : grid;
}

// Casting block size: 64, 128 or 256 threads.
inline int cast_block(int b) { return b <= 64 ? 64 : (b >= 256 ? 256 : 128); }

template <int STACK, int MINB>
cudaError_t launch_lanes(const DevScene &sc, const float4 *rays, uint32_t n, int4 *hits, uint32_t *counter,
                         uint32_t *err, const uint32_t *perm, const uint32_t *list, const uint32_t *list_count,
                         int spec, int block, bool refine, cudaStream_t st) {
  auto kern = k_trace_lanes<STACK, MINB>;
  kern<<<persistent_grid(kern, n, block), block, 0, st>>>(sc, rays, n, hits, counter, err, perm, list, list_count,
                                                           spec, refine);
  return cudaGetLastError();
}

template <int GSTACK>
cudaError_t launch_wide(const DevScene &sc, const float4 *rays, uint32_t n, int4 *hits, uint32_t *counter,
                        uint32_t *err, const uint32_t *perm, const uint32_t *list, const uint32_t *list_count,
                        int minblocks, int refill, int block, int visits, bool refine, cudaStream_t st) {
  auto kern = visits >= 3 ? (minblocks >= 8   ? k_trace_wide<GSTACK, 8, false, 3>
                            : minblocks >= 7 ? k_trace_wide<GSTACK, 7, false, 3>
                            : minblocks >= 6 ? k_trace_wide<GSTACK, 6, false, 3>
                                             : k_trace_wide<GSTACK, 5, false, 3>)
            : visits >= 2 ? (minblocks >= 8   ? k_trace_wide<GSTACK, 8, false, 2>
                            : minblocks >= 7 ? k_trace_wide<GSTACK, 7, false, 2>
                            : minblocks >= 6 ? k_trace_wide<GSTACK, 6, false, 2>
                                             : k_trace_wide<GSTACK, 5, false, 2>)
                          : (minblocks >= 8   ? k_trace_wide<GSTACK, 8, false, 1>
                            : minblocks >= 7 ? k_trace_wide<GSTACK, 7, false, 1>
                            : minblocks >= 6 ? k_trace_wide<GSTACK, 6, false, 1>
                                             : k_trace_wide<GSTACK, 5, false, 1>);
  const size_t smem = (size_t)(block / 32) * (visits >= 2 ? wide_warp_smem<2>() : wide_warp_smem<1>());
  static_assert(wide_warp_smem<3>() == wide_warp_smem<2>(), "visits 2 and 3 share the pool size");
  if (smem > 48 * 1024) {  // 256-thread blocks with the large pool
    const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  kern<<<persistent_grid(kern, n, block, smem), block, smem, st>>>(sc, rays, n, nullptr, hits, counter, err, perm,
                                                                   list, list_count, refill, refine);
  return cudaGetLastError();
}

// Group stack of the 8-wide caster: one entry per bvh8 level at most.
cudaError_t launch_wide_any(const DevScene &sc, const float4 *rays, uint32_t n, int4 *hits, uint32_t *counter,
                            uint32_t *err, const uint32_t *perm, const uint32_t *list, const uint32_t *list_count,
                            const TraceOpts &opts, bool refine, cudaStream_t st) {
  const int want = std::max<int>(opts.stack, (int)sc.levels8);
  const int block = cast_block(opts.block);
  if (want <= 16)
    return launch_wide<16>(sc, rays, n, hits, counter, err, perm, list, list_count, opts.wide_minblocks,
                                   opts.wide_refill, block, opts.wide_visits, refine, st);
  if (want <= 32)
    return launch_wide<32>(sc, rays, n, hits, counter, err, perm, list, list_count, opts.wide_minblocks,
                                   opts.wide_refill, block, opts.wide_visits, refine, st);
  return launch_wide<64>(sc, rays, n, hits, counter, err, perm, list, list_count, opts.wide_minblocks,
                                 opts.wide_refill, block, opts.wide_visits, refine, st);
}

template <int STACK>
cudaError_t launch_variant(const DevScene &sc, const rt_ray *rays, uint32_t n, rt_hit *hits, uint32_t *counter,
                           uint32_t *err, const TraceOpts &opts, const uint32_t *perm, uint32_t *chunk_scratch,
                           const RayCells *cells, bool refine, cudaStream_t st) {
  const float4 *r4 = reinterpret_cast<const float4 *>(rays);
  int4 *h4 = reinterpret_cast<int4 *>(hits);
  if (opts.refill >= 32) {
    const int block = cast_block(opts.block);
    // chunk_scratch: [0] listed chunks, [1] lane-pass counter, list from word 64.
    const uint32_t *list = nullptr, *list_count = nullptr;
    uint32_t *lane_counter = counter;
    if (opts.packet && chunk_scratch) {
      cudaError_t e = cudaMemsetAsync(chunk_scratch, 0, 256, st);
      if (e != cudaSuccess) return e;
      uint32_t *plist = opts.defer ? chunk_scratch + 64 : nullptr;
      if ((opts.beam == 1 || (opts.beam == 2 && sc.median_tree)) && cells && perm) {
        auto bk = k_trace_beams<STACK, 4>;
        const size_t smem = (size_t)(kBeamRays / 32) * STACK * sizeof(int);
        bk<<<persistent_grid(bk, n, kBeamRays, smem), kBeamRays, smem, st>>>(
            sc, r4, n, h4, counter, err, perm, plist, chunk_scratch, cells->tiles, cells->count, cells->ext,
            opts.beam_round, refine);
      } else {
        auto pk = opts.packet_minblocks >= 16   ? k_trace_packets<STACK, 16>
                  : opts.packet_minblocks >= 12 ? k_trace_packets<STACK, 12>
                                                : k_trace_packets<STACK, 10>;
        const size_t smem = (size_t)(block / 32) * STACK * sizeof(int);
        pk<<<persistent_grid(pk, n, block, smem), block, smem, st>>>(sc, r4, n, h4, counter, err, perm, plist,
                                                                     chunk_scratch, refine);
      }
      if (!opts.defer) return cudaGetLastError();
      list = chunk_scratch + 64;
      list_count = chunk_scratch;
      lane_counter = chunk_scratch + 1;
    }
    if (use_wide(opts, sc))
      return launch_wide_any(sc, r4, n, h4, lane_counter, err, perm, list, list_count, opts, refine, st);
    if (opts.minblocks >= 16)
      return launch_lanes<STACK, 16>(sc, r4, n, h4, lane_counter, err, perm, list, list_count, opts.spec,
                                             block, refine, st);
    if (opts.minblocks >= 12)
      return launch_lanes<STACK, 12>(sc, r4, n, h4, lane_counter, err, perm, list, list_count, opts.spec,
                                             block, refine, st);
    return launch_lanes<STACK, 10>(sc, r4, n, h4, lane_counter, err, perm, list, list_count, opts.spec,
                                           block, refine, st);
  }
  auto kt = k_trace<STACK>;
  kt<<<persistent_grid(kt, n), kTraceBlock, 0, st>>>(sc, r4, n, h4, counter, err, opts.refill, perm, refine);
  return cudaGetLastError();
}

}  // namespace

bool wide_ok(const DevScene &sc) {
  // Group entries pack the node number into 24 bits.
  return sc.bvh8 && sc.levels8 >= 1 && sc.levels8 <= 64 && sc.n8 < (1u << 24) && sc.ntris < (1u << 27);
}

cudaError_t launch_wide_leaf(const DevScene &sc, const rt_ray *rays, uint32_t cap, const uint32_t *d_n,
                             const uint32_t *perm, const uint32_t *list, const uint32_t *list_count, int2 *hits,
                             uint32_t *counter, uint32_t *err, int minblocks, int refill, cudaStream_t st) {
  if (!wide_ok(sc)) return cudaErrorInvalidValue;
  if (g_num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
  }
  const float4 *r4 = reinterpret_cast<const float4 *>(rays);
  // minblocks 8: one node step per iteration (64 registers); otherwise three.
  auto go = [&](auto kern, size_t warp_smem) {
    const size_t smem = (size_t)(kTraceBlock / 32) * warp_smem;
    kern<<<persistent_grid(kern, cap, kTraceBlock, smem), kTraceBlock, smem, st>>>(sc, r4, cap, d_n, hits, counter,
                                                                                   err, perm, list, list_count,
                                                                                   refill, false);
    return cudaGetLastError();
  };
  const bool narrow = minblocks >= 8;
  const size_t s1 = wide_warp_smem<1>(), s3 = wide_warp_smem<3>();
  if (sc.levels8 <= 16)
    return narrow ? go(k_trace_wide<16, 8, true, 1>, s1) : go(k_trace_wide<16, 6, true, 3>, s3);
  if (sc.levels8 <= 32)
    return narrow ? go(k_trace_wide<32, 8, true, 1>, s1) : go(k_trace_wide<32, 6, true, 3>, s3);
  return narrow ? go(k_trace_wide<64, 8, true, 1>, s1) : go(k_trace_wide<64, 6, true, 3>, s3);
}

size_t trace_chunk_scratch_bytes(uint32_t n) { return 4ull * (64 + (n + 31) / 32); }

cudaError_t launch_trace(const DevScene &sc, const rt_ray *rays, uint32_t n, rt_hit *hits, uint32_t *counter,
                         uint32_t *err, bool refine, const TraceOpts &opts, cudaStream_t st, const uint32_t *perm,
                         uint32_t *chunk_scratch, const RayCells *cells) {
  if (n == 0) return cudaSuccess;
  if (g_num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
  }
  // The work counter is private to this launch; reset it in stream order.
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  // Traversal stack: trace.stack entries (16, 32 or 64), raised to the
  // smallest size that holds the tree's depth.
  const int stk = trace_stack_entries(opts, sc);
  return stk <= 16 ? launch_variant<16>(sc, rays, n, hits, counter, err, opts, perm, chunk_scratch, cells, refine, st)
         : stk <= 32
             ? launch_variant<32>(sc, rays, n, hits, counter, err, opts, perm, chunk_scratch, cells, refine, st)
             : launch_variant<64>(sc, rays, n, hits, counter, err, opts, perm, chunk_scratch, cells, refine, st);
}

cudaError_t launch_trace_literal16(const DevScene &sc, const rt_ray *rays, uint32_t n, rt_hit *hits,
                                   cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_trace_literal16<<<(n + kTraceBlock - 1) / kTraceBlock, kTraceBlock, 0, st>>>(
      sc, reinterpret_cast<const float4 *>(rays), n, reinterpret_cast<int4 *>(hits));
  return cudaGetLastError();
}

}  // namespace rtgb
