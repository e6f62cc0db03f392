// The 8-wide quantized node test (bvh8.cu builds the nodes), shared by the
// warp caster (trace.cu: k_trace_wide) and the per-thread traversal of the
// megakernel (traverse_wide_lane).
#pragma once
#include "rt_internal.h"
#include "rt_math.cuh"
#include "traverse.cuh"

namespace rtgb {

// 32 bytes in one 256-bit load. A quantized node is 96 bytes and the slab
// is 256-byte aligned, so the node's three 32-byte parts are aligned.
__device__ __forceinline__ void load_slot8(const float4 *P, float4 &a, float4 &b) {
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(P));
}

// 2^e as fp32 for e in [-126, 127].
__device__ __forceinline__ float pow2i(int e) { return __int_as_float((e + 127) << 23); }
// Byte b of w as the fp32 value 2^23 + byte (exact), assembled by a byte
// permute; the caster subtracts 2^23 from two such values with one packed
// instruction, which gives the byte exactly.
__device__ __forceinline__ float qraw(uint32_t w, int b) {
  return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u + (uint32_t)b));
}

// Slot-order bits to rank order: bit s moves to bit s ^ oct (three
// conditional swaps of bit groups).
__device__ __forceinline__ uint32_t rank_bits(uint32_t x, uint32_t oct) {
  if (oct & 1u) x = ((x & 0x55u) << 1) | ((x >> 1) & 0x55u);
  if (oct & 2u) x = ((x & 0x33u) << 2) | ((x >> 2) & 0x33u);
  if (oct & 4u) x = ((x & 0x0fu) << 4) | ((x >> 4) & 0x0fu);
  return x;
}

// ref[s] without local memory: a select tree on the bits of s.
__device__ __forceinline__ int32_t pick8(const int32_t (&ref)[8], uint32_t s) {
  const int32_t r01 = (s & 1u) ? ref[1] : ref[0], r23 = (s & 1u) ? ref[3] : ref[2];
  const int32_t r45 = (s & 1u) ? ref[5] : ref[4], r67 = (s & 1u) ? ref[7] : ref[6];
  const int32_t r03 = (s & 2u) ? r23 : r01, r47 = (s & 2u) ? r67 : r45;
  return (s & 4u) ? r47 : r03;
}

// One node step of one ray: the node's child refs, the entered inner slots
// (slot order), the hit leaf slots, and the nearest entered inner slot.
struct WideStep {
  int32_t ref[8];
  uint32_t hin, leafmask, nearest;
};

// A step loads the 96-byte node with three 256-bit loads: a child's plane
// o + q * 2^e is entered at (o - ray.o) / d + q * (2^e / d), one FMA per
// plane on the byte q. Each axis's near and far byte words are picked once
// per node by the sign of 1/d. Per slot and axis, the near and far planes
// take one packed FMA on the pair of exact byte values (2^23 + q assembled by
// a byte permute, 2^23 subtracted). The nearest entered inner child is the
// minimum of keys (entry distance with its low three bits replaced by the
// slot), an order within 8 ulps of the distances; an infinite entry distance
// leaves no usable key, and the lowest entered slot is taken instead. Empty
// slots hold an inverted box and miss.
__device__ __forceinline__ void wide_node_test(const float4 *__restrict__ bvh8, int node, const TraceRay &r,
                                               uint32_t oct, float closest, WideStep &w) {
  const float INF = __int_as_float(0x7f800000);
  const f2 qbias2 = pk2(8388608.0f, 8388608.0f);  // the 2^23 of qraw, twice
  const float4 *N = bvh8 + 6ll * node;
  float4 q0, q1, q2, q3, q4, q5;
  load_slot8(N, q0, q1);
  load_slot8(N + 2, q2, q3);
  load_slot8(N + 4, q4, q5);
  const uint32_t ew = __float_as_uint(q0.w);
  const float sx = r.ix() * pow2i((int)(int8_t)(ew & 0xffu));
  const float sy = r.iy() * pow2i((int)(int8_t)((ew >> 8) & 0xffu));
  const float sz = r.iz() * pow2i((int)(int8_t)((ew >> 16) & 0xffu));
  const float ax = (q0.x - r.o.x) * r.ix(), ay = (q0.y - r.o.y) * r.iy(), az = (q0.z - r.o.z) * r.iz();
  // Near and far byte words per axis (slots 0-3, 4-7): lo for a positive
  // 1/d, hi for a negative one.
  const bool fx = (oct & 1u) != 0, fy = (oct & 2u) != 0, fz = (oct & 4u) != 0;
  const uint32_t lx0 = __float_as_uint(q1.x), lx1 = __float_as_uint(q1.y);
  const uint32_t ly0 = __float_as_uint(q1.z), ly1 = __float_as_uint(q1.w);
  const uint32_t lz0 = __float_as_uint(q2.x), lz1 = __float_as_uint(q2.y);
  const uint32_t hx0 = __float_as_uint(q2.z), hx1 = __float_as_uint(q2.w);
  const uint32_t hy0 = __float_as_uint(q3.x), hy1 = __float_as_uint(q3.y);
  const uint32_t hz0 = __float_as_uint(q3.z), hz1 = __float_as_uint(q3.w);
  const uint32_t nw[6] = {fx ? hx0 : lx0, fx ? hx1 : lx1, fy ? hy0 : ly0,
                          fy ? hy1 : ly1, fz ? hz0 : lz0, fz ? hz1 : lz1};
  const uint32_t fw[6] = {fx ? lx0 : hx0, fx ? lx1 : hx1, fy ? ly0 : hy0,
                          fy ? ly1 : hy1, fz ? lz0 : hz0, fz ? lz1 : hz1};
  w.ref[0] = __float_as_int(q4.x), w.ref[1] = __float_as_int(q4.y), w.ref[2] = __float_as_int(q4.z);
  w.ref[3] = __float_as_int(q4.w), w.ref[4] = __float_as_int(q5.x), w.ref[5] = __float_as_int(q5.y);
  w.ref[6] = __float_as_int(q5.z), w.ref[7] = __float_as_int(q5.w);
  const f2 sxx = pk2(sx, sx), syy = pk2(sy, sy), szz = pk2(sz, sz);
  const f2 axx = pk2(ax, ax), ayy = pk2(ay, ay), azz = pk2(az, az);
  uint32_t hin = 0, leafmask = 0;
  float kbest = INF;
#pragma unroll
  for (int s = 0; s < 8; s++) {
    const int wi = s >> 2, b = s & 3;
    const f2 tx = fma2(sub2(pk2(qraw(nw[0 + wi], b), qraw(fw[0 + wi], b)), qbias2), sxx, axx);
    const f2 ty = fma2(sub2(pk2(qraw(nw[2 + wi], b), qraw(fw[2 + wi], b)), qbias2), syy, ayy);
    const f2 tz = fma2(sub2(pk2(qraw(nw[4 + wi], b), qraw(fw[4 + wi], b)), qbias2), szz, azz);
    const float tn = max3f(lo2(tx), lo2(ty), fmaxf(lo2(tz), r.tmin));
    const float tf = min3f(hi2(tx), hi2(ty), fminf(hi2(tz), closest));
    if (tn <= tf) {
      if (w.ref[s] >= 0) {
        hin |= 1u << s;
        kbest = fminf(kbest, __uint_as_float((__float_as_uint(tn) & ~7u) | (uint32_t)s));
      } else {
        leafmask |= 1u << s;
      }
    }
  }
  w.hin = hin;
  w.leafmask = leafmask;
  w.nearest = kbest < INF ? (__float_as_uint(kbest) & 7u) : (uint32_t)(__ffs(hin) - 1);
}

// Closest hit of one ray through the 8-wide nodes, one thread on its own
// (the megakernel's bounce rays): the nearest entered child next, the node
// and its other entered children kept as one group entry (rank bits s ^ oct)
// on a stack of GSTACK entries (one per bvh8 level at most), leaves tested
// when their node is reached. The hit equals every other traversal's (the
// acceptance rule of test_triangle). Returns the leaf index or -1.
template <int GSTACK>
__device__ __forceinline__ int traverse_wide_lane(const DevScene &sc, const TraceRay &r, float &closest, float &bu,
                                                  float &bv, uint32_t *err) {
  const float root = slab_enter(r, sc.root_lo[0], sc.root_hi[0], sc.root_lo[1], sc.root_hi[1], sc.root_lo[2],
                                sc.root_hi[2], closest);
  if (!(root < __int_as_float(0x7f800000))) return -1;
  const uint32_t oct = (uint32_t)ray_octant(r);
  const int32_t *__restrict__ words8 = reinterpret_cast<const int32_t *>(sc.bvh8);
  uint32_t gstack[GSTACK];
  int gsp = 0, best = -1;
  uint32_t gnode = 0, gmask = 0, steps = 0;
  const uint32_t step_cap = sc.n8 + 16u;
  int node = sc.root8;
  for (;;) {
    if (node < 0) {
      if (gmask == 0) {
        if (gsp == 0) break;
        const uint32_t e = gstack[--gsp];
        gnode = e >> 8;
        gmask = e & 0xffu;
      }
      const uint32_t rk = (uint32_t)(__ffs(gmask) - 1);
      gmask &= gmask - 1u;
      node = __ldg(words8 + 24ll * gnode + 16 + (rk ^ oct));
    }
    if ((uint32_t)node >= sc.n8 || ++steps > step_cap) {
      atomicOr(err, (uint32_t)node >= sc.n8 ? KERR_BAD_INDEX : KERR_TIMEOUT);
      break;
    }
    WideStep ws;
    wide_node_test(sc.bvh8, node, r, oct, closest, ws);
    // Leaf refs were range-checked when the bvh8 was built (k_encode8).
    for (uint32_t m = ws.leafmask; m; m &= m - 1u)
      test_triangle(sc.tpre, sc.leaf_tri, ~pick8(ws.ref, (uint32_t)(__ffs(m) - 1)), r, closest, best, bu, bv);
    const int node_idx = node;
    node = -1;
    if (ws.hin) {
      if (gmask) {
        if (gsp >= GSTACK) {
          atomicOr(err, KERR_STACK_OVERFLOW);
          break;
        }
        gstack[gsp++] = (gnode << 8) | gmask;
      }
      gnode = (uint32_t)node_idx;
      gmask = rank_bits(ws.hin, oct) & ~(1u << (ws.nearest ^ oct));
      node = pick8(ws.ref, ws.nearest);
    }
  }
  return best;
}

}  // namespace rtgb
