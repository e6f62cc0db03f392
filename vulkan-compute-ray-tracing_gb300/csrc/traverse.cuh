// Closest-hit traversal over the children-pair layout (see rt_internal.h).
//
// Semantics: the hit_bvh loop of ray-trace-compute.comp:262-311 — the
// closest triangle with tmin < t < closest, accepted with the strict `t <
// closest` of comp:217, tested with triIntersect (comp:157-173) in the same
// fp32 rounding. What changes is the visiting order and the pruning: boxes
// are tested with the current closest t (the reference tests only
// tNear <= tFar, comp:286) and the nearer child is visited first. Pruning
// never skips a box that holds a closer accepted hit, because every box is
// the union of its triangles' boxes padded by 1e-4 (Bvh.h:94-98); so the hit
// index and t equal the reference's except when two triangles return exactly
// the same t: the reference keeps the first one its order meets, here the
// lower triangle index wins (test_triangle), which no order or tree changes.
#pragma once
#include "rt_internal.h"
#include "rt_math.cuh"

namespace rtgb {

// The slab planes of a box are entered at fma(plane, 1/d, -o/d), computed
// two at a time with packed FMAs: (lo.x, lo.y) and (hi.x, hi.y) against
// (1/dx, 1/dy), (lo.z, hi.z) against (1/dz, 1/dz).
struct TraceRay {
  f3 o, d;
  f2 ixy, izz;  // 1 / d (tiny components clamped) as (x, y) and (z, z)
  f2 nxy, nzz;  // -o / d in the same pairs
  float tmin;
  __device__ __forceinline__ float ix() const { return lo2(ixy); }
  __device__ __forceinline__ float iy() const { return hi2(ixy); }
  __device__ __forceinline__ float iz() const { return lo2(izz); }
};

__device__ __forceinline__ float safe_rcp(float x) {
  const float tiny = 1e-30f;
  return __frcp_rn(fabsf(x) > tiny ? x : copysignf(tiny, x));
}

__device__ __forceinline__ TraceRay make_ray(f3 o, f3 d, float tmin) {
  TraceRay r;
  r.o = o;
  r.d = d;
  const float ix = safe_rcp(d.x), iy = safe_rcp(d.y), iz = safe_rcp(d.z);
  const float ox = __fmul_rn(o.x, ix), oy = __fmul_rn(o.y, iy), oz = __fmul_rn(o.z, iz);
  r.ixy = pk2(ix, iy);
  r.izz = pk2(iz, iz);
  r.nxy = pk2(-ox, -oy);
  r.nzz = pk2(-oz, -oz);
  r.tmin = tmin;
  return r;
}

// One children-pair node (64 bytes, see rt_internal.h) in two 256-bit loads
// (sm_100 and later; the pair array starts 256-byte aligned and every node
// is 64 bytes, so both halves are 32-byte aligned). Half the load
// instructions, and half the L1 requests, of four 128-bit loads.
__device__ __forceinline__ void load_node(const float4 *N, float4 &a, float4 &b, float4 &c, float4 &d) {
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(N));
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(c.x), "=f"(c.y), "=f"(c.z), "=f"(c.w), "=f"(d.x), "=f"(d.y), "=f"(d.z), "=f"(d.w)
      : "l"(N + 2));
}

// Three-operand fp32 min/max (sm_100 and later), NaN operands ignored as
// with fminf/fmaxf.
__device__ __forceinline__ float max3f(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// Slab test of [lo, hi] against [tmin, tmax]; returns the entry distance or
// +inf when the box is missed.
//
// OCT = -1: the near/far plane of each axis is picked with min/max. OCT in
// 0..7: the caller knows the signs of the ray's inverse direction (bit 0: x
// negative, bit 1: y, bit 2: z), so the near plane is lo for a positive
// component and hi for a negative one, chosen at compile time. For boxes with
// lo <= hi both forms give the same bits: fma(lo, i, -o) <= fma(hi, i, -o)
// for i > 0 because rounding is monotonic, so min/max pick exactly those
// values. The fixed form saves six ALU operations per box.
// The box is given as the pairs (lo.x, lo.y), (hi.x, hi.y), (lo.z, hi.z).
template <int OCT = -1>
__device__ __forceinline__ void slab_span(const TraceRay &r, f2 lxy, f2 hxy, f2 lhz, float tmax, float &tn,
                                          float &tf) {
  const f2 pa = fma2(lxy, r.ixy, r.nxy), pb = fma2(hxy, r.ixy, r.nxy), pz = fma2(lhz, r.izz, r.nzz);
  const float ax = lo2(pa), ay = hi2(pa), bx = lo2(pb), by = hi2(pb), az = lo2(pz), bz = hi2(pz);
  if (OCT < 0) {
    tn = max3f(fminf(ax, bx), fminf(ay, by), fmaxf(fminf(az, bz), r.tmin));
    tf = min3f(fmaxf(ax, bx), fmaxf(ay, by), fminf(fmaxf(az, bz), tmax));
  } else {
    const float nx = (OCT & 1) ? bx : ax, fx = (OCT & 1) ? ax : bx;
    const float ny = (OCT & 2) ? by : ay, fy = (OCT & 2) ? ay : by;
    const float nz = (OCT & 4) ? bz : az, fz = (OCT & 4) ? az : bz;
    tn = max3f(nx, ny, fmaxf(nz, r.tmin));
    tf = min3f(fx, fy, fminf(fz, tmax));
  }
}

template <int OCT = -1>
__device__ __forceinline__ float slab_enter(const TraceRay &r, float lx, float hx, float ly, float hy, float lz,
                                            float hz, float tmax) {
  float tn, tf;
  slab_span<OCT>(r, pk2(lx, ly), pk2(hx, hy), pk2(lz, hz), tmax, tn, tf);
  return tn <= tf ? tn : __int_as_float(0x7f800000);
}

// The same test as a flag, for loops that order children without distances,
// on one child record of a pair node: (lo.x, lo.y, hi.x, hi.y) in `p`,
// (lo.z, hi.z, ref, order) in `q` (load_node gives child 0 as (a, b) and
// child 1 as (c, d)).
template <int OCT = -1>
__device__ __forceinline__ bool slab_hit_child(const TraceRay &r, float4 p, float4 q, float tmax) {
  float tn, tf;
  slab_span<OCT>(r, pk2(p.x, p.y), pk2(p.z, p.w), pk2(q.x, q.y), tmax, tn, tf);
  return tn <= tf;
}

// Near-first order at a pair node: true when child 1 is visited first by
// rays of sign octant `oct` (the order bits, in either child record's `q`,
// relayout.cu). Any order
// gives the same hit; this one needs no entry distance.
__device__ __forceinline__ bool child1_first(float4 q, int oct) { return (__float_as_uint(q.w) >> oct) & 1u; }

// Sign octant of the ray's inverse direction (the OCT of slab_enter).
__device__ __forceinline__ int ray_octant(const TraceRay &r) {
  return (r.ix() < 0.0f ? 1 : 0) | (r.iy() < 0.0f ? 2 : 0) | (r.iz() < 0.0f ? 4 : 0);
}

// The octant shared by every active lane of the warp, or -1 (mixed, or no
// active lane). Warp-converged call.
__device__ __forceinline__ int warp_octant(bool active, const TraceRay &r) {
  const uint32_t act = __ballot_sync(0xffffffffu, active);
  if (act == 0) return -1;
  const int mine = ray_octant(r);
  const int first = __shfl_sync(0xffffffffu, mine, __ffs(act) - 1);
  return __all_sync(0xffffffffu, !active || mine == first) ? first : -1;
}

// triIntersect on a precomputed record; updates (closest, best, u, v) when
// the triangle is accepted. Bit-exact with the fp32 evaluation of comp:157-173.
// Acceptance is the shader's tmin < t < closest, except that a triangle at
// exactly the current closest t replaces the current one when its triangle
// index is lower: the reference keeps whichever equal-t triangle its
// visiting order meets first, which makes the winner depend on the order
// (and on the tree); with this rule every traversal order, ray ordering and
// tree returns the same triangle. The index loads happen only on exact ties.
__device__ __forceinline__ void test_triangle(const float4 *__restrict__ tpre, const int32_t *__restrict__ leaf_tri,
                                              int k, const TraceRay &r, float &closest, int &best, float &bu,
                                              float &bv) {
  const float4 *T = tpre + 3ll * k;
  float4 t0 = __ldg(T), t1 = __ldg(T + 1), t2 = __ldg(T + 2);
  f3 v0 = mk3(t0.x, t0.y, t0.z), n = mk3(t0.w, t1.x, t1.y);
  f3 a = mk3(t1.z, t1.w, t2.x), b = mk3(t2.y, t2.z, t2.w);
  f3 p = sub3(v0, r.o);
  float idet = __frcp_rn(dot3(r.d, n));  // correctly rounded 1/x: the value of the IEEE division 1.0f / x
  float t = __fmul_rn(dot3(n, p), idet);
  if (t > r.tmin &&
      (t < closest || (t == closest && best >= 0 && __ldg(leaf_tri + k) < __ldg(leaf_tri + best)))) {
    f3 q = cross3(p, r.d);
    float u = __fmul_rn(dot3(q, b), idet);
    float v = __fmul_rn(dot3(q, a), idet);
    if (!(u < 0.0f || u > 1.0f || v < 0.0f || __fadd_rn(u, v) > 1.0f)) {
      closest = t;
      best = k;
      bu = u;
      bv = v;
    }
  }
}

// Returns the leaf index (position in tpre) of the closest hit or -1.
// The traversal stack is stack[i * stride] for i < STACK: a per-thread local
// array (stride 1) or a column of a shared-memory block (stride = threads
// per block, so each lane keeps to its own bank).
template <int STACK>
__device__ __forceinline__ int traverse_closest_on(const DevScene &sc, const TraceRay &r, float &closest, float &bu,
                                                   float &bv, uint32_t *err, int *stack, int stride) {
  int best = -1;
  float root = slab_enter(r, sc.root_lo[0], sc.root_hi[0], sc.root_lo[1], sc.root_hi[1], sc.root_lo[2],
                          sc.root_hi[2], closest);
  if (!(root < __int_as_float(0x7f800000))) return -1;
  int sp = 0;
  int node = sc.root_ref;
  const int oct = ray_octant(r);
  const float4 *__restrict__ bvh = sc.bvh2;
  for (;;) {
    while (node >= 0) {
      const float4 *N = bvh + 4ll * node;
      float4 a, b, c, d;
      load_node(N, a, b, c, d);
      const bool h0 = slab_hit_child(r, a, b, closest);
      const bool h1 = slab_hit_child(r, c, d, closest);
      int r0 = __float_as_int(b.z), r1 = __float_as_int(d.z);
      if (h0 && h1) {
        const bool f1 = child1_first(b, oct);
        const int nearc = f1 ? r1 : r0, farc = f1 ? r0 : r1;
        if (sp >= STACK) {
          atomicOr(err, KERR_STACK_OVERFLOW);
          return best;
        }
        stack[(sp++) * stride] = farc;
        node = nearc;
      } else if (h0) {
        node = r0;
      } else if (h1) {
        node = r1;
      } else {
        if (sp == 0) return best;
        node = stack[(--sp) * stride];
      }
    }
    test_triangle(sc.tpre, sc.leaf_tri, ~node, r, closest, best, bu, bv);
    if (sp == 0) return best;
    node = stack[(--sp) * stride];
  }
}

template <int STACK>
__device__ __forceinline__ int traverse_closest(const DevScene &sc, const TraceRay &r, float &closest, float &bu,
                                                float &bv, uint32_t *err) {
  int stack[STACK];
  return traverse_closest_on<STACK>(sc, r, closest, bu, bv, err, stack, 1);
}

// Per-lane traversal with postponed leaves (Aila and Laine, "Understanding
// the Efficiency of Ray Traversal on GPUs", HPG 2009, speculative
// traversal): a lane that reaches a leaf parks it and keeps descending inner
// nodes until every lane of the warp in the loop holds a leaf; then all
// parked leaves are tested together. Lanes no longer idle in the inner loop
// while others are still descending. The extra nodes a lane may visit before
// its parked triangle shortens `closest` never change the result: every
// reached triangle is tested with the same acceptance rule. The warp votes
// only decide when to switch phases. Refs: inner node >= 0, leaf ~k < 0,
// kEnd (the stack's bottom entry) when the lane is finished.
template <int STACK, int OCT = -1>
__device__ __forceinline__ int traverse_spec(const DevScene &sc, const TraceRay &r, bool active, float &closest,
                                             float &bu, float &bv, uint32_t *err) {
  constexpr int kEnd = 0x7fffffff;
  int stack[STACK];
  stack[0] = kEnd;
  int sp = 1;
  int best = -1;
  int node = kEnd, leaf = 0;
  if (active) {
    float root = slab_enter(r, sc.root_lo[0], sc.root_hi[0], sc.root_lo[1], sc.root_hi[1], sc.root_lo[2],
                            sc.root_hi[2], closest);
    if (root < __int_as_float(0x7f800000)) node = sc.root_ref;
  }
  const int oct = OCT >= 0 ? OCT : ray_octant(r);
  const float4 *__restrict__ bvh = sc.bvh2;
  while (node != kEnd || leaf < 0) {
    // A leaf in hand and none parked (only when the root is a leaf).
    if (node < 0 && leaf >= 0) {
      leaf = node;
      node = stack[--sp];
    }
    while (node >= 0 && node != kEnd) {
      const float4 *N = bvh + 4ll * node;
      float4 a, b, c, d;
      load_node(N, a, b, c, d);
      const bool h0 = slab_hit_child<OCT>(r, a, b, closest);
      const bool h1 = slab_hit_child<OCT>(r, c, d, closest);
      int r0 = __float_as_int(b.z), r1 = __float_as_int(d.z);
      if (h0 && h1) {
        const bool f1 = child1_first(b, oct);
        const int nearc = f1 ? r1 : r0, farc = f1 ? r0 : r1;
        if (sp >= STACK) {
          atomicOr(err, KERR_STACK_OVERFLOW);
          return best;
        }
        stack[sp++] = farc;
        node = nearc;
      } else if (h0) {
        node = r0;
      } else if (h1) {
        node = r1;
      } else {
        node = stack[--sp];
      }
      // Park the first leaf reached and keep going.
      if (node < 0 && leaf >= 0) {
        leaf = node;
        node = stack[--sp];
      }
      // Every lane still here holds a parked leaf: test them.
      if (!__any_sync(__activemask(), leaf >= 0)) break;
    }
    // The parked leaf, then any leaves the lane stands on.
    while (leaf < 0) {
      test_triangle(sc.tpre, sc.leaf_tri, ~leaf, r, closest, best, bu, bv);
      leaf = node;
      if (node < 0) node = stack[--sp];
    }
  }
  return best;
}

// Dispatch to the octant-specialised instance when the warp's rays share
// one sign octant (warp-uniform branch), else the generic one.
#define RTGB_OCT_DISPATCH(oct, CALL)                     \
  switch (oct) {                                         \
    case 0: CALL(0); break;                              \
    case 1: CALL(1); break;                              \
    case 2: CALL(2); break;                              \
    case 3: CALL(3); break;                              \
    case 4: CALL(4); break;                              \
    case 5: CALL(5); break;                              \
    case 6: CALL(6); break;                              \
    case 7: CALL(7); break;                              \
    default: CALL(-1); break;                            \
  }

// Warp-wide packet traversal for 32 coherent rays: the warp walks one node
// sequence with one stack, descending into a child when ANY active lane's
// box test passes with that lane's own closest t; every active lane then
// tests each reached leaf's triangle against its own ray. Each lane's result
// is exactly its per-ray closest hit (the packet visits a superset of every
// lane's required nodes); only the number of visited nodes changes.
// Inactive lanes carry closest = -inf, so they miss every box and accept no
// triangle without extra tests. Near/far order comes from the node's order
// bits for the packet's octant. The stack is warp-distributed in registers for STACK <= 32 (entry j
// in lane j, read back with a shuffle), else in shared memory. All branches
// are warp-uniform except inside the triangle test.
template <int STACK, int OCT = -1>
__device__ __forceinline__ int traverse_packet(const DevScene &sc, const TraceRay &r, bool active, float &closest,
                                               float &bu, float &bv, volatile int *stack, uint32_t *err) {
  // Hardware lane id: callers run 1-D and 2-D blocks alike.
  uint32_t lane;
  asm("mov.u32 %0, %%laneid;" : "=r"(lane));
  const float INF = __int_as_float(0x7f800000);
  const float saved = closest;
  if (!active) closest = -INF;
  int best = -1;
  const uint32_t act = __ballot_sync(0xffffffffu, active);
  const int src = act ? __ffs(act) - 1 : 0;
  float root = slab_enter(r, sc.root_lo[0], sc.root_hi[0], sc.root_lo[1], sc.root_hi[1], sc.root_lo[2],
                          sc.root_hi[2], closest);
  if (!__any_sync(0xffffffffu, root < INF)) {
    closest = saved;
    return -1;
  }
  int sp = 0;
  int node = sc.root_ref;
  int reg_stack = 0;  // entry `lane` of the register stack (STACK <= 32)
  // The packet's octant (the first active lane's for a mixed warp) picks
  // the near child from the node's order bits.
  const int oct = OCT >= 0 ? OCT : __shfl_sync(0xffffffffu, ray_octant(r), src);
  const uint32_t ref_span = 2u * sc.ntris - 1u;
  const float4 *__restrict__ bvh = sc.bvh2;
  for (;;) {
    if (node >= 0) {
      const float4 *N = bvh + 4ll * node;
      float4 a, b, c, d;
      load_node(N, a, b, c, d);
      const bool any0 = __any_sync(0xffffffffu, slab_hit_child<OCT>(r, a, b, closest));
      const bool any1 = __any_sync(0xffffffffu, slab_hit_child<OCT>(r, c, d, closest));
      const int r0 = __float_as_int(b.z), r1 = __float_as_int(d.z);
      if (any0 && any1) {
        const bool f1 = child1_first(b, oct);
        if (sp >= STACK) {
          if (lane == 0) atomicOr(err, KERR_STACK_OVERFLOW);
          break;
        }
        const int farc = f1 ? r0 : r1;
        if (STACK <= 32) {
          if (lane == (uint32_t)sp) reg_stack = farc;
        } else {
          if (lane == 0) stack[sp] = farc;
          __syncwarp();
        }
        sp++;
        node = f1 ? r1 : r0;
        continue;
      } else if (any0) {
        node = r0;
        continue;
      } else if (any1) {
        node = r1;
        continue;
      }
    } else {
      test_triangle(sc.tpre, sc.leaf_tri, ~node, r, closest, best, bu, bv);
    }
    if (sp == 0) break;
    --sp;
    node = STACK <= 32 ? __shfl_sync(0xffffffffu, reg_stack, sp) : stack[sp];
    // A popped ref is an inner node (< ntris - 1) or a leaf ~k (k < ntris):
    // node + ntris lies in [0, 2 ntris - 1).
    if ((uint32_t)node + sc.ntris >= ref_span) {
      if (lane == 0) atomicOr(err, KERR_BAD_INDEX);
      break;
    }
  }
  if (!active) closest = saved;
  return active ? best : -1;
}

// True when the warp's 32 rays suit packet traversal: active lanes share one
// origin and all directions lie within ~72 degrees of the first active one.
// Morton-ordered camera rays are within a fraction of a degree of each other
// except for the few chunks that straddle a jump of the Z-order curve (two
// tight clusters up to half the field of view apart); a packet over such a
// chunk visits at most the two clusters' nodes, far cheaper than leaving it
// to a per-lane pass at the end of the cast.
__device__ __forceinline__ bool warp_is_coherent(bool active, const TraceRay &r) {
  const uint32_t act = __ballot_sync(0xffffffffu, active);
  if (act == 0) return false;
  const int src = __ffs(act) - 1;
  float ox = __shfl_sync(0xffffffffu, r.o.x, src), oy = __shfl_sync(0xffffffffu, r.o.y, src);
  float oz = __shfl_sync(0xffffffffu, r.o.z, src);
  float dx = __shfl_sync(0xffffffffu, r.d.x, src), dy = __shfl_sync(0xffffffffu, r.d.y, src);
  float dz = __shfl_sync(0xffffffffu, r.d.z, src);
  bool ok = true;
  if (active) {
    float dd = r.d.x * dx + r.d.y * dy + r.d.z * dz;
    float n0 = dx * dx + dy * dy + dz * dz, n1 = r.d.x * r.d.x + r.d.y * r.d.y + r.d.z * r.d.z;
    ok = r.o.x == ox && r.o.y == oy && r.o.z == oz && dd > 0.3f * sqrtf(n0 * n1);
  }
  return __all_sync(0xffffffffu, ok);
}

}  // namespace rtgb
