// Beam traversal for tiles of rays that share an origin (camera tiles):
// up to 256 rays walk the binary tree once, as one beam, instead of once per
// warp packet. The beam is the cone of directions over the tile's rays,
// bounded by four planes through the origin in the projection on the rays'
// dominant axis (u = d_u / d_z, v = d_v / d_z over the tile), plus the
// half-space in front of the origin. A producer warp expands the beam's
// frontier, up to 32 stacked nodes at a time (one per lane, nearest first),
// and collects the leaves whose boxes meet the beam into rounds of at least
// 64; while it fills the next round, the eight ray warps test the current
// one: each warp first drops the leaves outside its own, narrower cone (one
// leaf per lane), then every lane runs its own slab test on each remaining
// leaf and the triangle test where that passes (traverse.cuh:
// slab_hit_child, test_triangle).
//
// Results equal the per-ray traversal's. A ray's slab test passes a box
// only if the ray meets the box (to within the rounding of the slab
// values, ~1e-7 relative), and every child box lies inside its parent's.
// The cone tests run on boxes inflated by 1e-5 of their distance from the
// origin and on cones widened beyond their rays' directions, so a box a
// cone drops is one none of its rays enters: every leaf a ray's own
// traversal would test is tested. Boxes farther from the origin than every
// ray's current closest hit (distance = t * |d|, plus 1%) are dropped too;
// that bound only shrinks. The hit rule is order-free (test_triangle), so
// the order of the leaves does not matter.
#pragma once
#include "rt_internal.h"
#include "rt_math.cuh"
#include "traverse.cuh"

namespace rtgb {

constexpr int kBeamRayWarps = 8;                       // warps holding rays
constexpr int kBeamRays = 32 * kBeamRayWarps;          // rays per tile, one per thread
constexpr int kBeamThreads = kBeamRays + 32;           // plus the producer warp
constexpr int kBeamStack = 2048;                       // frontier entries (inner node refs)
constexpr int kBeamBatch = 64;                         // leaves per round (at least, but the last)
constexpr int kBeamPop = 1;                            // frontier entries per producer lane and step
constexpr int kBeamLeafCap = kBeamBatch + 64 * kBeamPop;  // one step adds at most 64 per entry a lane pops
// Largest extent of a tile's directions in the projection (u and v each);
// wider tiles go to the warp packets.
constexpr float kBeamMaxSpan = 0.25f;

// Round states (rstate): the last round, more rounds follow, abandoned.
constexpr int kRoundLast = 0, kRoundMore = 1, kRoundAbandon = 2;

struct BeamShared {
  float4 leaf[2][kBeamLeafCap][2];  // two rounds of child records (traverse.cuh layout)
  int stack[kBeamStack];
  float o[3];       // the tile's origin
  float lim[4];     // umin, umax, vmin, vmax of the tile's cone (widened)
  float sz;         // sign of the dominant axis
  uint32_t u_lo, u_hi, v_lo, v_hi;  // ordered-float reductions of u and v
  uint32_t md[2];   // per round: farthest closest-hit distance after its tests (fp32 bits, >= 0)
  uint32_t tile;    // the tile being cast
  int za, oct, ok;  // dominant axis, near-first octant, beam usable
  int sp;           // frontier size (producer only)
  int nleaf[2], rstate[2];
};

// fp32 to uint32 with unsigned order equal to float order (for min/max).
__device__ __forceinline__ uint32_t beam_ord(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float beam_unord(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// A cone of directions from an origin: u, v bounds in the projection on
// axis za (rays go to sz * z > 0).
struct Cone {
  float o[3];
  float umin, umax, vmin, vmax, sz;
  int za;
};

// True when the child box (p, q) may meet the cone within distance^2 maxd2.
// Child record layout: lo = (p.x, p.y, q.x), hi = (p.z, p.w, q.y). ZA: the
// cone's axis when known at compile time (-1: read c.za).
template <int ZA = -1>
__device__ __forceinline__ bool cone_box(const Cone &c, float4 p, float4 q, float maxd2) {
  const int za = ZA >= 0 ? ZA : c.za;
  // Box relative to the origin, axes permuted to (u, v, z).
  const float lx = p.x - c.o[0], hx = p.z - c.o[0], ly = p.y - c.o[1], hy = p.w - c.o[1];
  const float lz = q.x - c.o[2], hz = q.y - c.o[2];
  float ul = za == 0 ? ly : (za == 1 ? lz : lx), uh = za == 0 ? hy : (za == 1 ? hz : hx);
  float vl = za == 0 ? lz : (za == 1 ? lx : ly), vh = za == 0 ? hz : (za == 1 ? hx : hy);
  float zl = za == 0 ? lx : (za == 1 ? ly : lz), zh = za == 0 ? hx : (za == 1 ? hy : hz);
  // Inflated by 1e-5 of the distance from the origin.
  const float eu = 1e-5f * fmaxf(fabsf(ul), fabsf(uh)) + 1e-30f;
  const float ev = 1e-5f * fmaxf(fabsf(vl), fabsf(vh)) + 1e-30f;
  const float ez = 1e-5f * fmaxf(fabsf(zl), fabsf(zh)) + 1e-30f;
  ul -= eu, uh += eu, vl -= ev, vh += ev, zl -= ez, zh += ez;
  // Depth along the dominant axis, signed so that the rays go to +Z.
  const float Zl = c.sz > 0.0f ? zl : -zh, Zh = c.sz > 0.0f ? zh : -zl;
  // In front of the origin and inside the four side planes (u * Z <= y_u
  // <= ...): each plane keeps the box when its best corner is inside.
  const bool in = Zh >= 0.0f && uh - c.umin * (c.umin >= 0.0f ? Zl : Zh) >= 0.0f &&
                  c.umax * (c.umax >= 0.0f ? Zh : Zl) - ul >= 0.0f &&
                  vh - c.vmin * (c.vmin >= 0.0f ? Zl : Zh) >= 0.0f && c.vmax * (c.vmax >= 0.0f ? Zh : Zl) - vl >= 0.0f;
  // Nearest point of the box to the origin.
  const float du = fmaxf(fmaxf(ul, -uh), 0.0f), dv = fmaxf(fmaxf(vl, -vh), 0.0f), dz = fmaxf(fmaxf(zl, -zh), 0.0f);
  return in && (du * du + dv * dv + dz * dz <= maxd2);
}

// The producer warp (all 32 lanes, converged) fills round buffer `buf`:
// it expands the frontier until the round holds kBeamBatch leaves or the
// frontier is empty. Each step pops up to 32 * E entries (entry j in lane
// j % 32, the top first), tests both children of each popped node against
// the tile's cone (the E node loads of a lane in flight together), appends
// the leaves to the round and pushes the inner children back with the
// popped order kept (entry 0's near child on top). A frontier overflow, a
// bad ref or more steps than the tree has nodes abandon the beam: the tile
// is then cast by warp packets.
template <int ZA, int E>
__device__ __forceinline__ void beam_expand(BeamShared &s, const Cone &cone, const DevScene &sc, uint32_t lane,
                                            uint32_t *err, int buf, float maxd2) {
  const uint32_t lt = (1u << lane) - 1u, gt = ~lt & ~(1u << lane);
  int sp = s.sp, nleaf = 0, state = kRoundMore;
  const float4 *__restrict__ bvh = sc.bvh2;
  const uint32_t inner_count = sc.ntris - 1u;  // pair nodes
  uint32_t steps = 0;
  while (sp > 0 && nleaf < kBeamBatch) {
    const int take = sp < 32 * E ? sp : 32 * E;
    int node[E];
    bool mine[E], bad = false;
#pragma unroll
    for (int e = 0; e < E; e++) {
      mine[e] = (int)lane + 32 * e < take;
      node[e] = mine[e] ? s.stack[sp - 1 - (int)lane - 32 * e] : 0;
      bad |= mine[e] && (uint32_t)node[e] >= inner_count;
    }
    sp -= take;
    bad = __any_sync(0xffffffffu, bad);
    if (bad || ++steps > sc.ntris + 16u) {
      if (lane == 0) atomicOr(err, bad ? KERR_BAD_INDEX : KERR_TIMEOUT);
      state = kRoundAbandon;
      break;
    }
    float4 a[E], b[E], c[E], d[E];
#pragma unroll
    for (int e = 0; e < E; e++) {
      a[e] = b[e] = c[e] = d[e] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (mine[e]) load_node(bvh + 4ll * node[e], a[e], b[e], c[e], d[e]);
    }
    // Deeper popped entries (higher j) first: their children go below.
    bool full = false;
#pragma unroll
    for (int e = E - 1; e >= 0; e--) {
      const bool h0 = mine[e] && cone_box<ZA>(cone, a[e], b[e], maxd2);
      const bool h1 = mine[e] && cone_box<ZA>(cone, c[e], d[e], maxd2);
      const int r0 = __float_as_int(b[e].z), r1 = __float_as_int(d[e].z);
      const bool in0 = h0 && r0 >= 0, in1 = h1 && r1 >= 0, lf0 = h0 && r0 < 0, lf1 = h1 && r1 < 0;
      const uint32_t bi0 = __ballot_sync(0xffffffffu, in0), bi1 = __ballot_sync(0xffffffffu, in1);
      const uint32_t bl0 = __ballot_sync(0xffffffffu, lf0), bl1 = __ballot_sync(0xffffffffu, lf1);
      const int pushes = __popc(bi0) + __popc(bi1), leaves = __popc(bl0) + __popc(bl1);
      if (sp + pushes > kBeamStack || nleaf + leaves > kBeamLeafCap) {
        full = true;
        break;
      }
      const int pos = sp + __popc(bi0 & gt) + __popc(bi1 & gt);
      if (in0 && in1) {
        const bool f1 = child1_first(b[e], s.oct);
        s.stack[pos] = f1 ? r0 : r1;      // far
        s.stack[pos + 1] = f1 ? r1 : r0;  // near, on top
      } else if (in0 || in1) {
        s.stack[pos] = in0 ? r0 : r1;
      }
      sp += pushes;
      int lpos = nleaf + __popc(bl0 & lt) + __popc(bl1 & lt);
      if (lf0) {
        s.leaf[buf][lpos][0] = a[e];
        s.leaf[buf][lpos][1] = b[e];
        lpos++;
      }
      if (lf1) {
        s.leaf[buf][lpos][0] = c[e];
        s.leaf[buf][lpos][1] = d[e];
      }
      nleaf += leaves;
    }
    if (full) {
      state = kRoundAbandon;
      break;
    }
    __syncwarp();
  }
  if (state == kRoundMore && sp == 0) state = kRoundLast;
  __syncwarp();
  if (lane == 0) {
    s.sp = sp;
    s.nleaf[buf] = nleaf;
    s.rstate[buf] = state;
  }
}

// A ray warp tests round `buf`: leaves outside the warp's cone (within the
// warp's farthest closest hit) are dropped one leaf per lane, then every
// lane tests the rest against its own ray.
template <int OCT>
__device__ __forceinline__ void beam_test_round(const BeamShared &s, int buf, int nleaf, const Cone &wcone,
                                                float wmaxd2, uint32_t lane, const DevScene &sc,
                                                const TraceRay &r, bool active, float &closest, int &best,
                                                float &bu, float &bv) {
  for (int c0 = 0; c0 < nleaf; c0 += 32) {
    const int j = c0 + (int)lane;
    const bool keep = j < nleaf && cone_box<>(wcone, s.leaf[buf][j][0], s.leaf[buf][j][1], wmaxd2);
    uint32_t m = __ballot_sync(0xffffffffu, keep);
    if (!active) continue;
    for (; m; m &= m - 1u) {
      const int k = c0 + __ffs(m) - 1;
      const float4 p = s.leaf[buf][k][0], q = s.leaf[buf][k][1];
      if (slab_hit_child<OCT>(r, p, q, closest))
        test_triangle(sc.tpre, sc.leaf_tri, ~__float_as_int(q.z), r, closest, best, bu, bv);
    }
  }
}

}  // namespace rtgb
