// Beam traversal for tiles of rays that share an origin (camera tiles):
// up to 256 rays walk the binary tree once, as one beam, instead of once per
// warp packet. The beam is the cone of directions over the tile's rays,
// bounded by four planes through the origin in the projection on the rays'
// dominant axis (u = d_u / d_z, v = d_v / d_z over the tile), plus the
// half-space in front of the origin. The block alternates two phases.
// Expansion: all eight warps pop up to 256 frontier nodes at once (one per
// thread, nearest first), test both children of each against the tile's
// cone, append the leaves to the round and push the inner children back
// in order; steps repeat until the round holds trace.beam_round leaves (64)
// or the frontier is empty. Testing: each warp drops the round's leaves outside its own,
// narrower cone (one leaf per lane), then every lane runs its own slab test
// on each remaining leaf and the triangle test where that passes
// (traverse.cuh: slab_hit_child, test_triangle).
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

constexpr int kBeamWarps = 8;
constexpr int kBeamRays = 32 * kBeamWarps;            // rays per tile, one per thread
constexpr int kBeamStack = 2048;                      // frontier entries (inner node refs)
constexpr int kBeamRoundMax = 256;                    // leaves a round collects before testing (trace.beam_round, at most)
constexpr int kBeamLeafCap = kBeamRoundMax + 2 * kBeamRays;  // one step adds at most two per thread
// Largest extent of a tile's directions in the projection (u and v each);
// wider tiles go to the warp packets.
constexpr float kBeamMaxSpan = 0.25f;

struct BeamShared {
  float4 leaf[kBeamLeafCap][2];  // the round's child records (traverse.cuh layout)
  int stack[kBeamStack];
  int2 cnt[kBeamWarps];  // per warp and step: pushes, leaves
  float o[3];       // the tile's origin
  float lim[4];     // umin, umax, vmin, vmax of the tile's cone (widened)
  float sz;         // sign of the dominant axis
  uint32_t u_lo, u_hi, v_lo, v_hi;  // ordered-float reductions of u and v
  uint32_t md[2];   // per round (alternating): farthest closest-hit distance after its tests (fp32 bits)
  uint32_t tile;    // the tile being cast
  int za, oct, ok;  // dominant axis, near-first octant, beam usable
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

// One expansion step by the whole block (block-converged call with two
// block barriers; sp and nleaf are the same in every thread). Thread j
// pops frontier entry j from the top, tests both children of its node
// against the tile's cone, and the block appends the leaves to the round
// and pushes the inner children back with the popped order kept: deeper
// entries' children below, entry 0's near child on top. Returns false,
// with nothing written, on a bad ref (reported) or when the frontier or the
// round would overflow.
template <int ZA>
__device__ __forceinline__ bool beam_step(BeamShared &s, const Cone &cone, const DevScene &sc, uint32_t lane,
                                          uint32_t warp, int &sp, int &nleaf, float maxd2, uint32_t *err) {
  const uint32_t lt = (1u << lane) - 1u, gt = ~lt & ~(1u << lane);
  const int j = (int)(warp * 32u + lane);
  const int take = sp < kBeamRays ? sp : kBeamRays;
  const bool mine = j < take;
  const int node = mine ? s.stack[sp - 1 - j] : 0;
  bool bad = mine && (uint32_t)node >= sc.ntris - 1u;  // pair nodes are 0 .. ntris - 2
  float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a, c = a, d = a;
  bool h0 = false, h1 = false;
  if (mine && !bad) {
    load_node(sc.bvh2 + 4ll * node, a, b, c, d);
    h0 = cone_box<ZA>(cone, a, b, maxd2);
    h1 = cone_box<ZA>(cone, c, d, maxd2);
  }
  const int r0 = __float_as_int(b.z), r1 = __float_as_int(d.z);
  // Leaf refs ~k name a triangle record, k < ntris.
  bad |= (h0 && r0 < 0 && (uint32_t)~r0 >= sc.ntris) || (h1 && r1 < 0 && (uint32_t)~r1 >= sc.ntris);
  const bool in0 = h0 && r0 >= 0, in1 = h1 && r1 >= 0, lf0 = h0 && r0 < 0, lf1 = h1 && r1 < 0;
  const uint32_t bi0 = __ballot_sync(0xffffffffu, in0), bi1 = __ballot_sync(0xffffffffu, in1);
  const uint32_t bl0 = __ballot_sync(0xffffffffu, lf0), bl1 = __ballot_sync(0xffffffffu, lf1);
  if (lane == 0) s.cnt[warp] = make_int2(__popc(bi0) + __popc(bi1), __popc(bl0) + __popc(bl1));
  if (__syncthreads_or(bad)) {
    if (warp == 0 && lane == 0) atomicOr(err, KERR_BAD_INDEX);
    return false;
  }
  // Deeper warps' children go below; leaves in warp order.
  int below = sp - take, lbase = nleaf, pushes = 0, leaves = 0;
#pragma unroll
  for (int w = 0; w < kBeamWarps; w++) {
    const int2 cw = s.cnt[w];
    pushes += cw.x;
    leaves += cw.y;
    if (w > (int)warp) below += cw.x;
    if (w < (int)warp) lbase += cw.y;
  }
  const int nsp = sp - take + pushes, nnl = nleaf + leaves;
  if (nsp > kBeamStack || nnl > kBeamLeafCap) return false;
  const int pos = below + __popc(bi0 & gt) + __popc(bi1 & gt);
  if (in0 && in1) {
    const bool f1 = child1_first(b, s.oct);
    s.stack[pos] = f1 ? r0 : r1;      // far
    s.stack[pos + 1] = f1 ? r1 : r0;  // near, on top
  } else if (in0 || in1) {
    s.stack[pos] = in0 ? r0 : r1;
  }
  int lpos = lbase + __popc(bl0 & lt) + __popc(bl1 & lt);
  if (lf0) {
    s.leaf[lpos][0] = a;
    s.leaf[lpos][1] = b;
    lpos++;
  }
  if (lf1) {
    s.leaf[lpos][0] = c;
    s.leaf[lpos][1] = d;
  }
  __syncthreads();
  sp = nsp;
  nleaf = nnl;
  return true;
}

// A warp tests the round: leaves outside the warp's cone (within the
// warp's farthest closest hit) are dropped one leaf per lane, then every
// lane tests the rest against its own ray.
template <int OCT>
__device__ __forceinline__ void beam_test_round(const BeamShared &s, int nleaf, const Cone &wcone,
                                                float wmaxd2, uint32_t lane, const DevScene &sc,
                                                const TraceRay &r, bool active, float &closest, int &best,
                                                float &bu, float &bv) {
  for (int c0 = 0; c0 < nleaf; c0 += 32) {
    const int j = c0 + (int)lane;
    const bool keep = j < nleaf && cone_box<>(wcone, s.leaf[j][0], s.leaf[j][1], wmaxd2);
    uint32_t m = __ballot_sync(0xffffffffu, keep);
    if (!active) continue;
    for (; m; m &= m - 1u) {
      const int k = c0 + __ffs(m) - 1;
      const float4 p = s.leaf[k][0], q = s.leaf[k][1];
      if (slab_hit_child<OCT>(r, p, q, closest))
        test_triangle(sc.tpre, sc.leaf_tri, ~__float_as_int(q.z), r, closest, best, bu, bv);
    }
  }
}

}  // namespace rtgb
