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
// index and t equal the reference's except when two triangles return the
// same t, where "first found" depends on the visiting order.
#pragma once
#include "rt_internal.h"
#include "rt_math.cuh"

namespace rtgb {

struct TraceRay {
  f3 o, d;
  float ix, iy, iz;     // 1 / d (tiny components clamped)
  float ox, oy, oz;     // o / d, for fma slab planes
  float tmin;
};

__device__ __forceinline__ float safe_rcp(float x) {
  const float tiny = 1e-30f;
  return __frcp_rn(fabsf(x) > tiny ? x : copysignf(tiny, x));
}

__device__ __forceinline__ TraceRay make_ray(f3 o, f3 d, float tmin) {
  TraceRay r;
  r.o = o;
  r.d = d;
  r.ix = safe_rcp(d.x);
  r.iy = safe_rcp(d.y);
  r.iz = safe_rcp(d.z);
  r.ox = o.x * r.ix;
  r.oy = o.y * r.iy;
  r.oz = o.z * r.iz;
  r.tmin = tmin;
  return r;
}

// Slab test of [lo, hi] against [tmin, tmax]; returns the entry distance or
// +inf when the box is missed.
__device__ __forceinline__ float slab_enter(const TraceRay &r, float lx, float hx, float ly, float hy, float lz,
                                            float hz, float tmax) {
  float ax = fmaf(lx, r.ix, -r.ox), bx = fmaf(hx, r.ix, -r.ox);
  float ay = fmaf(ly, r.iy, -r.oy), by = fmaf(hy, r.iy, -r.oy);
  float az = fmaf(lz, r.iz, -r.oz), bz = fmaf(hz, r.iz, -r.oz);
  float tn = fmaxf(fmaxf(fminf(ax, bx), fminf(ay, by)), fmaxf(fminf(az, bz), r.tmin));
  float tf = fminf(fminf(fmaxf(ax, bx), fmaxf(ay, by)), fminf(fmaxf(az, bz), tmax));
  return tn <= tf ? tn : __int_as_float(0x7f800000);
}

// triIntersect on a precomputed record; updates (closest, best, u, v) when
// the triangle is accepted. Bit-exact with the fp32 evaluation of comp:157-173.
__device__ __forceinline__ void test_triangle(const float4 *__restrict__ tpre, int k, const TraceRay &r,
                                              float &closest, int &best, float &bu, float &bv) {
  const float4 *T = tpre + 3ll * k;
  float4 t0 = __ldg(T), t1 = __ldg(T + 1), t2 = __ldg(T + 2);
  f3 v0 = mk3(t0.x, t0.y, t0.z), n = mk3(t0.w, t1.x, t1.y);
  f3 a = mk3(t1.z, t1.w, t2.x), b = mk3(t2.y, t2.z, t2.w);
  f3 p = sub3(v0, r.o);
  float idet = __fdiv_rn(1.0f, dot3(r.d, n));
  float t = __fmul_rn(dot3(n, p), idet);
  if (t > r.tmin && t < closest) {
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
template <int STACK>
__device__ __forceinline__ int traverse_closest(const DevScene &sc, const TraceRay &r, float &closest, float &bu,
                                                float &bv, uint32_t *err) {
  int best = -1;
  float root = slab_enter(r, sc.root_lo[0], sc.root_hi[0], sc.root_lo[1], sc.root_hi[1], sc.root_lo[2],
                          sc.root_hi[2], closest);
  if (!(root < __int_as_float(0x7f800000))) return -1;
  int stack[STACK];
  int sp = 0;
  int node = sc.root_ref;
  const float4 *__restrict__ bvh = sc.bvh2;
  for (;;) {
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
          return best;
        }
        stack[sp++] = farc;
        node = nearc;
      } else if (h0) {
        node = r0;
      } else if (h1) {
        node = r1;
      } else {
        if (sp == 0) return best;
        node = stack[--sp];
      }
    }
    test_triangle(sc.tpre, ~node, r, closest, best, bu, bv);
    if (sp == 0) return best;
    node = stack[--sp];
  }
}

}  // namespace rtgb
