// The per-path part of the reference shader: hit records, spheres, scatter,
// light sampling, ray_color and the running-mean accumulation
// (resources/shaders/source/ray-trace-compute.comp:44-155, 175-203,
// 314-379; include/definitions.glsl:42-53; include/random.glsl:24-52).
// Every floating-point step is written in the shader's order with
// round-to-nearest intrinsics (rt_math.cuh).
#pragma once
#include "rt_internal.h"
#include "rt_math.cuh"
#include "traverse.cuh"
#include "wide.cuh"

namespace rtgb {

constexpr float kPi = 3.1415926535897932385f;  // random.glsl:1
constexpr float kTmin = 0.001f;                 // comp:264
constexpr float kTmax = 10000.0f;               // comp:265

struct HitRec {
  f3 p, normal;
  uint32_t mat;
  float t;
  int back;
};

// Shader-literal hit_bvh (comp:262-311) for RT_COMPAT_STACK16: always push
// left then right, no t-culling, and stop when 16 entries are in use.
__device__ __forceinline__ int traverse_literal16(const DevScene &sc, f3 o, f3 d, float tmin, float &closest,
                                                  float &bu, float &bv) {
  int stack[18];
  int sp = 0, best = -1;
  stack[sp++] = 0;
  while (sp > 0 && sp < 16) {
    sp--;
    int node = stack[sp];
    if (node == -1) continue;
    const rt_bvh_node nd = sc.nodes[node];
    float ax = __fdiv_rn(__fsub_rn(nd.min[0], o.x), d.x), bx = __fdiv_rn(__fsub_rn(nd.max[0], o.x), d.x);
    float ay = __fdiv_rn(__fsub_rn(nd.min[1], o.y), d.y), by = __fdiv_rn(__fsub_rn(nd.max[1], o.y), d.y);
    float az = __fdiv_rn(__fsub_rn(nd.min[2], o.z), d.z), bz = __fdiv_rn(__fsub_rn(nd.max[2], o.z), d.z);
    float tn = fmaxf(fmaxf(fminf(ax, bx), fminf(ay, by)), fminf(az, bz));
    float tf = fminf(fminf(fmaxf(ax, bx), fmaxf(ay, by)), fmaxf(az, bz));
    if (tn > tf) continue;
    if (nd.object != -1) {
      const rt_triangle tr = sc.tris[nd.object];
      f3 v0 = ld3(tr.v0), v1 = ld3(tr.v1), v2 = ld3(tr.v2);
      f3 a = sub3(v0, v1), b = sub3(v2, v0);
      f3 n = cross3(b, a);
      f3 p = sub3(v0, o);
      float idet = __frcp_rn(dot3(d, n));  // correctly rounded 1/x: the value of the IEEE division 1.0f / x
      float t = __fmul_rn(dot3(n, p), idet);
      f3 q = cross3(p, d);
      float u = __fmul_rn(dot3(q, b), idet);
      float v = __fmul_rn(dot3(q, a), idet);
      if (!(u < 0.0f || u > 1.0f || v < 0.0f || __fadd_rn(u, v) > 1.0f) && t > tmin && t < closest) {
        closest = t;
        best = nd.object;
        bu = u;
        bv = v;
      }
    }
    stack[sp++] = nd.left;
    stack[sp++] = nd.right;
  }
  return best;
}

// hit_triangle's record (comp:209-216) for an accepted triangle with
// face normal n = cross(b, a).
__device__ __forceinline__ void triangle_record(f3 o, f3 d, float t, f3 n, uint32_t mat, HitRec &rec) {
  rec.p = add3(o, mul3(t, d));
  rec.normal = normalize3(n);
  rec.back = dot3(d, rec.normal) > 0.0f ? 1 : 0;
  rec.normal = mul3((float)(1 - 2 * rec.back), rec.normal);
  rec.p = add3(rec.p, mul3(0.0001f, rec.normal));
  rec.t = t;
  rec.mat = mat;
}

// hit_sphere (comp:175-203).
__device__ __forceinline__ bool hit_sphere(const rt_sphere &sp, f3 o, f3 d, float tmin, float tmax, HitRec &rec) {
  f3 c = mk3(sp.s[0], sp.s[1], sp.s[2]);
  float radius = sp.s[3];
  f3 oc = sub3(o, c);
  float a = dot3(d, d);
  float half_b = dot3(oc, d);
  float cc = __fsub_rn(dot3(oc, oc), __fmul_rn(radius, radius));
  float disc = __fsub_rn(__fmul_rn(half_b, half_b), __fmul_rn(a, cc));
  if (disc < 0.0f) return false;
  float sq = __fsqrt_rn(disc);
  int back = 0;
  float root = __fdiv_rn(__fsub_rn(-half_b, sq), a);
  if (root < tmin || tmax < root) {
    root = __fdiv_rn(__fadd_rn(-half_b, sq), a);
    back = 1;
    if (root < tmin || tmax < root) return false;
  }
  rec.back = back;
  rec.t = root;
  rec.p = add3(o, mul3(root, d));
  rec.normal = divs3(mul3((float)(1 - 2 * back), sub3(rec.p, c)), radius);
  rec.mat = sp.material_index;
  return true;
}

struct PathState {
  uint32_t nlights;   // lights.length() as the path sees it
  uint32_t nspheres;  // spheres.length() as the path sees it
  int sphere_mode;    // 0 none, 1 closest hit, 2 reference override
  uint32_t flags;
};

__device__ __forceinline__ PathState path_state(const DevScene &sc, uint32_t flags) {
  PathState ps;
  bool len1 = (flags & RT_COMPAT_LEN1) != 0;
  ps.nlights = len1 ? min(sc.nlights, 1u) : sc.nlights;
  ps.nspheres = len1 ? min(sc.nspheres, 1u) : sc.nspheres;
  ps.sphere_mode = (flags & RT_COMPAT_NO_SPHERES) ? 0 : ((flags & RT_COMPAT_SPHERE_OVERRIDE) ? 2 : 1);
  ps.flags = flags;
  return ps;
}

// Spheres after the BVH: with `closest` carried over (true closest hit),
// reset to tmax as the reference's hit_scene does (comp:236), or skipped.
__device__ __forceinline__ bool sphere_pass(const DevScene &sc, const PathState &ps, f3 o, f3 d, bool hit,
                                            HitRec &rec) {
  if (ps.sphere_mode != 0) {
    float lim = (ps.sphere_mode == 2) ? kTmax : (hit ? rec.t : kTmax);
    for (uint32_t j = 0; j < ps.nspheres; j++) {
      HitRec tmp;
      if (hit_sphere(sc.spheres[j], o, d, kTmin, lim, tmp)) {
        hit = true;
        lim = tmp.t;
        rec = tmp;
      }
    }
  }
  return hit;
}

// Record of the triangle leaf k (position in tpre) hit at t, then the sphere
// pass. Shared by the megakernel and the wavefront shade step.
__device__ __forceinline__ bool resolve_hit(const DevScene &sc, const PathState &ps, f3 o, f3 d, int k,
                                            float closest, HitRec &rec) {
  bool hit = false;
  if (k >= 0) {
    const float4 *T = sc.tpre + 3ll * k;
    float4 t0 = __ldg(T), t1 = __ldg(T + 1);
    uint32_t mat = __ldg(&sc.tris[__ldg(sc.leaf_tri + k)].material_index);
    triangle_record(o, d, closest, mk3(t0.w, t1.x, t1.y), mat, rec);
    hit = true;
  }
  return sphere_pass(sc, ps, o, d, hit, rec);
}

// Closest hit of a path segment: triangles through the BVH, then spheres.
template <int STACK>
__device__ __forceinline__ bool closest_hit(const DevScene &sc, const PathState &ps, f3 o, f3 d, HitRec &rec,
                                            uint32_t *err) {
  float closest = kTmax, u = 0.0f, v = 0.0f;
  if (ps.flags & RT_COMPAT_STACK16) {
    bool hit = false;
    int ti = traverse_literal16(sc, o, d, kTmin, closest, u, v);
    if (ti >= 0) {
      const rt_triangle tr = sc.tris[ti];
      f3 v0 = ld3(tr.v0), v1 = ld3(tr.v1), v2 = ld3(tr.v2);
      triangle_record(o, d, closest, cross3(sub3(v2, v0), sub3(v0, v1)), tr.material_index, rec);
      hit = true;
    }
    return sphere_pass(sc, ps, o, d, hit, rec);
  }
  TraceRay r = make_ray(o, d, kTmin);
  // Bounce rays: per thread over the 8-wide nodes (levels of the fold never
  // exceed the binary tree's, so STACK group entries suffice).
  int k = sc.bvh8 ? traverse_wide_lane<STACK>(sc, r, closest, u, v, err)
                  : traverse_spec<STACK>(sc, r, true, closest, u, v, err);
  return resolve_hit(sc, ps, o, d, k, closest, rec);
}

// random_in_unit_sphere (random.glsl:29-32) through random(min, max) (24-27).
__device__ __forceinline__ f3 random_in_unit_sphere(Rng &g) {
  const float lo = -0.3f, span = __fsub_rn(0.3f, -0.3f);
  float x = __fadd_rn(lo, __fmul_rn(span, g.next()));
  float y = __fadd_rn(lo, __fmul_rn(span, g.next()));
  float z = __fadd_rn(lo, __fmul_rn(span, g.next()));
  return normalize3(mk3(x, y, z));
}

// sampleLambertian (comp:91-99) with Onb/onbLocal and random_cosine_direction.
__device__ __forceinline__ f3 sample_lambertian(f3 normal, Rng &g) {
  f3 w = normalize3(normal);
  f3 a = (fabsf(w.x) > 0.9f) ? mk3(0.0f, 1.0f, 0.0f) : mk3(1.0f, 0.0f, 0.0f);
  f3 v = normalize3(cross3(w, a));
  f3 u = cross3(w, v);
  float r1 = g.next();
  float r2 = g.next();
  float z = __fsqrt_rn(__fsub_rn(1.0f, r2));
  float phi = __fmul_rn(__fmul_rn(2.0f, kPi), r1);
  float sr2 = __fsqrt_rn(r2);
  float x = __fmul_rn(cosf(phi), sr2);
  float y = __fmul_rn(sinf(phi), sr2);
  return normalize3(add3(add3(mul3(x, u), mul3(y, v)), mul3(z, w)));
}

// sampleGlass (comp:106-116); `ir` is the index of refraction.
__device__ __forceinline__ f3 sample_glass(f3 I, const HitRec &rec, float ir) {
  float ratio = __fadd_rn(__fdiv_rn(__fmul_rn((float)(1 - rec.back), 1.0f), ir), __fmul_rn((float)rec.back, ir));
  f3 i = normalize3(I);
  float cos_t = gmin(dot3(neg3(i), rec.normal), 1.0f);
  float sin_t = __fsqrt_rn(__fsub_rn(1.0f, __fmul_rn(cos_t, cos_t)));
  float t = floorf(gclamp(__fmul_rn(ratio, sin_t), 0.0f, 1.0f));
  f3 rf = reflect3(i, rec.normal);
  f3 rr = refract3(i, rec.normal, ratio);
  return add3(mul3(t, rf), mul3(__fsub_rn(1.0f, t), rr));
}

// sampleLight + randomOnATriangle (comp:67-89); false when |cos| < 0.001.
__device__ __forceinline__ bool sample_light(const DevScene &sc, uint32_t nlights, f3 p, Rng &g, f3 &dir) {
  float len = (float)nlights;
  int idx = (int)floorf(__fmul_rn(len, g.next()));
  if (idx >= (int)nlights) idx = (int)nlights - 1;  // random() may return exactly 1.0
  const rt_triangle tr = sc.tris[sc.lights[idx].triangle_index];
  float s = g.next();
  float t = g.next();
  f3 v0 = ld3(tr.v0), v1 = ld3(tr.v1), v2 = ld3(tr.v2);
  f3 v01 = add3(neg3(v0), v1);
  f3 v02 = add3(neg3(v0), v2);
  f3 on = add3(add3(v0, mul3(s, v01)), mul3(t, v02));
  f3 to = normalize3(sub3(on, p));
  dir = to;
  return !(fabsf(fabsf(to.y)) < 0.001f);
}

// scatter (comp:118-155); returns true for an emitter.
__device__ __forceinline__ bool scatter(const DevScene &sc, const PathState &ps, f3 d_in, const HitRec &rec, Rng &g,
                                        f3 &albedo, f3 &out_dir) {
  const rt_material m = sc.mats[rec.mat];
  albedo = ld3(m.albedo);
  if (ps.flags & RT_SHADE_SIMPLE) {
    // ray-trace-compute-simple.comp:62-68.
    f3 in = random_in_unit_sphere(g);
    f3 h = (dot3(in, rec.normal) > 0.0f) ? in : neg3(in);
    out_dir = normalize3(h);
    return m.type == RT_MATERIAL_LIGHT;
  }
  f3 ms = mk3(0.0f, 0.0f, 0.0f);
  if (m.type == RT_MATERIAL_LAMBERTIAN) {
    ms = sample_lambertian(rec.normal, g);
  } else if (m.type == RT_MATERIAL_METAL) {
    ms = reflect3(d_in, rec.normal);
    if (m.fuzz > 0.0f) ms = add3(ms, mul3(m.fuzz, random_in_unit_sphere(g)));
  } else if (m.type == RT_MATERIAL_GLASS) {
    ms = sample_glass(d_in, rec, m.ior > 0.0f ? m.ior : 1.5f);
    albedo = mk3(1.0f, 1.0f, 1.0f);
  }
  f3 fin = ms;
  float coin = g.next();
  if (coin < 0.5f && m.type == RT_MATERIAL_LAMBERTIAN && ps.nlights > 0) {
    f3 ld;
    if (sample_light(sc, ps.nlights, rec.p, g, ld)) fin = ld;
  }
  out_dir = fin;
  return m.type == RT_MATERIAL_LIGHT;
}

// ray_color (comp:314-338) for the camera ray through pixel (x, y);
// `segments` counts traced segments.
// k0 value that asks ray_color to trace the first segment itself.
constexpr int kTraceFirst = -2;

template <int STACK>
__device__ __forceinline__ f3 ray_color(const DevScene &sc, const PathState &ps, f3 o, f3 d, int k0, float t0,
                                        uint32_t max_bounces, Rng &g, uint32_t &segments, uint32_t *err) {
  // The bounce loop of comp:314-338. The first segment's triangle result
  // (leaf k0, distance t0) comes from the caller, which traces it once for
  // every sample; the sphere pass and the hit record are redone here.
  f3 color = mk3(1.0f, 1.0f, 1.0f);
  for (uint32_t i = 0; i < max_bounces; i++) {
    HitRec rec;
    bool hit;
    if (i == 0 && k0 != kTraceFirst) {
      hit = resolve_hit(sc, ps, o, d, k0, t0, rec);
    } else {
      segments++;
      hit = closest_hit<STACK>(sc, ps, o, d, rec, err);
    }
    if (hit) {
      f3 albedo, nd;
      bool emits = scatter(sc, ps, d, rec, g, albedo, nd);
      color = mulv3(color, albedo);
      o = rec.p;
      d = nd;
      if (emits) break;
    } else {
      color = mul3(0.0f, color);
      break;
    }
  }
  return color;
}

// Triangles along the camera segment of a warp's pixels (warp-converged call;
// inactive lanes take part without a ray): coherent warps traverse as one
// packet, others lane by lane with postponed leaves. Returns the leaf index
// (or -1) and its distance in t; kTraceFirst under the 16-entry compat
// traversal, which stays per sample as in the shader.
template <int STACK>
__device__ __forceinline__ int camera_hit(const DevScene &sc, const PathState &ps, f3 o, f3 d, bool active,
                                          float &t, uint32_t *err, volatile int *s_stack) {
  if (ps.flags & RT_COMPAT_STACK16) return kTraceFirst;
  TraceRay r = make_ray(o, d, kTmin);
  float closest = kTmax, u = 0.0f, v = 0.0f;
  int k;
  const int oct = warp_octant(active, r);
  if (warp_is_coherent(active, r)) {
#define RTGB_CALL(O) k = traverse_packet<STACK, O>(sc, r, active, closest, u, v, s_stack, err)
    RTGB_OCT_DISPATCH(oct, RTGB_CALL)
#undef RTGB_CALL
  } else {
#define RTGB_CALL(O) k = traverse_spec<STACK, O>(sc, r, active, closest, u, v, err)
    RTGB_OCT_DISPATCH(oct, RTGB_CALL)
#undef RTGB_CALL
  }
  t = closest;
  return k;
}

// Camera ray direction for pixel (x, y) (comp:371-372).
__device__ __forceinline__ f3 camera_dir(const rt_camera &cam, uint32_t x, uint32_t y, uint32_t W, uint32_t H) {
  float u = __fdiv_rn((float)x, (float)W), v = __fdiv_rn((float)y, (float)H);
  f3 llc = ld3(cam.lower_left), hor = ld3(cam.horizontal), ver = ld3(cam.vertical), org = ld3(cam.origin);
  return sub3(add3(add3(llc, mul3(u, hor)), mul3(v, ver)), org);
}

__device__ __forceinline__ float unorm8(float x) {
  float c = gclamp(x, 0.0f, 1.0f);
  return __fdiv_rn(floorf(__fadd_rn(__fmul_rn(c, 255.0f), 0.5f)), 255.0f);
}

// spp samples of one pixel accumulated into the running mean (comp:375-379).
// Warp-converged call; `active` lanes own a pixel. The camera ray carries no
// jitter (comp:371-372: uv = gid / size), so every sample of the call starts
// with the same first segment: its triangles are traversed once (camera_hit)
// and each sample's bounce loop continues from that result with its own RNG
// stream, which gives the same image as tracing it per sample. Returns the
// number of segments traced.
template <int STACK>
__device__ __forceinline__ uint32_t render_pixel(const DevScene &sc, const PathState &ps, const rt_camera &cam,
                                                 const rt_render_params &p, uint32_t x, uint32_t y, bool active,
                                                 float4 *accum, uint32_t *err, volatile int *s_stack) {
  f3 org = ld3(cam.origin);
  f3 d0 = active ? normalize3(camera_dir(cam, x, y, p.width, p.height)) : mk3(1.0f, 0.0f, 0.0f);
  int k0 = kTraceFirst;
  float t0 = 0.0f;
  uint32_t segments = 0;
  if (p.max_bounces > 0 && p.spp > 0) {  // uniform across the warp (one job per tile)
    k0 = camera_hit<STACK>(sc, ps, org, d0, active, t0, err, s_stack);
    if (k0 != kTraceFirst && active) segments = 1;
  }
  if (!active) return 0;
  float4 acc = accum[(size_t)y * p.width + x];
  for (uint32_t k = 0; k < p.spp; k++) {
    uint32_t s = p.sample_index + k;
    Rng g{(600u * x + y) * (s + 1u)};
    f3 c = ray_color<STACK>(sc, ps, org, d0, k0, t0, p.max_bounces, g, segments, err);
    float sf = (float)s;
    float keep = gmin(sf, 1.0f);
    float den = __fadd_rn(sf, 1.0f);
    acc.x = __fdiv_rn(__fadd_rn(c.x, __fmul_rn(__fmul_rn(acc.x, keep), sf)), den);
    acc.y = __fdiv_rn(__fadd_rn(c.y, __fmul_rn(__fmul_rn(acc.y, keep), sf)), den);
    acc.z = __fdiv_rn(__fadd_rn(c.z, __fmul_rn(__fmul_rn(acc.z, keep), sf)), den);
    acc.w = __fdiv_rn(__fadd_rn(1.0f, __fmul_rn(__fmul_rn(acc.w, keep), sf)), den);
    if (p.flags & RT_COMPAT_UNORM8) {
      acc.x = unorm8(acc.x);
      acc.y = unorm8(acc.y);
      acc.z = unorm8(acc.z);
      acc.w = unorm8(acc.w);
    }
  }
  accum[(size_t)y * p.width + x] = acc;
  return segments;
}

}  // namespace rtgb
