// Test infrastructure (oracle) — NOT part of the product.
//
// A CPU restatement of the reference's ray-trace hot path, used only by the
// tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, as the
// oracle. Nothing in the product links, loads or calls this file.
//
// What it restates (reference paths relative to the reference checkout):
//   * Bvh::createBvh            src/ray-tracing/Bvh.h:141-209 (with helpers 16-122)
//   * RtScene light list        src/ray-tracing/RtScene.h:87-96
//   * the compute shader        resources/shaders/source/ray-trace-compute.comp:44-380
//     with include/definitions.glsl:1-53 and include/random.glsl:1-52
//   * the alternate scatter     resources/shaders/source/ray-trace-compute-simple.comp:62-68
//
// Parity pins: the BVH restatement is checked field-for-field against the
// reference's own Bvh.h compiled by oracle/Makefile (oracle/_ref); the shader
// restatement has no reference output to pin to (the reference ships no tests
// and its GLSL needs a Vulkan stack that is not available), so its parity is
// unpinned by the reference and rests on review against the shader source and
// on the golden vectors committed under tests/golden.
//
// Arithmetic is written operation by operation in GLSL's order and built with
// -ffp-contract=off, so the fp32 instantiation is bit-reproducible on x86-64
// and aarch64. The fp64 instantiation evaluates the same formulas in double
// and is the error reference for t and the barycentrics.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <omp.h>

#include "../include/rtgb/rt_types.h"

namespace {

// ---------------------------------------------------------------- GLSL helpers
template <typename T> struct V3 {
  T x, y, z;
};
template <typename T> inline V3<T> mk(T x, T y, T z) { return V3<T>{x, y, z}; }
template <typename T> inline V3<T> ld3(const float *p) { return mk<T>((T)p[0], (T)p[1], (T)p[2]); }
template <typename T> inline V3<T> add(V3<T> a, V3<T> b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
template <typename T> inline V3<T> sub(V3<T> a, V3<T> b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
template <typename T> inline V3<T> mul(T s, V3<T> a) { return mk(s * a.x, s * a.y, s * a.z); }
template <typename T> inline V3<T> mulv(V3<T> a, V3<T> b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
template <typename T> inline V3<T> divs(V3<T> a, T s) { return mk(a.x / s, a.y / s, a.z / s); }
template <typename T> inline V3<T> neg(V3<T> a) { return mk(-a.x, -a.y, -a.z); }
template <typename T> inline T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename T> inline V3<T> cross(V3<T> a, V3<T> b) {
  return mk(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
template <typename T> inline T gsqrt(T x) { return std::sqrt(x); }
template <typename T> inline T length(V3<T> a) { return gsqrt(dot(a, a)); }
template <typename T> inline V3<T> normalize(V3<T> a) { return divs(a, length(a)); }
// GLSL min/max as the specification words them.
template <typename T> inline T gmin(T x, T y) { return (y < x) ? y : x; }
template <typename T> inline T gmax(T x, T y) { return (x < y) ? y : x; }
template <typename T> inline T gclamp(T x, T lo, T hi) { return gmin(gmax(x, lo), hi); }
// reflect(I, N) = I - 2 * dot(N, I) * N
template <typename T> inline V3<T> reflect(V3<T> I, V3<T> N) {
  T s = (T)2 * dot(N, I);
  return sub(I, mul(s, N));
}
// refract(I, N, eta) as GLSL defines it (k < 0 gives the zero vector).
template <typename T> inline V3<T> refract(V3<T> I, V3<T> N, T eta) {
  T d = dot(N, I);
  T k = (T)1 - eta * eta * ((T)1 - d * d);
  if (k < (T)0) return mk<T>(0, 0, 0);
  return sub(mul(eta, I), mul(eta * d + gsqrt(k), N));
}

template <typename T> struct Consts;
template <> struct Consts<float> {
  static float pi() { return 3.1415926535897932385f; }
  static float inv_u32() { return 4294967295.0f; }
};
template <> struct Consts<double> {
  // The shader's constants are fp32; the fp64 path uses their fp32 values.
  static double pi() { return (double)3.1415926535897932385f; }
  static double inv_u32() { return (double)4294967295.0f; }
};
template <typename T> inline T tsin(T x) { return std::sin(x); }
template <typename T> inline T tcos(T x) { return std::cos(x); }

// ---------------------------------------------------------------- RNG (A7)
// random.glsl:4-22 — PCG-style step with inc = 1 and the RXS-M-XS output.
struct Rng {
  uint32_t s;
  template <typename T> T next() {
    s = s * 747796405u + 1u;
    uint32_t w = ((s >> ((s >> 28) + 4u)) ^ s) * 277803737u;
    w = (w >> 22) ^ w;
    return (T)((float)w / 4294967295.0f);
  }
};

// ---------------------------------------------------------------- hit record
template <typename T> struct Hit {
  V3<T> p, normal;
  uint32_t mat;
  T t;
  int back;
};

// triIntersect (comp:157-173) and hit_triangle (comp:205-220).
template <typename T>
inline bool tri_intersect(const rt_triangle &tr, V3<T> ro, V3<T> rd, T &t, T &u, T &v, V3<T> &n) {
  V3<T> v0 = ld3<T>(tr.v0), v1 = ld3<T>(tr.v1), v2 = ld3<T>(tr.v2);
  V3<T> a = sub(v0, v1);
  V3<T> b = sub(v2, v0);
  V3<T> p = sub(v0, ro);
  n = cross(b, a);
  V3<T> q = cross(p, rd);
  T idet = (T)1 / dot(rd, n);
  u = dot(q, b) * idet;
  v = dot(q, a) * idet;
  t = dot(n, p) * idet;
  return !(u < (T)0 || u > (T)1 || v < (T)0 || (u + v) > (T)1);
}

template <typename T>
inline bool hit_triangle(const rt_triangle &tr, V3<T> ro, V3<T> rd, T tmin, T tmax, Hit<T> &rec, T *uo,
                         T *vo) {
  T t, u, v;
  V3<T> n;
  if (!tri_intersect(tr, ro, rd, t, u, v, n)) return false;
  rec.p = add(ro, mul(t, rd));
  rec.normal = normalize(n);
  rec.back = dot(rd, rec.normal) > (T)0 ? 1 : 0;
  rec.normal = mul((T)(1 - 2 * rec.back), rec.normal);
  rec.p = add(rec.p, mul((T)0.0001f, rec.normal));
  rec.t = t;
  rec.mat = tr.material_index;
  if (uo) *uo = u;
  if (vo) *vo = v;
  return t > tmin && t < tmax;
}

// hit_sphere (comp:175-203).
template <typename T>
inline bool hit_sphere(const rt_sphere &sp, V3<T> ro, V3<T> rd, T tmin, T tmax, Hit<T> &rec) {
  V3<T> c = mk<T>((T)sp.s[0], (T)sp.s[1], (T)sp.s[2]);
  T radius = (T)sp.s[3];
  V3<T> oc = sub(ro, c);
  T a = dot(rd, rd);
  T half_b = dot(oc, rd);
  T cc = dot(oc, oc) - radius * radius;
  T disc = half_b * half_b - a * cc;
  if (disc < (T)0) return false;
  T sq = gsqrt(disc);
  int back = 0;
  T root = (-half_b - sq) / a;
  if (root < tmin || tmax < root) {
    root = (-half_b + sq) / a;
    back = 1;
    if (root < tmin || tmax < root) return false;
  }
  rec.back = back;
  rec.t = root;
  rec.p = add(ro, mul(root, rd));
  rec.normal = divs(mul((T)(1 - 2 * back), sub(rec.p, c)), radius);
  rec.mat = sp.material_index;
  return true;
}

// intersectAABB (comp:250-258) by division; NaN slabs (origin on a slab plane
// with a zero direction component) are dropped by fmin/fmax semantics.
template <typename T>
inline void slab(const rt_bvh_node &nd, V3<T> ro, V3<T> rd, T &tn, T &tf) {
  V3<T> bmin = ld3<T>(nd.min), bmax = ld3<T>(nd.max);
  V3<T> t0 = mk((bmin.x - ro.x) / rd.x, (bmin.y - ro.y) / rd.y, (bmin.z - ro.z) / rd.z);
  V3<T> t1 = mk((bmax.x - ro.x) / rd.x, (bmax.y - ro.y) / rd.y, (bmax.z - ro.z) / rd.z);
  T ax = std::fmin(t0.x, t1.x), ay = std::fmin(t0.y, t1.y), az = std::fmin(t0.z, t1.z);
  T bx = std::fmax(t0.x, t1.x), by = std::fmax(t0.y, t1.y), bz = std::fmax(t0.z, t1.z);
  tn = std::fmax(std::fmax(ax, ay), az);
  tf = std::fmin(std::fmin(bx, by), bz);
}

struct Scene {
  const rt_triangle *tris;
  uint32_t ntris;
  const rt_material *mats;
  uint32_t nmats;
  const rt_bvh_node *nodes;
  uint32_t nnodes;
  const rt_light *lights;
  uint32_t nlights;
  const rt_sphere *spheres;
  uint32_t nspheres;
};

struct TraceStats {
  uint32_t nodes;      // node records fetched
  uint32_t tris;       // triangle records fetched
  uint32_t flags;      // bit0: a second candidate within the tie window; bit1: stack truncated
  uint32_t _pad;
};

enum { FLAG_TIE = 1u, FLAG_TRUNCATED = 2u };

// Closest hit over the reference node array.
//   literal = true : hit_bvh exactly (comp:262-311): DFS that always pushes
//                    left then right, no t-culling, a stack of `stack_size`
//                    entries whose overflow ends the traversal; among
//                    candidates with exactly equal t the first met wins.
//   literal = false: the same hit set with t-culling and near-first order
//                    (unbounded stack); this is the cheapest exact traversal
//                    of the reference tree in the reference layout, and its
//                    record counts define the algorithmic bytes per ray.
//                    Exactly equal t: the lower triangle index wins.
// `slack` widens the cull window (tn > closest * (1 + slack)) so that every
// candidate within the tie window is seen; slack = 0 counts records exactly.
template <typename T>
bool trace_closest(const Scene &sc, V3<T> ro, V3<T> rd, T tmin, T tmax, bool literal, int stack_size,
                   double slack, Hit<T> &rec, T *uo, T *vo, int32_t *tri_out, TraceStats *st) {
  bool hit = false;
  T closest = tmax;
  T second = tmax;  // smallest accepted-range t among candidates other than the best
  int32_t best_tri = -1;
  uint32_t nvis = 0, ntri = 0, flags = 0;
  auto test_tri = [&](int32_t ti) {
    Hit<T> tmp;
    T u = 0, v = 0;
    ntri++;
    // Evaluate against tmax so that candidates beyond `closest` still update
    // the tie tracker; acceptance below is the shader's `t < closest`.
    bool ok = hit_triangle(sc.tris[ti], ro, rd, tmin, tmax, tmp, &u, &v);
    if (!ok) return;
    // Exactly equal t: the shader keeps the first one its visiting order
    // meets (comp:217); the literal traversal does that, the culled one
    // resolves it by the lower triangle index so that the result does not
    // depend on the order (the GPU kernels use the same rule).
    bool better = tmp.t < closest || (!literal && hit && tmp.t == closest && ti < best_tri);
    if (better) {
      if (hit) second = std::min(second, closest);
      hit = true;
      closest = tmp.t;
      rec = tmp;
      best_tri = ti;
      if (uo) *uo = u;
      if (vo) *vo = v;
    } else {
      second = std::min(second, tmp.t);
    }
  };
  if (literal) {
    std::vector<int32_t> stack((size_t)stack_size + 2);
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0 && sp < stack_size) {
      sp--;
      int32_t node = stack[sp];
      if (node == -1) continue;
      const rt_bvh_node &nd = sc.nodes[node];
      nvis++;
      T tn, tf;
      slab(nd, ro, rd, tn, tf);
      if (tn > tf) continue;
      if (nd.object != -1) test_tri(nd.object);
      stack[sp++] = nd.left;
      stack[sp++] = nd.right;
    }
    if (sp >= stack_size) flags |= FLAG_TRUNCATED;
  } else {
    struct E {
      int32_t node;
      T tn;
    };
    E stack[256];
    int sp = 0;
    auto cull = [&](T tn, T tf) {
      T lim = (T)((double)closest * (1.0 + slack));
      return tn > tf || tf < tmin || tn > lim;
    };
    T tn, tf;
    nvis++;
    slab(sc.nodes[0], ro, rd, tn, tf);
    if (!cull(tn, tf)) stack[sp++] = E{0, tn};
    while (sp > 0) {
      E e = stack[--sp];
      if (e.tn > (T)((double)closest * (1.0 + slack))) continue;
      const rt_bvh_node &nd = sc.nodes[e.node];
      if (nd.left == -1 && nd.right == -1) {
        if (nd.object >= 0) test_tri(nd.object);
        continue;
      }
      E ch[2];
      int nc = 0;
      for (int32_t c : {nd.left, nd.right}) {
        if (c < 0) continue;
        nvis++;
        T a, b;
        slab(sc.nodes[c], ro, rd, a, b);
        if (!cull(a, b)) ch[nc++] = E{c, a};
      }
      if (nc == 2 && ch[1].tn < ch[0].tn) std::swap(ch[0], ch[1]);
      for (int i = nc - 1; i >= 0; i--) {
        if (sp >= 255) {  // cannot happen for trees of depth < 255
          flags |= FLAG_TRUNCATED;
          break;
        }
        stack[sp++] = ch[i];
      }
    }
  }
  if (hit && second <= closest + (T)((double)closest * 1e-6)) flags |= FLAG_TIE;
  if (tri_out) *tri_out = hit ? best_tri : -1;
  if (st) {
    st->nodes = nvis;
    st->tris = ntri;
    st->flags = flags;
  }
  return hit;
}

// ---------------------------------------------------------------- shading
struct Effective {
  uint32_t nlights;
  uint32_t nspheres;
  int sphere_mode;  // 0 none, 1 closest (default), 2 override
};

template <typename T> struct Shader {
  const Scene &sc;
  const Effective &ef;
  uint32_t flags;
  Rng rng;

  T rnd() { return rng.next<T>(); }

  // Onb + onbLocal (definitions.glsl:42-53), random_cosine_direction (random.glsl:42-52).
  V3<T> sample_lambertian(V3<T> normal) {
    V3<T> w = normalize(normal);
    V3<T> a = (std::fabs(w.x) > (T)0.9f) ? mk<T>(0, 1, 0) : mk<T>(1, 0, 0);
    V3<T> v = normalize(cross(w, a));
    V3<T> u = cross(w, v);
    T r1 = rnd();
    T r2 = rnd();
    T z = gsqrt((T)1 - r2);
    T phi = (T)2 * Consts<T>::pi() * r1;
    T sr2 = gsqrt(r2);
    T x = tcos(phi) * sr2;
    T y = tsin(phi) * sr2;
    V3<T> local = add(add(mul(x, u), mul(y, v)), mul(z, w));
    return normalize(local);
  }

  // random_in_unit_sphere (random.glsl:29-32) with random(min,max) (24-27).
  V3<T> random_in_unit_sphere() {
    T lo = (T)-0.3f, hi = (T)0.3f;
    T x = lo + (hi - lo) * rnd();
    T y = lo + (hi - lo) * rnd();
    T z = lo + (hi - lo) * rnd();
    return normalize(mk(x, y, z));
  }

  // sampleGlass (comp:106-116); ior 0 means the reference's 1.5.
  V3<T> sample_glass(V3<T> I, const Hit<T> &rec, T ir) {
    T ratio = (T)(1 - rec.back) * (T)1 / ir + (T)rec.back * ir;
    V3<T> i = normalize(I);
    T cos_t = gmin(dot(neg(i), rec.normal), (T)1);
    T sin_t = gsqrt((T)1 - cos_t * cos_t);
    T t = std::floor(gclamp(ratio * sin_t, (T)0, (T)1));
    V3<T> rf = reflect(i, rec.normal);
    V3<T> rr = refract(i, rec.normal, ratio);
    return add(mul(t, rf), mul((T)1 - t, rr));
  }

  // sampleLight + randomOnATriangle (comp:67-89). Returns false when the
  // light cosine is below 0.001 (the caller keeps the material sample).
  bool sample_light(V3<T> p, V3<T> &dir) {
    T len = (T)ef.nlights;
    T r = rnd();
    int idx = (int)std::floor(len * r);
    if (idx >= (int)ef.nlights) idx = (int)ef.nlights - 1;  // random() can return 1.0
    const rt_triangle &tr = sc.tris[sc.lights[idx].triangle_index];
    T s = rnd();
    T t = rnd();
    V3<T> v0 = ld3<T>(tr.v0), v1 = ld3<T>(tr.v1), v2 = ld3<T>(tr.v2);
    V3<T> v01 = add(neg(v0), v1);
    V3<T> v02 = add(neg(v0), v2);
    V3<T> on = add(add(v0, mul(s, v01)), mul(t, v02));
    V3<T> to = normalize(sub(on, p));
    T cosine = std::fabs(to.y);
    dir = to;
    return !(std::fabs(cosine) < (T)0.001f);
  }

  // scatter (comp:118-155). Returns true for an emitter.
  bool scatter(V3<T> dir_in, const Hit<T> &rec, V3<T> &albedo, V3<T> &out_dir) {
    const rt_material &m = sc.mats[rec.mat];
    albedo = ld3<T>(m.albedo);
    V3<T> ms = mk<T>(0, 0, 0);
    if (flags & RT_SHADE_SIMPLE) {
      // ray-trace-compute-simple.comp:62-68: normalize(random_in_hemisphere(normal)).
      V3<T> in = random_in_unit_sphere();
      V3<T> h = (dot(in, rec.normal) > (T)0) ? in : neg(in);
      out_dir = normalize(h);
      return m.type == RT_MATERIAL_LIGHT;
    }
    if (m.type == RT_MATERIAL_LAMBERTIAN) {
      ms = sample_lambertian(rec.normal);
    } else if (m.type == RT_MATERIAL_METAL) {
      ms = reflect(dir_in, rec.normal);
      if (m.fuzz > 0.0f) {
        V3<T> f = random_in_unit_sphere();
        ms = add(ms, mul((T)m.fuzz, f));
      }
    } else if (m.type == RT_MATERIAL_GLASS) {
      T ir = m.ior > 0.0f ? (T)m.ior : (T)1.5f;
      ms = sample_glass(dir_in, rec, ir);
      albedo = mk<T>(1, 1, 1);
    }
    V3<T> fin = ms;
    T coin = rnd();
    if (coin < (T)0.5f && m.type == RT_MATERIAL_LAMBERTIAN && ef.nlights > 0) {
      V3<T> ld;
      if (sample_light(rec.p, ld)) fin = ld;
    }
    out_dir = fin;
    return m.type == RT_MATERIAL_LIGHT;
  }

  bool closest(V3<T> ro, V3<T> rd, Hit<T> &rec, uint64_t &segments) {
    segments++;
    const T tmin = (T)0.001f, tmax = (T)10000.0f;
    bool literal = (flags & RT_COMPAT_STACK16) != 0;
    bool hit = trace_closest<T>(sc, ro, rd, tmin, tmax, literal, 16, 0.0, rec, nullptr, nullptr, nullptr,
                                nullptr);
    if (ef.sphere_mode != 0) {
      T closest = (ef.sphere_mode == 2) ? tmax : (hit ? rec.t : tmax);
      for (uint32_t j = 0; j < ef.nspheres; j++) {
        Hit<T> tmp;
        if (hit_sphere(sc.spheres[j], ro, rd, tmin, closest, tmp)) {
          hit = true;
          closest = tmp.t;
          rec = tmp;
        }
      }
    }
    return hit;
  }

  // ray_color (comp:314-338).
  V3<T> ray_color(V3<T> ro, V3<T> rd, uint32_t max_bounces, uint64_t &segments) {
    V3<T> color = mk<T>(1, 1, 1);
    V3<T> o = ro, d = normalize(rd);
    for (uint32_t i = 0; i < max_bounces; i++) {
      Hit<T> rec;
      if (closest(o, d, rec, segments)) {
        V3<T> albedo, nd;
        bool emits = scatter(d, rec, albedo, nd);
        color = mulv(color, albedo);
        o = rec.p;
        d = nd;
        if (emits) break;
      } else {
        color = mul((T)0, color);
        break;
      }
    }
    return color;
  }
};

inline float unorm8(float x) {
  float c = gclamp(x, 0.0f, 1.0f);
  return std::floor(c * 255.0f + 0.5f) / 255.0f;
}

template <typename T>
int render(const Scene &sc, const rt_camera &cam, const rt_render_params &pr, float *accum, double *accum64,
           uint64_t *segments_out, int threads) {
  Effective ef;
  bool len1 = (pr.flags & RT_COMPAT_LEN1) != 0;
  ef.nlights = len1 ? std::min<uint32_t>(sc.nlights, 1u) : sc.nlights;
  ef.nspheres = len1 ? std::min<uint32_t>(sc.nspheres, 1u) : sc.nspheres;
  ef.sphere_mode = (pr.flags & RT_COMPAT_NO_SPHERES) ? 0 : ((pr.flags & RT_COMPAT_SPHERE_OVERRIDE) ? 2 : 1);
  const uint32_t W = pr.width, H = pr.height;
  const int64_t npix = (int64_t)W * H;
  uint64_t total = 0;
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
  for (int64_t pix = 0; pix < npix; pix++) {
    uint32_t x = (uint32_t)(pix % W), y = (uint32_t)(pix / W);
    Shader<T> sh{sc, ef, pr.flags, Rng{0}};
    V3<T> org = ld3<T>(cam.origin), llc = ld3<T>(cam.lower_left);
    V3<T> hor = ld3<T>(cam.horizontal), ver = ld3<T>(cam.vertical);
    // uv = gid / size (comp:371): no pixel-centre offset.
    T u = (T)((float)x / (float)W), v = (T)((float)y / (float)H);
    V3<T> dir = sub(add(add(llc, mul(u, hor)), mul(v, ver)), org);
    uint64_t seg = 0;
    for (uint32_t k = 0; k < pr.spp; k++) {
      uint32_t s = pr.sample_index + k;
      sh.rng.s = (600u * x + y) * (s + 1u);
      V3<T> c = sh.ray_color(org, dir, pr.max_bounces, seg);
      // Running mean (comp:375-377).
      float sf = (float)s;
      float keep = gmin(sf, 1.0f);
      if (accum64) {
        double *a = accum64 + 4 * pix;
        double cc[4] = {(double)c.x, (double)c.y, (double)c.z, 1.0};
        for (int ch = 0; ch < 4; ch++) a[ch] = (cc[ch] + a[ch] * keep * sf) / ((double)sf + 1.0);
      } else {
        float *a = accum + 4 * pix;
        float cc[4] = {(float)c.x, (float)c.y, (float)c.z, 1.0f};
        for (int ch = 0; ch < 4; ch++) {
          float prev = a[ch] * keep;
          float w = (cc[ch] + prev * sf) / (sf + 1.0f);
          a[ch] = (pr.flags & RT_COMPAT_UNORM8) ? unorm8(w) : w;
        }
      }
    }
    total += seg;
  }
  if (segments_out) *segments_out = total;
  return 0;
}

inline float tri_key(const rt_triangle &t, int axis) {
  float a = t.v0[axis], b = t.v1[axis], c = t.v2[axis];
  return gmin(gmin(a, b), c) - 0.0001f;
}

}  // namespace

extern "C" {

// glibc rand() after srand(seed) — the generator Bvh.h's randomAxis uses.
void oracle_glibc_rand(uint32_t seed, uint32_t count, int32_t *out) {
  srand(seed);
  for (uint32_t i = 0; i < count; i++) out[i] = rand();
}

// Restatement of Bvh::createBvh (Bvh.h:141-209): DFS with an explicit stack
// (right child popped first), one rand() % 3 per popped node, std::sort by
// the per-triangle box minimum on that axis (Bvh.h:94-98, 116-122), median
// split, one triangle per leaf, output in creation-index order. Node boxes are
// the union of the node's triangle boxes (Bvh.h:100-114).
int oracle_build_bvh(const rt_triangle *tris, uint32_t n, rt_bvh_node *out, uint32_t seed, int *depth_out) {
  if (n == 0) return -1;
  srand(seed);
  struct Item {
    float key;
    uint32_t idx;
  };
  struct Pending {
    int32_t index;
    uint32_t depth;
    std::vector<uint32_t> objs;
  };
  std::vector<Pending> stack;
  std::vector<uint32_t> all(n);
  for (uint32_t i = 0; i < n; i++) all[i] = i;
  stack.push_back(Pending{0, 1, std::move(all)});
  int32_t counter = 1;
  int maxdepth = 0;
  std::vector<Item> items;
  while (!stack.empty()) {
    Pending cur = std::move(stack.back());
    stack.pop_back();
    maxdepth = std::max<int>(maxdepth, (int)cur.depth);
    rt_bvh_node &nd = out[cur.index];
    std::memset(&nd, 0, sizeof(nd));
    for (int a = 0; a < 3; a++) {
      nd.min[a] = 3.402823466e+38f;
      nd.max[a] = -3.402823466e+38f;
    }
    bool first = true;
    for (uint32_t o : cur.objs) {
      const rt_triangle &t = tris[o];
      for (int a = 0; a < 3; a++) {
        float lo = gmin(gmin(t.v0[a], t.v1[a]), t.v2[a]) - 0.0001f;
        float hi = gmax(gmax(t.v0[a], t.v1[a]), t.v2[a]) + 0.0001f;
        nd.min[a] = first ? lo : gmin(nd.min[a], lo);
        nd.max[a] = first ? hi : gmax(nd.max[a], hi);
      }
      first = false;
    }
    int axis = rand() % 3;
    items.resize(cur.objs.size());
    for (size_t i = 0; i < cur.objs.size(); i++) items[i] = Item{tri_key(tris[cur.objs[i]], axis), cur.objs[i]};
    std::sort(items.begin(), items.end(), [](const Item &a, const Item &b) { return a.key < b.key; });
    if (items.size() <= 1) {
      nd.left = nd.right = -1;
      nd.object = (int32_t)items[0].idx;
      continue;
    }
    size_t mid = items.size() / 2;
    Pending l{counter, cur.depth + 1, {}}, r{counter + 1, cur.depth + 1, {}};
    counter += 2;
    for (size_t i = 0; i < mid; i++) l.objs.push_back(items[i].idx);
    for (size_t i = mid; i < items.size(); i++) r.objs.push_back(items[i].idx);
    nd.left = l.index;
    nd.right = r.index;
    nd.object = -1;
    stack.push_back(std::move(l));
    stack.push_back(std::move(r));
  }
  if (depth_out) *depth_out = maxdepth;
  return 0;
}

// libstdc++'s introsort with an explicit depth limit, for pinning the GPU
// sorter's heap-sort fallback (std::sort itself uses 2*floor(log2 n)).
// Sorts `keys` and permutes `idx` alongside.
void oracle_sort_with_depth(float *keys, uint32_t *idx, uint32_t n, int depth_limit) {
  struct Item {
    float key;
    uint32_t idx;
  };
  std::vector<Item> v(n);
  for (uint32_t i = 0; i < n; i++) v[i] = Item{keys[i], idx[i]};
  auto cmp = [](const Item &a, const Item &b) { return a.key < b.key; };
  if (n > 0) {
    std::__introsort_loop(v.begin(), v.end(), (long)depth_limit, __gnu_cxx::__ops::__iter_comp_iter(cmp));
    std::__final_insertion_sort(v.begin(), v.end(), __gnu_cxx::__ops::__iter_comp_iter(cmp));
  }
  for (uint32_t i = 0; i < n; i++) {
    keys[i] = v[i].key;
    idx[i] = v[i].idx;
  }
}

// RtScene.h:87-96: one light per LightSource triangle, area = |v0 x v1| / 2.
uint32_t oracle_lights_from_materials(const rt_triangle *tris, uint32_t n, const rt_material *mats, uint32_t nm,
                                      rt_light *out) {
  uint32_t k = 0;
  for (uint32_t i = 0; i < n; i++) {
    uint32_t m = tris[i].material_index;
    if (m < nm && mats[m].type == RT_MATERIAL_LIGHT) {
      V3<float> v0 = ld3<float>(tris[i].v0), v1 = ld3<float>(tris[i].v1);
      float area = length(cross(v0, v1)) * 0.5f;
      if (out) out[k] = rt_light{i, area};
      k++;
    }
  }
  return k;
}

// The reference shader's camera (comp:357-372) for a given camPos and size.
void oracle_camera_from_reference(const float cam_pos[3], uint32_t W, uint32_t H, rt_camera *out) {
  float vfov = 30.0f;
  float pi = 3.1415926535897932385f;
  float theta = vfov * pi / 180.0f;
  float h = std::tan(theta / 2.0f);
  float vh = 2.0f * h;
  float vw = (float)W / (float)H * vh;
  float focal = 1.0f;
  float hor[3] = {vw, 0.0f, 0.0f}, ver[3] = {0.0f, -vh, 0.0f};
  float org[3] = {-cam_pos[2], cam_pos[0], cam_pos[1]};
  float foc[3] = {0.0f, 0.0f, focal};
  for (int a = 0; a < 3; a++) {
    out->origin[a] = org[a];
    out->horizontal[a] = hor[a];
    out->vertical[a] = ver[a];
    out->lower_left[a] = org[a] - hor[a] / 2.0f - ver[a] / 2.0f - foc[a];
  }
}

// Closest hit for a batch of rays. mode 0: culled near-first (default
// semantics), 1: the shader-literal traversal with a `stack_size` stack.
// stats (optional) receives 4 words per ray: nodes, triangles, flags, 0.
int oracle_trace(const rt_triangle *tris, uint32_t ntris, const rt_bvh_node *nodes, uint32_t nnodes,
                 const rt_ray *rays, uint32_t nrays, int mode, int stack_size, double slack, rt_hit *hits,
                 uint32_t *stats, int threads) {
  Scene sc{tris, ntris, nullptr, 0, nodes, nnodes, nullptr, 0, nullptr, 0};
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < (int64_t)nrays; i++) {
    const rt_ray &r = rays[i];
    Hit<float> rec;
    float u = 0, v = 0;
    int32_t tri = -1;
    TraceStats st{};
    bool h = trace_closest<float>(sc, ld3<float>(r.o), ld3<float>(r.d), r.tmin, r.tmax, mode == 1, stack_size,
                                  slack, rec, &u, &v, &tri, &st);
    hits[i] = h ? rt_hit{tri, rec.t, u, v} : rt_hit{-1, 0.0f, 0.0f, 0.0f};
    if (stats) std::memcpy(stats + 4 * i, &st, 16);
  }
  return 0;
}

// fp64 error reference: the same traversal and formulas in double.
int oracle_trace_f64(const rt_triangle *tris, uint32_t ntris, const rt_bvh_node *nodes, uint32_t nnodes,
                     const rt_ray *rays, uint32_t nrays, int32_t *tri_out, double *tuv_out, int threads) {
  Scene sc{tris, ntris, nullptr, 0, nodes, nnodes, nullptr, 0, nullptr, 0};
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < (int64_t)nrays; i++) {
    const rt_ray &r = rays[i];
    Hit<double> rec;
    double u = 0, v = 0;
    int32_t tri = -1;
    bool h = trace_closest<double>(sc, ld3<double>(r.o), ld3<double>(r.d), (double)r.tmin, (double)r.tmax, false,
                                   0, 1e-5, rec, &u, &v, &tri, nullptr);
    tri_out[i] = h ? tri : -1;
    tuv_out[3 * i + 0] = h ? rec.t : 0.0;
    tuv_out[3 * i + 1] = h ? u : 0.0;
    tuv_out[3 * i + 2] = h ? v : 0.0;
  }
  return 0;
}

// Progressive render into an RGBA32F accumulation image (W*H*4 floats,
// updated in place). segments_out receives the number of ray segments traced
// (camera rays plus every secondary ray).
int oracle_render(const rt_triangle *tris, uint32_t ntris, const rt_material *mats, uint32_t nmats,
                  const rt_bvh_node *nodes, uint32_t nnodes, const rt_light *lights, uint32_t nlights,
                  const rt_sphere *spheres, uint32_t nspheres, const rt_camera *cam, const rt_render_params *pr,
                  float *accum, uint64_t *segments_out, int threads) {
  Scene sc{tris, ntris, mats, nmats, nodes, nnodes, lights, nlights, spheres, nspheres};
  return render<float>(sc, *cam, *pr, accum, nullptr, segments_out, threads);
}

// The same render with every shading and intersection operation in double
// (accumulation in double as well).
int oracle_render_f64(const rt_triangle *tris, uint32_t ntris, const rt_material *mats, uint32_t nmats,
                      const rt_bvh_node *nodes, uint32_t nnodes, const rt_light *lights, uint32_t nlights,
                      const rt_sphere *spheres, uint32_t nspheres, const rt_camera *cam,
                      const rt_render_params *pr, double *accum, uint64_t *segments_out, int threads) {
  Scene sc{tris, ntris, mats, nmats, nodes, nnodes, lights, nlights, spheres, nspheres};
  return render<double>(sc, *cam, *pr, nullptr, accum, segments_out, threads);
}

int oracle_max_threads(void) { return omp_get_max_threads(); }

// The shading hit record of each ray (the `closest` step of ray_color under
// `flags`: BVH traversal, then the sphere pass of the flags' mode), in fp32.
// out gets 10 floats per ray: hit (0/1), t, p.xyz, normal.xyz, material
// index (uint bits), back-face flag (int bits). Rays are rt_ray records
// (only origin and direction are used; t runs over (0.001, 10000) as in the
// shader).
void oracle_hit_records(const rt_triangle *tris, uint32_t ntris, const rt_bvh_node *nodes, uint32_t nnodes,
                        const rt_sphere *spheres, uint32_t nspheres, const rt_ray *rays, uint32_t n, uint32_t flags,
                        float *out) {
  Scene sc{tris, ntris, nullptr, 0, nodes, nnodes, nullptr, 0, spheres, nspheres};
  Effective ef;
  bool len1 = (flags & RT_COMPAT_LEN1) != 0;
  ef.nlights = 0;
  ef.nspheres = len1 ? std::min<uint32_t>(nspheres, 1u) : nspheres;
  ef.sphere_mode = (flags & RT_COMPAT_NO_SPHERES) ? 0 : ((flags & RT_COMPAT_SPHERE_OVERRIDE) ? 2 : 1);
#pragma omp parallel for schedule(dynamic, 256)
  for (long i = 0; i < (long)n; i++) {
    Shader<float> sh{sc, ef, flags, Rng{0}};
    Hit<float> rec{};
    uint64_t seg = 0;
    V3<float> ro = ld3<float>(rays[i].o), rd = ld3<float>(rays[i].d);
    bool hit = sh.closest(ro, rd, rec, seg);
    float *o = out + 10 * i;
    o[0] = hit ? 1.0f : 0.0f;
    o[1] = rec.t;
    o[2] = rec.p.x;
    o[3] = rec.p.y;
    o[4] = rec.p.z;
    o[5] = rec.normal.x;
    o[6] = rec.normal.y;
    o[7] = rec.normal.z;
    std::memcpy(o + 8, &rec.mat, 4);
    std::memcpy(o + 9, &rec.back, 4);
  }
}

// smartDeNoise (post-process-shader.frag:26-68) over an RGBA32F image, as a
// texel-space restatement: taps at (px + x, py + y) fetched bilinearly with
// REPEAT wrap (the reference's sampler, src/memory/Image.cpp:353-357), every
// step one fp32 operation in shader order; out = mix * filtered + (1 - mix)
// * in. Built with -ffp-contract=off, so no step is fused.
void oracle_denoise(const float *in, uint32_t W, uint32_t H, float sigma, float ksigma, float threshold, float mix,
                    float *out) {
  const float kInvPi = 0.31830988618379067154f, kInvSqrt2Pi = 0.39894228040143267794f;
  const float radius = std::round(ksigma * sigma), rad_q = radius * radius;
  const float inv_sigma_q2 = 0.5f / (sigma * sigma), inv_sigma_q2pi = kInvPi * inv_sigma_q2;
  const float inv_thr_q2 = 0.5f / (threshold * threshold), inv_thr_sqrt2pi = kInvSqrt2Pi / threshold;
  auto tex = [&](long x, long y, int c) {
    x %= (long)W;
    y %= (long)H;
    if (x < 0) x += W;
    if (y < 0) y += H;
    return in[4 * ((size_t)y * W + x) + c];
  };
  auto lerp = [](float a, float b, float w) { return (1.0f - w) * a + w * b; };
#pragma omp parallel for schedule(dynamic, 4)
  for (long py = 0; py < (long)H; py++) {
    for (long px = 0; px < (long)W; px++) {
      float c[4], a[4] = {0, 0, 0, 0}, z = 0.0f;
      for (int k = 0; k < 4; k++) c[k] = in[4 * ((size_t)py * W + px) + k];
      for (float x = -radius; x <= radius; x = x + 1.0f) {
        const float pt = std::sqrt(rad_q - x * x);
        for (float y = -pt; y <= pt; y = y + 1.0f) {
          const float dd = x * x + y * y;
          const float blur = std::exp(-dd * inv_sigma_q2) * inv_sigma_q2pi;
          const float s = (float)px + x, t = (float)py + y;
          const float fs = std::floor(s), ft = std::floor(t);
          const float al = s - fs, be = t - ft;
          const long i0 = (long)fs, j0 = (long)ft;
          float w[4];
          for (int k = 0; k < 4; k++)
            w[k] = lerp(lerp(tex(i0, j0, k), tex(i0 + 1, j0, k), al), lerp(tex(i0, j0 + 1, k), tex(i0 + 1, j0 + 1, k), al),
                        be);
          const float d0 = w[0] - c[0], d1 = w[1] - c[1], d2 = w[2] - c[2], d3 = w[3] - c[3];
          const float dc2 = d0 * d0 + d1 * d1 + d2 * d2 + d3 * d3;
          const float delta = std::exp(-dc2 * inv_thr_q2) * inv_thr_sqrt2pi * blur;
          z = z + delta;
          for (int k = 0; k < 4; k++) a[k] = a[k] + delta * w[k];
        }
      }
      for (int k = 0; k < 4; k++) out[4 * ((size_t)py * W + px) + k] = lerp(c[k], a[k] / z, mix);
    }
  }
}

// ---------------------------------------------------------------- 8-wide model
// A host model of the GPU's 8-wide closest-hit traversal, used to check its
// central claim on many scenes without a GPU: pruning by quantized 8-bit
// child boxes, with the kernel's fp32 plane arithmetic, never drops the
// closest hit. oracle_wide_fold folds the reference node array into nodes
// of up to eight children with the GPU builder's rule (replace the inner
// child of largest half area, dx*dy + dy*dz + dz*dx, by its two children,
// left in place and right appended, first of equal areas), places the
// children in slots by octant (oracle_octant_slots) and numbers nodes
// breadth first, the inner children of a node in slot order; inner refs are
// node numbers, leaf refs ~triangle, empty slots INT_MIN. The caller
// quantizes each node with the library's host quantizer (96-byte words) and
// oracle_trace_wide traverses those words: planes entered at fmaf(q, ix *
// 2^e, (o - ray.o) * ix), the entered inner child of smallest entry distance
// (compared with the slot in the distance's low three bits) visited next and
// the others later in increasing order of slot ^ (the ray's direction sign
// bits), triangles tested when reached
// with the acceptance rule of the culled traversal (exactly equal t: the
// lower triangle index wins).

// Slot of each of `cnt` children (boxes lo.xyz, hi.xyz): slot bits (x, y,
// z) name the node corner on the positive side of each set axis; each child
// goes to the free slot of lowest cost -sum_k sign_k(slot) * offset_k, the
// offsets being twice the distance of the child's box centre from the
// node's (sums and differences of coordinates only), greedily, lowest cost
// first, ties to the lower child and then the lower slot.
static void oracle_octant_slots(const float (*box)[6], int cnt, int *slot_of) {
  float twice_centre[3];
  for (int k = 0; k < 3; k++) {
    float lo = box[0][k], hi = box[0][3 + k];
    for (int i = 1; i < cnt; i++) {
      lo = std::fmin(lo, box[i][k]);
      hi = std::fmax(hi, box[i][3 + k]);
    }
    twice_centre[k] = lo + hi;
  }
  bool kid_done[8] = {}, slot_taken[8] = {};
  for (int placed = 0; placed < cnt; placed++) {
    int bi = -1, bs = -1;
    float best = 0.0f;
    for (int i = 0; i < cnt; i++) {
      if (kid_done[i]) continue;
      float off[3];
      for (int k = 0; k < 3; k++) off[k] = (box[i][k] + box[i][3 + k]) - twice_centre[k];
      for (int sl = 0; sl < 8; sl++) {
        if (slot_taken[sl]) continue;
        float cost = 0.0f;
        for (int k = 0; k < 3; k++) cost = (sl >> k & 1) ? cost - off[k] : cost + off[k];
        if (bi < 0 || cost < best) {
          best = cost;
          bi = i;
          bs = sl;
        }
      }
    }
    kid_done[bi] = true;
    slot_taken[bs] = true;
    slot_of[bi] = bs;
  }
}

int oracle_octant_slot_assignment(const float *boxes, uint32_t cnt, int32_t *slot_of) {
  if (!boxes || !slot_of || cnt < 1 || cnt > 8) return 1;
  float b[8][6];
  for (uint32_t i = 0; i < cnt; i++)
    for (int k = 0; k < 6; k++) b[i][k] = boxes[6 * i + k];
  int so[8];
  oracle_octant_slots(b, (int)cnt, so);
  for (uint32_t i = 0; i < cnt; i++) slot_of[i] = so[i];
  return 0;
}

// mode 1 (the GPU's default "bvh8.collapse"): the inner nodes that become
// 8-wide nodes are chosen by the surface area heuristic with a fixed leaf
// cost, least summed node area. D(n, j), j = 1..8, is the least summed area
// covering n's subtree with at most j slots: n as one slot (n becomes a
// node: area(n) + the best split of 8 slots between its children) or its
// children splitting the j slots (left share l = 1..j-1, the lowest of
// equal sums); a leaf costs 0; n stays one slot when that is not dearer.
// The area of an inner node is that of its children's box union.
int oracle_wide_fold_mode(const rt_bvh_node *nodes, uint32_t nnodes, uint32_t cap, int mode, float *boxes,
                          int32_t *refs, uint32_t *fmask_out, uint32_t *n8_out, uint32_t *levels_out);

int oracle_wide_fold(const rt_bvh_node *nodes, uint32_t nnodes, uint32_t cap, float *boxes, int32_t *refs,
                     uint32_t *fmask_out, uint32_t *n8_out, uint32_t *levels_out) {
  return oracle_wide_fold_mode(nodes, nnodes, cap, 0, boxes, refs, fmask_out, n8_out, levels_out);
}

int oracle_wide_fold_mode(const rt_bvh_node *nodes, uint32_t nnodes, uint32_t cap, int mode, float *boxes,
                          int32_t *refs, uint32_t *fmask_out, uint32_t *n8_out, uint32_t *levels_out) {
  if (!nodes || nnodes == 0 || !boxes || !refs || !fmask_out || !n8_out || mode < 0 || mode > 1) return 1;
  struct Slot {
    float b[6];
    int32_t node;  // reference node index
  };
  auto slot_of = [&](int32_t i) {
    Slot s;
    for (int k = 0; k < 3; k++) {
      s.b[k] = nodes[i].min[k];
      s.b[3 + k] = nodes[i].max[k];
    }
    s.node = i;
    return s;
  };
  auto inner = [&](int32_t i) { return nodes[i].left != -1; };
  auto area = [](const Slot &s) {
    float dx = s.b[3] - s.b[0], dy = s.b[4] - s.b[1], dz = s.b[5] - s.b[2];
    return dx * dy + dy * dz + dz * dx;
  };
  // Each built node: its 8 slots (node -1 = empty).
  std::vector<std::array<Slot, 8>> built;
  std::vector<int32_t> frontier, next;
  uint32_t levels = 0;
  auto place = [&](const std::vector<Slot> &S) {
    std::array<Slot, 8> out;
    for (auto &o : out) o.node = -1;
    float b[8][6];
    for (size_t i = 0; i < S.size(); i++)
      for (int k = 0; k < 6; k++) b[i][k] = S[i].b[k];
    int so[8];
    oracle_octant_slots(b, (int)S.size(), so);
    for (size_t i = 0; i < S.size(); i++) out[so[i]] = S[i];
    return out;
  };
  // SAH costs, children before parents (Bvh.h numbers a child after its parent).
  std::vector<std::array<float, 9>> D;
  std::vector<std::array<int8_t, 9>> pick_j;  // j = 2..8: left share, 0 = one slot
  std::vector<int8_t> pick8;                  // split of 8 slots when a node
  if (mode == 1) {
    D.assign(nnodes, {});
    pick_j.assign(nnodes, {});
    pick8.assign(nnodes, 1);
    for (int64_t n = (int64_t)nnodes - 1; n >= 0; n--) {
      if (!inner((int32_t)n)) continue;
      const int32_t c[2] = {nodes[n].left, nodes[n].right};
      float dc[2][9];
      for (int i = 0; i < 2; i++)
        for (int j = 1; j <= 8; j++) dc[i][j] = inner(c[i]) ? D[c[i]][j] : 0.0f;
      Slot u = slot_of(c[0]);
      const Slot v = slot_of(c[1]);
      for (int k = 0; k < 3; k++) {
        u.b[k] = std::fmin(u.b[k], v.b[k]);
        u.b[3 + k] = std::fmax(u.b[3 + k], v.b[3 + k]);
      }
      auto split = [&](int j, int &kbest) {
        float best = INFINITY;
        kbest = 1;
        for (int l = 1; l < j; l++) {
          const float x = dc[0][l] + dc[1][j - l];
          if (x < best) {
            best = x;
            kbest = l;
          }
        }
        return best;
      };
      int k8;
      const float as_node = area(u) + split(8, k8);
      pick8[n] = (int8_t)k8;
      D[n][1] = as_node;
      for (int j = 2; j <= 8; j++) {
        int kj;
        const float x = split(j, kj);
        const bool keep = as_node <= x;
        D[n][j] = keep ? as_node : x;
        pick_j[n][j] = keep ? 0 : (int8_t)kj;
      }
    }
  }
  auto sah_children = [&](int32_t f) {
    std::vector<Slot> S;
    std::vector<std::pair<int32_t, int>> st = {{nodes[f].right, 8 - pick8[f]}, {nodes[f].left, pick8[f]}};
    while (!st.empty()) {
      const auto [m, j] = st.back();
      st.pop_back();
      const int kj = (inner(m) && j >= 2) ? pick_j[m][j] : 0;
      if (kj == 0) {
        S.push_back(slot_of(m));
        continue;
      }
      st.push_back({nodes[m].right, j - kj});
      st.push_back({nodes[m].left, kj});
    }
    return S;
  };
  if (!inner(0)) {
    std::array<Slot, 8> one;
    for (auto &o : one) o.node = -1;
    one[0] = slot_of(0);
    built.push_back(one);
    levels = 1;
  } else {
    frontier.push_back(0);
    while (!frontier.empty()) {
      next.clear();
      for (int32_t f : frontier) {
        std::vector<Slot> S = {slot_of(nodes[f].left), slot_of(nodes[f].right)};
        if (mode == 1) S = sah_children(f);
        while (mode == 0 && S.size() < 8) {
          int pick = -1;
          float best = -1.0f;
          for (size_t i = 0; i < S.size(); i++) {
            if (!inner(S[i].node)) continue;
            float a = area(S[i]);
            if (a > best) {
              best = a;
              pick = (int)i;
            }
          }
          if (pick < 0) break;
          int32_t p = S[pick].node;
          S[pick] = slot_of(nodes[p].left);
          S.push_back(slot_of(nodes[p].right));
        }
        built.push_back(place(S));
        for (const Slot &c : built.back())
          if (c.node >= 0 && inner(c.node)) next.push_back(c.node);
      }
      frontier.swap(next);
      levels++;
    }
  }
  if (built.size() > cap) return 2;
  // Node numbers: breadth first, the inner children of node i in slot order.
  uint32_t counter = 1;
  for (size_t i = 0; i < built.size(); i++) {
    uint32_t mask = 0;
    for (int s = 0; s < 8; s++) {
      float *b = boxes + 6 * (8 * i + s);
      const Slot &sl = built[i][s];
      if (sl.node < 0) {
        for (int k = 0; k < 6; k++) b[k] = 0.0f;
        refs[8 * i + s] = INT32_MIN;
        continue;
      }
      mask |= 1u << s;
      for (int k = 0; k < 6; k++) b[k] = sl.b[k];
      refs[8 * i + s] = inner(sl.node) ? (int32_t)(counter++) : ~nodes[sl.node].object;
    }
    fmask_out[i] = mask;
  }
  *n8_out = (uint32_t)built.size();
  if (levels_out) *levels_out = levels;
  return 0;
}

static inline float safe_rcp_model(float x) {
  const float tiny = 1e-30f;
  return 1.0f / (std::fabs(x) > tiny ? x : std::copysign(tiny, x));
}

// stats (optional): per ray, nodes visited and triangles tested.
int oracle_trace_wide(const rt_triangle *tris, uint32_t ntris, const uint32_t *qwords, uint32_t n8, int32_t root8,
                      const float *root_box, const rt_ray *rays, uint32_t nrays, rt_hit *hits, uint32_t *stats,
                      int threads) {
  if (!tris || !qwords || !root_box || !rays || !hits || n8 == 0) return 1;
  if (threads > 0) omp_set_num_threads(threads);
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(| : bad)
  for (int64_t i = 0; i < (int64_t)nrays; i++) {
    const rt_ray &r = rays[i];
    const float ix = safe_rcp_model(r.d[0]), iy = safe_rcp_model(r.d[1]), iz = safe_rcp_model(r.d[2]);
    const float inv[3] = {ix, iy, iz};
    const float oi[3] = {r.o[0] * ix, r.o[1] * iy, r.o[2] * iz};
    const uint32_t oct = (ix < 0.0f ? 1u : 0u) | (iy < 0.0f ? 2u : 0u) | (iz < 0.0f ? 4u : 0u);
    float closest = r.tmax, bu = 0, bv = 0;
    int32_t best = -1;
    // Root box: the kernels' slab test, fmaf(lo, 1/d, -o/d).
    float tn = r.tmin, tf = closest;
    for (int k = 0; k < 3; k++) {
      const float a = std::fmaf(root_box[k], inv[k], -oi[k]), b = std::fmaf(root_box[3 + k], inv[k], -oi[k]);
      tn = std::fmax(tn, std::fmin(a, b));
      tf = std::fmin(tf, std::fmax(a, b));
    }
    // Groups: (node, rank bits of its entered inner children not yet visited).
    std::vector<std::pair<uint32_t, uint32_t>> groups;
    int32_t node = tn <= tf ? root8 : -1;
    uint32_t steps = 0, ntests = 0;
    for (;;) {
      if (node < 0) {
        while (!groups.empty() && groups.back().second == 0) groups.pop_back();
        if (groups.empty()) break;
        auto &g = groups.back();
        const uint32_t rk = (uint32_t)__builtin_ctz(g.second);
        g.second &= g.second - 1u;
        node = (int32_t)qwords[24ull * g.first + 16 + (rk ^ oct)];
      }
      const uint32_t idx = (uint32_t)node;
      if (idx >= n8 || ++steps > n8 + 16) {
        bad = 1;
        break;
      }
      const uint32_t *w = qwords + 24ull * idx;
      const uint32_t fmask = w[3] >> 24;
      float org[3];
      std::memcpy(org, w, 12);
      float sc[3], ax[3];
      for (int k = 0; k < 3; k++) {
        const int e = (int)(int8_t)((w[3] >> (8 * k)) & 0xffu);
        float p2;
        const uint32_t pb = (uint32_t)(e + 127) << 23;
        std::memcpy(&p2, &pb, 4);
        sc[k] = inv[k] * p2;
        ax[k] = (org[k] - r.o[k]) * inv[k];
      }
      // The nearest entered inner child: the minimum of keys (entry distance
      // with its low three bits replaced by the slot), the lowest such slot
      // when no key is finite.
      uint32_t hin = 0;
      float kbest = INFINITY;
      for (int s = 0; s < 8; s++) {
        if (!((fmask >> s) & 1u)) continue;
        const int32_t ref = (int32_t)w[16 + s];
        float t[6];
        for (int k = 0; k < 3; k++) {
          const float ql = (float)((w[4 + 2 * k + (s >> 2)] >> (8 * (s & 3))) & 0xffu);
          const float qh = (float)((w[10 + 2 * k + (s >> 2)] >> (8 * (s & 3))) & 0xffu);
          t[k] = std::fmaf(ql, sc[k], ax[k]);
          t[3 + k] = std::fmaf(qh, sc[k], ax[k]);
        }
        const float n0 = std::fmax(std::fmax(std::fmin(t[0], t[3]), std::fmin(t[1], t[4])),
                                   std::fmax(std::fmin(t[2], t[5]), r.tmin));
        const float f0 = std::fmin(std::fmin(std::fmax(t[0], t[3]), std::fmax(t[1], t[4])),
                                   std::fmin(std::fmax(t[2], t[5]), closest));
        if (!(n0 <= f0)) continue;
        if (ref >= 0) {
          hin |= 1u << s;
          uint32_t kb;
          std::memcpy(&kb, &n0, 4);
          kb = (kb & ~7u) | (uint32_t)s;
          float key;
          std::memcpy(&key, &kb, 4);
          kbest = std::fmin(kbest, key);
          continue;
        }
        const int32_t tri = ~ref;
        if (tri < 0 || (uint32_t)tri >= ntris) {
          bad = 1;
          continue;
        }
        float t0, u, v;
        V3<float> nrm;
        ntests++;
        if (!tri_intersect<float>(tris[tri], ld3<float>(r.o), ld3<float>(r.d), t0, u, v, nrm)) continue;
        if (!(t0 > r.tmin && t0 < r.tmax)) continue;
        if (t0 < closest || (best >= 0 && t0 == closest && tri < best)) {
          closest = t0;
          best = tri;
          bu = u;
          bv = v;
        }
      }
      node = -1;
      if (hin) {
        uint32_t nearest = (uint32_t)__builtin_ctz(hin);
        if (kbest < INFINITY) {
          uint32_t kb;
          std::memcpy(&kb, &kbest, 4);
          nearest = kb & 7u;
        }
        uint32_t ibits = 0;
        for (int s = 0; s < 8; s++)
          if ((hin >> s) & 1u) ibits |= 1u << ((uint32_t)s ^ oct);
        // The nearest entered child next, the others later in rank order.
        node = (int32_t)w[16 + nearest];
        const uint32_t rest = ibits & ~(1u << (nearest ^ oct));
        if (rest) groups.push_back({idx, rest});
      }
    }
    hits[i] = best >= 0 ? rt_hit{best, closest, bu, bv} : rt_hit{-1, 0.0f, 0.0f, 0.0f};
    if (stats) {
      stats[2 * i] = steps;
      stats[2 * i + 1] = ntests;
    }
  }
  return bad ? 3 : 0;
}
}
