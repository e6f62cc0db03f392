// Test infrastructure (oracle) — NOT part of the product.
//
// Runs the reference's own compute shader (ray-trace-compute.comp, or with
// REF_SHADER_SIMPLE ray-trace-compute-simple.comp; rewritten into C++ by
// glsl2cpp.py and included here as SHADER_GEN) on the host the way the
// reference application drives it (src/main.cpp:166-261):
//   per frame: the UBO gets currentSample, every pixel runs main() with its
//   gl_GlobalInvocationID (rngState re-initialised per invocation, as GLSL
//   evaluates global initialisers per invocation), the shader writes the
//   rgba8 target image, then the target is copied into the rgba8
//   accumulation image that the next frame reads.
// Buffers are bound from the product's std430 records (rt_types.h); the
// bound lengths of the light and sphere arrays are parameters because the
// reference binds them with a one-element range (src/memory/Buffer.h:37,85).
#include <omp.h>

#include <cstring>

#include "glsl.h"
#include SHADER_GEN
#include "../include/rtgb/rt_types.h"

thread_local uvec3 gl_GlobalInvocationID;
UniformBufferObject ubo;
image2D targetTexture, accumulationTex;
GlslArray<triangle> triangles;
GlslArray<material> materials;
GlslArray<bvhNode> bvh;
GlslArray<light> lights;
GlslArray<sphere> spheres;

static vec3 v3(const float *p) { return vec3(p[0], p[1], p[2]); }

static std::vector<triangle> g_T;
static std::vector<bvhNode> g_B;

// Binds the triangle and node buffers only (closest-hit casting).
static void bind_geometry(const rt_triangle *tris, uint32_t nt, const rt_bvh_node *nodes, uint32_t nn) {
  g_T.resize(nt);
  for (uint32_t i = 0; i < nt; i++)
    g_T[i] = triangle{v3(tris[i].v0), v3(tris[i].v1), v3(tris[i].v2), tris[i].material_index};
  g_B.resize(nn);
  for (uint32_t i = 0; i < nn; i++)
    g_B[i] = bvhNode{v3(nodes[i].min), v3(nodes[i].max), nodes[i].left, nodes[i].right, nodes[i].object};
  triangles = GlslArray<triangle>{g_T.data(), (int)nt};
  bvh = GlslArray<bvhNode>{g_B.data(), (int)nn};
}

// The shader's own closest-hit traversal (hit_bvh: 16-entry stack, every
// hit box pushes both children, t in (0.001, 10000)) for each ray; t_out
// receives the hit distance or -1. Used as the reference's CPU timing.
extern "C" int ref_shader_trace(const rt_triangle *tris, uint32_t nt, const rt_bvh_node *nodes, uint32_t nn,
                                const rt_ray *rays, uint32_t n, float *t_out, int threads) {
  if (!tris || !nodes || !rays || !t_out) return 1;
  bind_geometry(tris, nt, nodes, nn);
  if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for num_threads(threads) schedule(dynamic, 256)
  for (long i = 0; i < (long)n; i++) {
    ray r{v3(rays[i].o), v3(rays[i].d)};
    hit_record rec{};
    t_out[i] = hit_bvh(r, rec) ? rec.t : -1.0f;
  }
  return 0;
}

// The shader's own hit records: hit_scene (comp:222-246: every triangle in a
// linear loop, then every bound sphere with `closest` reset to t_max) or
// hit_bvh (comp:262-311), per ray; out as oracle_hit_records (10 floats).
extern "C" int ref_shader_hit_records(const rt_triangle *tris, uint32_t nt, const rt_bvh_node *nodes, uint32_t nn,
                                      const rt_sphere *sph, uint32_t ns, uint32_t spheres_len, const rt_ray *rays,
                                      uint32_t n, int use_scene, float *out, int threads) {
  if (!tris || !nodes || !rays || !out || spheres_len > ns) return 1;
  bind_geometry(tris, nt, nodes, nn);
  static std::vector<sphere> S;
  S.resize(ns > 0 ? ns : 1);
  for (uint32_t i = 0; i < ns; i++)
    S[i] = sphere{vec4(sph[i].s[0], sph[i].s[1], sph[i].s[2], sph[i].s[3]), sph[i].material_index};
  spheres = GlslArray<sphere>{S.data(), (int)spheres_len};
  ubo.numTriangles = nt;
  if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for num_threads(threads) schedule(dynamic, 256)
  for (long i = 0; i < (long)n; i++) {
    ray r{v3(rays[i].o), v3(rays[i].d)};
    hit_record rec{};
    bool h = use_scene ? hit_scene(r, rec) : hit_bvh(r, rec);
    float *o = out + 10 * i;
    o[0] = h ? 1.0f : 0.0f;
    o[1] = rec.t;
    o[2] = rec.p.x;
    o[3] = rec.p.y;
    o[4] = rec.p.z;
    o[5] = rec.normal.x;
    o[6] = rec.normal.y;
    o[7] = rec.normal.z;
    std::memcpy(o + 8, &rec.materialIndex, 4);
    std::memcpy(o + 9, &rec.backFaceInt, 4);
  }
  return 0;
}

extern "C" int ref_shader_render(const rt_triangle *tris, uint32_t nt, const rt_material *mats, uint32_t nm,
                                 const rt_bvh_node *nodes, uint32_t nn, const rt_light *ls, uint32_t nl,
                                 uint32_t lights_len, const rt_sphere *sph, uint32_t ns, uint32_t spheres_len,
                                 const float cam_pos[3], uint32_t W, uint32_t H, uint32_t first_sample,
                                 uint32_t frames, float *out_rgba, int threads) {
  if (!tris || !mats || !nodes || !cam_pos || !out_rgba || W == 0 || H == 0) return 1;
  if (lights_len > nl || spheres_len > ns) return 2;
  std::vector<triangle> T(nt);
  for (uint32_t i = 0; i < nt; i++)
    T[i] = triangle{v3(tris[i].v0), v3(tris[i].v1), v3(tris[i].v2), tris[i].material_index};
  std::vector<material> M(nm);
  for (uint32_t i = 0; i < nm; i++) M[i] = material{mats[i].type, v3(mats[i].albedo)};
  std::vector<bvhNode> B(nn);
  for (uint32_t i = 0; i < nn; i++)
    B[i] = bvhNode{v3(nodes[i].min), v3(nodes[i].max), nodes[i].left, nodes[i].right, nodes[i].object};
  std::vector<light> L(nl > 0 ? nl : 1);
  for (uint32_t i = 0; i < nl; i++) L[i] = light{ls[i].triangle_index, ls[i].area};
  std::vector<sphere> S(ns > 0 ? ns : 1);
  for (uint32_t i = 0; i < ns; i++)
    S[i] = sphere{vec4(sph[i].s[0], sph[i].s[1], sph[i].s[2], sph[i].s[3]), sph[i].material_index};
  triangles = GlslArray<triangle>{T.data(), (int)nt};
  materials = GlslArray<material>{M.data(), (int)nm};
  bvh = GlslArray<bvhNode>{B.data(), (int)nn};
  lights = GlslArray<light>{L.data(), (int)lights_len};
  spheres = GlslArray<sphere>{S.data(), (int)spheres_len};
  targetTexture.w = accumulationTex.w = (int)W;
  targetTexture.h = accumulationTex.h = (int)H;
  targetTexture.px.assign(4ull * W * H, 0);
  accumulationTex.px.assign(4ull * W * H, 0);
  ubo.camPos = v3(cam_pos);
  ubo.time = 0.0f;
  ubo.numTriangles = nt;
  ubo.numLights = nl;
  ubo.numSpheres = ns;
  if (threads <= 0) threads = omp_get_max_threads();
  for (uint32_t f = 0; f < frames; f++) {
    ubo.currentSample = first_sample + f;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
    for (long y = 0; y < (long)H; y++) {
      for (uint32_t x = 0; x < W; x++) {
        gl_GlobalInvocationID = uvec3{x, (uint)y, 0u};
        glsl_init_globals();
        glsl_main();
      }
    }
    accumulationTex.px = targetTexture.px;
  }
  for (size_t i = 0; i < 4ull * W * H; i++) out_rgba[i] = targetTexture.px[i] / 255.0f;
  return 0;
}
