/*
 * rt_types.h — plain-old-data records shared by the host, the CUDA kernels and
 * callers of the C ABI.
 *
 * The scene records are byte-for-byte the std430 layouts that the reference's
 * compute shader binds (binding 3 triangles, 4 materials, 5 BVH nodes,
 * 6 lights, 7 spheres), so a buffer filled for the reference can be handed to
 * rtUploadScene unchanged:
 *
 *   rt_triangle  <- GpuModel::Triangle   src/ray-tracing/GpuModels.h:32-38
 *                   GLSL `triangle`      resources/shaders/source/include/definitions.glsl:6-11
 *   rt_material  <- GpuModel::Material   src/ray-tracing/GpuModels.h:26-30
 *                   GLSL `material`      definitions.glsl:1-4
 *   rt_bvh_node  <- GpuModel::BvhNode    src/ray-tracing/GpuModels.h:47-54
 *                   GLSL `bvhNode`       definitions.glsl:23-29
 *   rt_light     <- GpuModel::Light      src/ray-tracing/GpuModels.h:57-63
 *   rt_sphere    <- GpuModel::Sphere     src/ray-tracing/GpuModels.h:40-44
 *
 * Padding bytes of the reference structs are unspecified there; here two of
 * the Material padding words carry optional extensions (metal fuzz, glass
 * index of refraction). A zero in either keeps the reference behaviour.
 */
#ifndef RTGB_RT_TYPES_H
#define RTGB_RT_TYPES_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Material type ids: definitions.glsl:37-40, GpuModels.h:18-24. */
enum {
  RT_MATERIAL_LIGHT = 0,
  RT_MATERIAL_LAMBERTIAN = 1,
  RT_MATERIAL_METAL = 2,
  RT_MATERIAL_GLASS = 3
};

/* 48 bytes: v0@0, v1@16, v2@32 (vec3 in 16-byte slots), material_index@44. */
typedef struct rt_triangle {
  float v0[3];
  float _pad0;
  float v1[3];
  float _pad1;
  float v2[3];
  uint32_t material_index;
} rt_triangle;

/* 32 bytes: type@0, albedo@16.
 * fuzz@4 (metal only): 0 = perfect mirror as in the reference; > 0 perturbs the
 *   reflection by fuzz * random_in_unit_sphere() (three extra RNG draws).
 * ior@8 (glass only): 0 = the reference's hard-coded 1.5. */
typedef struct rt_material {
  uint32_t type;
  float fuzz;
  float ior;
  uint32_t _reserved;
  float albedo[3];
  float _pad;
} rt_material;

/* 48 bytes: min@0, max@16, left@28, right@32, object@36.
 * A leaf has left == right == -1 and object = triangle index; an inner node
 * has object == -1. Node 0 is the root. */
typedef struct rt_bvh_node {
  float min[3];
  float _pad0;
  float max[3];
  int32_t left;
  int32_t right;
  int32_t object;
  int32_t _pad1[2];
} rt_bvh_node;

/* 8 bytes: triangle_index@0, area@4. */
typedef struct rt_light {
  uint32_t triangle_index;
  float area;
} rt_light;

/* 32 bytes: s = (center.xyz, radius)@0, material_index@16. */
typedef struct rt_sphere {
  float s[4];
  uint32_t material_index;
  uint32_t _pad[3];
} rt_sphere;

/* A pinhole camera in the form the reference builds in its shader
 * (ray-trace-compute.comp:365-372): the ray through pixel (x, y) of a W x H
 * image is origin -> lower_left + (x/W) * horizontal + (y/H) * vertical. */
typedef struct rt_camera {
  float origin[3];
  float lower_left[3];
  float horizontal[3];
  float vertical[3];
} rt_camera;

/* 32 bytes: a ray for closest-hit casting; hits are accepted for
 * tmin < t < tmax. */
typedef struct rt_ray {
  float o[3];
  float tmin;
  float d[3];
  float tmax;
} rt_ray;

/* 16 bytes: closest hit. tri = -1 on a miss (t, u, v are then 0). u, v are the
 * barycentrics of the reference's triIntersect (comp:157-173). */
typedef struct rt_hit {
  int32_t tri;
  float t;
  float u;
  float v;
} rt_hit;

/* Compatibility switches that reproduce reference quirks bit-for-bit. */
enum {
  /* Traversal stack of 16 entries that silently drops work on overflow
   * (comp:262, 280). Default: no truncation. */
  RT_COMPAT_STACK16 = 1u << 0,
  /* lights.length() and spheres.length() evaluate to 1 because the reference
   * binds each storage buffer with range sizeof(T) (src/memory/Buffer.h:37,85). */
  RT_COMPAT_LEN1 = 1u << 1,
  /* Spheres tested after the BVH with `closest` reset to tmax, as in the
   * reference's linear hit_scene (comp:236). */
  RT_COMPAT_SPHERE_OVERRIDE = 1u << 2,
  /* No spheres at all, as in the reference's hit_bvh-only render path
   * (comp:323). */
  RT_COMPAT_NO_SPHERES = 1u << 3,
  /* Round the accumulation to RGBA8 UNORM after every sample, as the
   * reference's rgba8 storage images do (comp:17-19, main.cpp:108-140). */
  RT_COMPAT_UNORM8 = 1u << 4,
  /* Shade with the alternate shader's hemisphere scatter
   * (ray-trace-compute-simple.comp:62-68). */
  RT_SHADE_SIMPLE = 1u << 5,
  /* Closest-hit queries: report t, u, v exactly as the reference's fp32
   * triIntersect computes them. By default the winning triangle (chosen with
   * that fp32 arithmetic) is re-intersected in fp64 with the same formula and
   * t, u, v are that result rounded to fp32. */
  RT_HIT_FP32 = 1u << 6
};

/* Per-render parameters (the reference's UBO plus its compile-time knobs:
 * NUM_BOUNCES comp:313, currentSample main.cpp:165-183). */
typedef struct rt_render_params {
  uint32_t width;
  uint32_t height;
  uint32_t spp;          /* samples accumulated by this call */
  uint32_t max_bounces;  /* reference: 2 */
  uint32_t sample_index; /* running-mean index of the first sample (0 = reset) */
  uint32_t flags;        /* RT_COMPAT_* */
  uint32_t _reserved[2];
} rt_render_params;

#ifdef __cplusplus
}
#endif

#endif /* RTGB_RT_TYPES_H */
