/*
 * rt_scenes.h — deterministic synthetic workloads.
 *
 * The reference renders one hard-coded scene loaded from OBJ files
 * (src/ray-tracing/RtScene.h:44-101); the workloads measured here are seeded
 * synthetic scenes instead. Every generator uses a project-written SplitMix64
 * stream and only +, -, *, / and sqrt in IEEE double (a series logarithm
 * replaces libm), so the same seed gives the same bytes on x86-64 and
 * aarch64.
 *
 * None of these functions touches the GPU.
 */
#ifndef RTGB_RT_SCENES_H
#define RTGB_RT_SCENES_H

#include <stdint.h>
#include "rt_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Cornell-style box of 12 wall triangles spanning [-5,5]^3 with the front
 * (z = -5) open: floor, ceiling, back, left and right walls (10 triangles)
 * and an emissive quad just under the ceiling (2 triangles), followed by
 * `n_soup` soup triangles (centroid U[-4,4]^3, vertices centroid +
 * N(0, 0.25^2) per axis, material uniform over the 7 non-light materials)
 * and `n_spheres` spheres (centre U[-3.5,3.5]^3, radius U[r_lo, r_hi]).
 * Materials (8): 0-3 lambertian albedo U[0,1]^3; 4-5 metal albedo
 * U[0.5,1]^3, fuzz U[0,0.5]; 6 glass ior 1.5; 7 light with radiance
 * `light_radiance` (albedo of a LightSource material).
 * tris needs 12 + n_soup entries, mats 8, spheres n_spheres (may be NULL
 * when n_spheres == 0). Returns the triangle count. */
uint32_t rtgbGenCornell(uint64_t seed, uint32_t n_soup, uint32_t n_spheres, float r_lo, float r_hi,
                        float light_radiance, rt_triangle *tris, rt_material *mats, rt_sphere *spheres);

/* Icosphere: the icosahedron subdivided `level` times by edge midpoints and
 * projected to the unit sphere, scaled by `radius`, then every vertex
 * displaced radially by a factor (1 + sigma * N(0,1)). 20 * 4^level
 * triangles, all with material `material`. Returns the triangle count
 * (tris may be NULL to query it). */
uint32_t rtgbGenIcosphere(uint64_t seed, uint32_t level, float radius, float sigma, uint32_t material,
                          rt_triangle *tris);

/* Primary rays of a pinhole camera (one per pixel, row-major, y down):
 * origin = camera origin, direction = normalize(lower_left + (x/W)*horizontal
 * + (y/H)*vertical - origin). */
void rtgbGenCameraRays(const rt_camera *cam, uint32_t W, uint32_t H, float tmin, float tmax, rt_ray *rays);

/* Incoherent rays: origin U[lo,hi]^3, direction uniform on the unit sphere. */
void rtgbGenRandomRays(uint64_t seed, uint64_t n, float lo, float hi, float tmin, float tmax, rt_ray *rays);

/* Large scene: a gx x gz grid of icospheres of `level` (flattened in y by
 * `flatten`, radial noise sigma) of which the first `keep_per_sphere`
 * triangles are kept, plus the 12-triangle Cornell box scaled by `box_scale`.
 * Sphere materials: 40% glass, 30% metal, 30% lambertian by sphere. Writes
 * 12 + gx*gz*keep triangles and 8 materials; returns the triangle count. */
uint32_t rtgbGenGrid(uint64_t seed, uint32_t gx, uint32_t gz, uint32_t level, float flatten, float sigma,
                     uint32_t keep_per_sphere, float box_scale, rt_triangle *tris, rt_material *mats);

/* Uniform double in [0,1) from the SplitMix64 stream at (seed, index). */
double rtgbUniform(uint64_t seed, uint64_t index);

/* Host form of the 8-wide node quantization the scene upload runs on the
 * GPU: `boxes` holds 8 child slots as lo.xyz, hi.xyz and `refs` their refs,
 * of which the slots set in `fmask` (bit s: slot s, at least one) are
 * filled; `out` receives the node's 24 words (origin, int8 exponents and
 * the filled mask, 8-bit child bounds with qlo = 255, qhi = 0 in empty
 * slots, refs with ~0 in empty slots). Returns 1, or 0 when a box
 * does not fit the node's grid. Exposed so the decoded boxes can be checked
 * to contain the originals without a GPU. */
uint32_t rtgbQuantizeNode8(const float *boxes, const int32_t *refs, uint32_t fmask, uint32_t *out);

/* Host form of the 8-wide fold's slot assignment: child i of `cnt` (1..8)
 * boxes (lo.xyz, hi.xyz) goes to slot slot_of[i], slot bits (x, y, z) naming
 * the node corner on the positive side of each set axis (greedy on the
 * offset of the box centre from the node centre). Returns 1, or 0 on bad
 * arguments. */
uint32_t rtgbAssignOctantSlots(const float *boxes, uint32_t cnt, int32_t *slot_of);

#ifdef __cplusplus
}
#endif

#endif /* RTGB_RT_SCENES_H */
