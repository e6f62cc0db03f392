/*
 * rt_obj.h — Wavefront OBJ triangles and the reference's demo scene.
 *
 * The reference loads every object of its scene with tinyobjloader
 * (src/scene/mesh.cpp:96-139), keeps only the vertex positions of each face
 * (src/ray-tracing/RtScene.h:13-31) and concatenates the objects into one
 * triangle array with a material index per object (RtScene.h:44-101).
 * These entry points do the same on the host; nothing here touches the GPU.
 */
#ifndef RTGB_RT_OBJ_H
#define RTGB_RT_OBJ_H

#include <stdint.h>
#include "rt_api.h"
#include "rt_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Triangles of one OBJ file, every one with material `material_index`:
 * replaces GpuModel::getTriangles(path, materialIndex) (RtScene.h:13-31).
 *
 * Faces are emitted in file order (tinyobj's shapes in order, each shape's
 * indices in order). A face index is the vertex part of `v`, `v/vt`,
 * `v//vn` or `v/vt/vn`: positive 1-based, or negative counting back from
 * the last vertex read so far. Faces with more than three vertices are
 * split as a fan from their first vertex; faces with fewer are skipped.
 * Other statements (vn, vt, o, g, s, usemtl, mtllib, l, p, comments) are
 * ignored. Coordinates are parsed digit by digit in double precision as
 * tinyobjloader does and rounded once to float.
 *
 * out may be NULL to count. Returns RT_ERR_NOT_FOUND if the file cannot be
 * read, RT_ERR_INVALID_SCENE for an index of 0 or one outside the vertices
 * read so far (rtGetLastError-style text in rtObjLastError), and
 * RT_ERR_INVALID_ARGUMENT if `capacity` is below the count; *count is
 * always set to the file's triangle count when the file parses. */
rt_status rtLoadObj(const char *path, uint32_t material_index, rt_triangle *out, uint32_t capacity,
                    uint32_t *count);

/* Text of the last rtLoadObj / rtLoadReferenceScene failure on this thread. */
const char *rtObjLastError(void);

/* The reference's scene (RtScene.h:44-101) from a directory holding its
 * doge_scene OBJ files: buff-doge, cheems, right, left, back, ceil, floor
 * and light, concatenated in that order with materials 0, 0, 1, 2, 0, 0, 0,
 * 3; the six materials gray, red, green, white light (albedo 2), metal and
 * glass; and one glass sphere at (0.6, 1, -1) with radius 0.6. Lights are
 * not returned: rtUploadScene derives them (or rtLightsFromMaterials).
 * tris may be NULL to count (*n_tris set); mats needs 6 entries and spheres
 * 1 (each may be NULL). No counterpart loads a directory in the reference,
 * which hard-codes its resources path (RtScene.h:46). */
rt_status rtLoadReferenceScene(const char *model_dir, rt_triangle *tris, uint32_t capacity, uint32_t *n_tris,
                               rt_material *mats, rt_sphere *spheres);

#ifdef __cplusplus
}
#endif

#endif /* RTGB_RT_OBJ_H */
