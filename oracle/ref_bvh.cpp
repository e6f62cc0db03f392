// Test infrastructure (oracle): a C entry point around the REFERENCE's own
// BVH builder. This file holds no reference code: it includes the
// reference's src/ray-tracing/Bvh.h (and through it GpuModels.h) from the
// reference checkout at build time (see oracle/Makefile, target `ref`) and
// compiles it against the glm stand-in in oracle/shim. The result,
// oracle/_ref/libref_bvh.so, is the ground truth that pins the oracle's
// restatement of Bvh::createBvh (oracle/rt_oracle.cpp) and the GPU builder.
//
// The reference never seeds rand(), so a process that builds one scene draws
// from glibc's default state (seed 1); ref_create_bvh reseeds with `seed`
// before every build so each call behaves like that fresh process.
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdlib>
#include <vector>
#include "Bvh.h"

extern "C" {

int ref_create_bvh(const void *triangles48, uint32_t n, void *out_nodes48, uint32_t seed) {
  static_assert(sizeof(GpuModel::Triangle) == 48, "Triangle layout");
  static_assert(sizeof(GpuModel::BvhNode) == 48, "BvhNode layout");
  if (n == 0) return -1;  // the reference indexes objects[0] of an empty leaf
  srand(seed);
  std::vector<Bvh::Object0> objects(n);
  const char *src = static_cast<const char *>(triangles48);
  for (uint32_t i = 0; i < n; i++) {
    objects[i].index = i;
    std::memcpy(&objects[i].t, src + 48ull * i, 48);
  }
  std::vector<GpuModel::BvhNode> nodes = Bvh::createBvh(objects);
  if (nodes.size() != 2ull * n - 1) return -2;
  char *dst = static_cast<char *>(out_nodes48);
  for (size_t i = 0; i < nodes.size(); i++) {
    // Copy fields only: the reference leaves padding bytes indeterminate.
    float rec[12];
    std::memset(rec, 0, sizeof(rec));
    std::memcpy(&rec[0], &nodes[i].min, 12);
    std::memcpy(&rec[4], &nodes[i].max, 12);
    std::memcpy(&rec[7], &nodes[i].leftNodeIndex, 4);
    std::memcpy(&rec[8], &nodes[i].rightNodeIndex, 4);
    std::memcpy(&rec[9], &nodes[i].objectIndex, 4);
    std::memcpy(dst + 48 * i, rec, 48);
  }
  return 0;
}

// Field offsets of the reference structs, for the layout tests.
int ref_layout(int *out, int cap) {
  int v[] = {
      (int)sizeof(GpuModel::Triangle), (int)offsetof(GpuModel::Triangle, v0),
      (int)offsetof(GpuModel::Triangle, v1), (int)offsetof(GpuModel::Triangle, v2),
      (int)offsetof(GpuModel::Triangle, materialIndex),
      (int)sizeof(GpuModel::BvhNode), (int)offsetof(GpuModel::BvhNode, min),
      (int)offsetof(GpuModel::BvhNode, max), (int)offsetof(GpuModel::BvhNode, leftNodeIndex),
      (int)offsetof(GpuModel::BvhNode, rightNodeIndex), (int)offsetof(GpuModel::BvhNode, objectIndex),
      (int)sizeof(GpuModel::Material), (int)offsetof(GpuModel::Material, type),
      (int)offsetof(GpuModel::Material, albedo),
      (int)sizeof(GpuModel::Sphere), (int)offsetof(GpuModel::Sphere, s),
      (int)offsetof(GpuModel::Sphere, materialIndex),
      (int)sizeof(GpuModel::Light), (int)offsetof(GpuModel::Light, triangleIndex),
      (int)offsetof(GpuModel::Light, area)};
  int n = (int)(sizeof(v) / sizeof(v[0]));
  for (int i = 0; i < n && i < cap; i++) out[i] = v[i];
  return n;
}

// glibc rand() after srand(seed), for pinning the builder's own generator.
void ref_rand_sequence(uint32_t seed, uint32_t count, int32_t *out) {
  srand(seed);
  for (uint32_t i = 0; i < count; i++) out[i] = rand();
}
}
