// Host runtime behind the C ABI (include/rtgb/rt_api.h).
//
// A context owns one device, one stream, a device error word, a ring of
// per-launch work counters and the registry of resident scenes. A scene is
// one device allocation holding the reference-layout arrays (triangles,
// materials, lights, spheres, Bvh.h nodes) and the derived traversal layout.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "rt_internal.h"

using namespace rtgb;

namespace {

constexpr uint32_t kCounterRing = 1024;

struct Scene {
  DevScene dev{};
  void *slab = nullptr;
  uint64_t bytes = 0;
  rt_camera camera{};
  bool has_camera = false;
  float build_ms = 0.0f, relayout_ms = 0.0f;
  uint64_t last_use = 0;
};

}  // namespace

// Staging of one rtTraceClosestHost call: two streams whose chunks
// alternate, each with its own device buffer.
struct HostLane {
  cudaStream_t st[2] = {nullptr, nullptr};
  void *stage[2] = {nullptr, nullptr};
  size_t bytes = 0;
};

struct rt_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::mutex mu;
  std::unordered_map<uint32_t, Scene *> scenes;
  uint32_t next_id = 1;
  std::string last_error;
  uint32_t *d_err = nullptr;       // [0] kernel error bits
  uint32_t *d_counters = nullptr;  // kCounterRing launch-private work counters
  unsigned long long *d_segments = nullptr;
  std::atomic<uint32_t> counter_slot{0};
  TraceOpts trace_opts;
  RenderOpts render_opts;
  BuildOpts build_opts;
  uint64_t budget = 0, used = 0, tick = 0;
  // rtTraceClosestHost staging: every lane ever made, and the idle ones
  // (a call takes one, so calls from several host threads overlap).
  std::vector<HostLane *> host_lanes, idle_lanes;
};

namespace {

thread_local std::string tl_error;

rt_status fail(rt_ctx *ctx, rt_status s, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (ctx) {
    std::lock_guard<std::mutex> g(ctx->mu);
    ctx->last_error = buf;
  }
  return s;
}

rt_status cuda_fail(rt_ctx *ctx, cudaError_t e, const char *what) {
  return fail(ctx, e == cudaErrorMemoryAllocation ? RT_ERR_OUT_OF_MEMORY : RT_ERR_CUDA, "%s: %s", what,
              cudaGetErrorString(e));
}

#define CK(call, what)                              \
  do {                                              \
    cudaError_t e_ = (call);                        \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what); \
  } while (0)

inline bool finite3(const float *v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

cudaStream_t pick_stream(rt_ctx *ctx, void *s) { return s ? (cudaStream_t)s : ctx->stream; }

uint32_t *next_counter(rt_ctx *ctx) {
  uint32_t slot = ctx->counter_slot.fetch_add(1) % kCounterRing;
  return ctx->d_counters + slot;
}

// Structural check of a Bvh.h node array: a full binary tree rooted at 0 in
// which every node is reached once and leaves name valid triangles. Returns
// the depth (levels) or 0 when the array is malformed.
uint32_t check_tree(const rt_bvh_node *nodes, uint32_t nn, uint32_t ntris, std::string &why) {
  std::vector<uint8_t> seen(nn, 0);
  std::vector<std::pair<uint32_t, uint32_t>> stack{{0u, 1u}};
  uint32_t depth = 0, visited = 0;
  while (!stack.empty()) {
    auto [i, d] = stack.back();
    stack.pop_back();
    if (i >= nn || seen[i]) {
      why = "node array is not a tree";
      return 0;
    }
    seen[i] = 1;
    visited++;
    depth = std::max(depth, d);
    const rt_bvh_node &n = nodes[i];
    if (n.left == -1 && n.right == -1) {
      if (n.object < 0 || (uint32_t)n.object >= ntris) {
        why = "leaf names a triangle out of range";
        return 0;
      }
    } else {
      if (n.left < 0 || n.right < 0 || n.object != -1) {
        why = "inner node must have two children and object -1";
        return 0;
      }
      stack.push_back({(uint32_t)n.left, d + 1});
      stack.push_back({(uint32_t)n.right, d + 1});
    }
  }
  if (visited != nn) {
    why = "node array has unreachable nodes";
    return 0;
  }
  return depth;
}

struct SlabLayout {
  size_t tris, mats, lights, spheres, nodes, bvh2, tpre, leaf, bvh8, total;
};

SlabLayout slab_layout(uint32_t nt, uint32_t nm, uint32_t nl, uint32_t ns) {
  const uint32_t nnodes = 2 * nt - 1, ninner = nt > 1 ? nt - 1 : 1;
  SlabLayout L;
  L.tris = 0;
  L.mats = L.tris + align256(sizeof(rt_triangle) * nt);
  L.lights = L.mats + align256(sizeof(rt_material) * nm);
  L.spheres = L.lights + align256(sizeof(rt_light) * std::max(nl, 1u));
  L.nodes = L.spheres + align256(sizeof(rt_sphere) * std::max(ns, 1u));
  L.bvh2 = L.nodes + align256(sizeof(rt_bvh_node) * nnodes);
  L.tpre = L.bvh2 + align256(64ull * ninner);
  L.leaf = L.tpre + align256(48ull * nt);
  L.bvh8 = L.leaf + align256(4ull * nt);
  L.total = L.bvh8 + align256(kBvh8NodeBytes * bvh8_capacity(nt));
  return L;
}

Scene *find_scene(rt_ctx *ctx, rt_scene_id id) {
  auto it = ctx->scenes.find(id);
  if (it == ctx->scenes.end()) return nullptr;
  it->second->last_use = ++ctx->tick;
  return it->second;
}

}  // namespace

extern "C" {

const char *rtStatusString(rt_status s) {
  switch (s) {
    case RT_SUCCESS: return "success";
    case RT_ERR_INVALID_ARGUMENT: return "invalid argument";
    case RT_ERR_OUT_OF_MEMORY: return "out of device memory";
    case RT_ERR_CUDA: return "CUDA error";
    case RT_ERR_NOT_FOUND: return "scene not found";
    case RT_ERR_INVALID_SCENE: return "invalid scene data";
    case RT_ERR_STACK_OVERFLOW: return "traversal stack overflow";
    case RT_ERR_TIMEOUT: return "timed out";
    case RT_ERR_BUDGET: return "HBM budget exceeded";
    case RT_ERR_BUSY: return "busy";
    case RT_ERR_INTERNAL: return "internal error";
  }
  return "unknown status";
}

const char *rtGetLastError(rt_ctx *ctx) {
  if (!ctx) return "null context";
  std::lock_guard<std::mutex> g(ctx->mu);
  tl_error = ctx->last_error;
  return tl_error.c_str();
}

rt_status rtCreate(rt_ctx **out, const rt_ctx_desc *desc) {
  if (!out) return RT_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  rt_ctx *ctx = new rt_ctx();
  ctx->device = desc ? desc->device : 0;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc((void **)&ctx->d_err, 64);
  if (e == cudaSuccess) e = cudaMemset(ctx->d_err, 0, 64);
  if (e == cudaSuccess) e = cudaMalloc((void **)&ctx->d_counters, sizeof(uint32_t) * kCounterRing);
  if (e == cudaSuccess) e = cudaMalloc((void **)&ctx->d_segments, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(ctx->d_segments, 0, sizeof(unsigned long long));
  if (e != cudaSuccess) {
    tl_error = std::string("rtCreate: ") + cudaGetErrorString(e);
    rtDestroy(ctx);
    return e == cudaErrorMemoryAllocation ? RT_ERR_OUT_OF_MEMORY : RT_ERR_CUDA;
  }
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  ctx->budget = (desc && desc->hbm_budget_bytes) ? desc->hbm_budget_bytes : (uint64_t)(0.8 * (double)free_b);
  *out = ctx;
  return RT_SUCCESS;
}

rt_status rtDestroy(rt_ctx *ctx) {
  if (!ctx) return RT_ERR_INVALID_ARGUMENT;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (auto &kv : ctx->scenes) {
    cudaFree(kv.second->slab);
    delete kv.second;
  }
  for (HostLane *l : ctx->host_lanes) {
    for (int i = 0; i < 2; i++) {
      if (l->stage[i]) cudaFree(l->stage[i]);
      if (l->st[i]) cudaStreamDestroy(l->st[i]);
    }
    delete l;
  }
  if (ctx->d_err) cudaFree(ctx->d_err);
  if (ctx->d_counters) cudaFree(ctx->d_counters);
  if (ctx->d_segments) cudaFree(ctx->d_segments);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return RT_SUCCESS;
}

uint32_t rtLightsFromMaterials(const rt_triangle *tris, uint32_t n, const rt_material *mats, uint32_t nm,
                               rt_light *out) {
  uint32_t k = 0;
  for (uint32_t i = 0; i < n; i++) {
    uint32_t m = tris[i].material_index;
    if (m < nm && mats[m].type == RT_MATERIAL_LIGHT) {
      // area = length(cross(v0, v1)) * 0.5 (RtScene.h:93); this file is
      // built with -ffp-contract=off, so each operation rounds separately.
      const float *a = tris[i].v0, *b = tris[i].v1;
      float x = a[1] * b[2] - b[1] * a[2];
      float y = a[2] * b[0] - b[2] * a[0];
      float z = a[0] * b[1] - b[0] * a[1];
      float len = std::sqrt(x * x + y * y + z * z);
      if (out) out[k] = rt_light{i, len * 0.5f};
      k++;
    }
  }
  return k;
}

rt_status rtCameraFromReference(const float cam_pos[3], uint32_t W, uint32_t H, rt_camera *out) {
  if (!cam_pos || !out || W == 0 || H == 0) return RT_ERR_INVALID_ARGUMENT;
  // comp:358-369 in fp32: theta = vfov*pi/180, h = tan(theta/2), viewport
  // 2h high and W/H * 2h wide, origin = camPos.zxy * (-1, 1, 1).
  const float vfov = 30.0f, pi = 3.1415926535897932385f;
  float theta = vfov * pi / 180.0f;
  float h = std::tan(theta / 2.0f);
  float vh = 2.0f * h;
  float vw = (float)W / (float)H * vh;
  float hor[3] = {vw, 0.0f, 0.0f}, ver[3] = {0.0f, -vh, 0.0f};
  float org[3] = {-cam_pos[2], cam_pos[0], cam_pos[1]};
  float foc[3] = {0.0f, 0.0f, 1.0f};
  for (int a = 0; a < 3; a++) {
    out->origin[a] = org[a];
    out->horizontal[a] = hor[a];
    out->vertical[a] = ver[a];
    out->lower_left[a] = org[a] - hor[a] / 2.0f - ver[a] / 2.0f - foc[a];
  }
  return RT_SUCCESS;
}

rt_status rtCameraLookAt(const float eye[3], const float target[3], const float up[3], float vfov_deg, uint32_t W,
                         uint32_t H, rt_camera *out) {
  if (!eye || !target || !up || !out || W == 0 || H == 0 || !(vfov_deg > 0.0f && vfov_deg < 180.0f))
    return RT_ERR_INVALID_ARGUMENT;
  // Computed in double and rounded once: the camera is an input to both
  // the kernels and the oracle, so only its stored fp32 values matter.
  double f[3], r[3], u[3];
  for (int a = 0; a < 3; a++) f[a] = (double)target[a] - (double)eye[a];
  double fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
  if (!(fl > 0.0)) return RT_ERR_INVALID_ARGUMENT;
  for (double &x : f) x /= fl;
  r[0] = f[1] * up[2] - f[2] * up[1];
  r[1] = f[2] * up[0] - f[0] * up[2];
  r[2] = f[0] * up[1] - f[1] * up[0];
  double rl = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  if (!(rl > 0.0)) return RT_ERR_INVALID_ARGUMENT;
  for (double &x : r) x /= rl;
  u[0] = r[1] * f[2] - r[2] * f[1];
  u[1] = r[2] * f[0] - r[0] * f[2];
  u[2] = r[0] * f[1] - r[1] * f[0];
  const double kPi = 3.14159265358979323846;
  double vh = 2.0 * std::tan((double)vfov_deg * kPi / 360.0);
  double vw = vh * (double)W / (double)H;
  for (int a = 0; a < 3; a++) {
    double hor = vw * r[a], ver = -vh * u[a];
    out->origin[a] = eye[a];
    out->horizontal[a] = (float)hor;
    out->vertical[a] = (float)ver;
    out->lower_left[a] = (float)((double)eye[a] + f[a] - 0.5 * hor - 0.5 * ver);
  }
  return RT_SUCCESS;
}

rt_status rtUploadScene(rt_ctx *ctx, const rt_triangle *tris, uint32_t nt, const rt_material *mats, uint32_t nm,
                        const rt_bvh_node *nodes, uint32_t nn, const rt_light *lights, uint32_t nl,
                        const rt_sphere *spheres, uint32_t ns, uint32_t bvh_seed, rt_scene_id *out) {
  if (!ctx || !out) return RT_ERR_INVALID_ARGUMENT;
  *out = 0;
  if (!tris || nt == 0) return fail(ctx, RT_ERR_INVALID_SCENE, "a scene needs at least one triangle");
  if (nt > (1u << 30)) return fail(ctx, RT_ERR_INVALID_SCENE, "too many triangles (%u)", nt);
  if (!mats || nm == 0) return fail(ctx, RT_ERR_INVALID_SCENE, "a scene needs at least one material");
  if ((ns && !spheres) || (nl && !lights && lights != nullptr))
    return fail(ctx, RT_ERR_INVALID_ARGUMENT, "null array with nonzero count");
  for (uint32_t i = 0; i < nm; i++) {
    if (mats[i].type > RT_MATERIAL_GLASS) return fail(ctx, RT_ERR_INVALID_SCENE, "material %u: type %u", i, mats[i].type);
    if (!finite3(mats[i].albedo) || !std::isfinite(mats[i].fuzz) || !std::isfinite(mats[i].ior) ||
        mats[i].fuzz < 0.0f || mats[i].ior < 0.0f)
      return fail(ctx, RT_ERR_INVALID_SCENE, "material %u: non-finite or negative parameter", i);
  }
  for (uint32_t i = 0; i < nt; i++) {
    if (!finite3(tris[i].v0) || !finite3(tris[i].v1) || !finite3(tris[i].v2))
      return fail(ctx, RT_ERR_INVALID_SCENE, "triangle %u: non-finite vertex", i);
    if (tris[i].material_index >= nm)
      return fail(ctx, RT_ERR_INVALID_SCENE, "triangle %u: material %u out of range", i, tris[i].material_index);
  }
  for (uint32_t i = 0; i < ns; i++) {
    if (!finite3(spheres[i].s) || !std::isfinite(spheres[i].s[3]) || spheres[i].material_index >= nm)
      return fail(ctx, RT_ERR_INVALID_SCENE, "sphere %u: bad centre, radius or material", i);
  }
  std::vector<rt_light> derived;
  if (!lights) {
    derived.resize(rtLightsFromMaterials(tris, nt, mats, nm, nullptr));
    rtLightsFromMaterials(tris, nt, mats, nm, derived.data());
    lights = derived.data();
    nl = (uint32_t)derived.size();
  }
  for (uint32_t i = 0; i < nl; i++)
    if (lights[i].triangle_index >= nt) return fail(ctx, RT_ERR_INVALID_SCENE, "light %u: triangle out of range", i);
  const uint32_t nnodes = 2 * nt - 1;
  uint32_t depth = 0;
  if (nodes) {
    if (nn != nnodes) return fail(ctx, RT_ERR_INVALID_SCENE, "expected %u nodes, got %u", nnodes, nn);
    std::string why;
    depth = check_tree(nodes, nn, nt, why);
    if (!depth) return fail(ctx, RT_ERR_INVALID_SCENE, "%s", why.c_str());
    if (depth > 64) return fail(ctx, RT_ERR_INVALID_SCENE, "tree depth %u exceeds 64", depth);
  }

  // One slab per scene.
  SlabLayout L = slab_layout(nt, nm, nl, ns);
  size_t off_tris = L.tris, off_mats = L.mats, off_lights = L.lights, off_spheres = L.spheres, off_nodes = L.nodes,
         off_bvh2 = L.bvh2, off_tpre = L.tpre, off_leaf = L.leaf, off_bvh8 = L.bvh8, total = L.total;
  {
    std::lock_guard<std::mutex> g(ctx->mu);
    if (ctx->used + total > ctx->budget)
      return RT_ERR_BUDGET;
    ctx->used += total;
  }
  auto unreserve = [&]() {
    std::lock_guard<std::mutex> g(ctx->mu);
    ctx->used -= total;
  };
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  char *slab = nullptr;
  cudaError_t e = cudaMalloc((void **)&slab, total);
  if (e != cudaSuccess) {
    unreserve();
    return cuda_fail(ctx, e, "scene allocation");
  }
  Scene *sc = new Scene();
  sc->slab = slab;
  sc->bytes = total;
  DevScene &d = sc->dev;
  d.tris = (const rt_triangle *)(slab + off_tris);
  d.mats = (const rt_material *)(slab + off_mats);
  d.lights = (const rt_light *)(slab + off_lights);
  d.spheres = (const rt_sphere *)(slab + off_spheres);
  d.nodes = (const rt_bvh_node *)(slab + off_nodes);
  d.bvh2 = (const float4 *)(slab + off_bvh2);
  d.tpre = (const float4 *)(slab + off_tpre);
  d.leaf_tri = (const int32_t *)(slab + off_leaf);
  d.ntris = nt;
  d.nmats = nm;
  d.nlights = nl;
  d.nspheres = ns;
  d.nnodes = nnodes;
  cudaStream_t st = ctx->stream;
  auto abort_upload = [&](rt_status s) {
    cudaStreamSynchronize(st);
    cudaFree(slab);
    delete sc;
    unreserve();
    return s;
  };
#define UCK(call, what)                                                   \
  do {                                                                    \
    cudaError_t e_ = (call);                                              \
    if (e_ != cudaSuccess) return abort_upload(cuda_fail(ctx, e_, what)); \
  } while (0)
  UCK(cudaMemcpyAsync(slab + off_tris, tris, sizeof(rt_triangle) * nt, cudaMemcpyHostToDevice, st), "upload triangles");
  UCK(cudaMemcpyAsync(slab + off_mats, mats, sizeof(rt_material) * nm, cudaMemcpyHostToDevice, st), "upload materials");
  if (nl) UCK(cudaMemcpyAsync(slab + off_lights, lights, sizeof(rt_light) * nl, cudaMemcpyHostToDevice, st), "upload lights");
  if (ns) UCK(cudaMemcpyAsync(slab + off_spheres, spheres, sizeof(rt_sphere) * ns, cudaMemcpyHostToDevice, st), "upload spheres");
  rt_bvh_node *dnodes = (rt_bvh_node *)(slab + off_nodes);
  bool median_tree = nodes != nullptr;
  if (nodes) {
    UCK(cudaMemcpyAsync(dnodes, nodes, sizeof(rt_bvh_node) * nnodes, cudaMemcpyHostToDevice, st), "upload nodes");
  } else {
    int builder = 0, test_error_level = -1, ploc_radius = 16;
    {
      std::lock_guard<std::mutex> g(ctx->mu);
      builder = ctx->build_opts.builder;
      test_error_level = ctx->build_opts.test_error_level;
      ploc_radius = ctx->build_opts.ploc_radius;
    }
    char errbuf[256] = {0};
    rt_status bs;
    if (builder == 1) {
      bs = gpu_build_lbvh((const rt_triangle *)(slab + off_tris), nt, dnodes, st, &sc->build_ms, &depth, errbuf,
                          sizeof(errbuf));
    } else if (builder == 2) {
      bs = gpu_build_ploc((const rt_triangle *)(slab + off_tris), nt, (uint32_t)ploc_radius, dnodes, st,
                          &sc->build_ms, &depth, errbuf, sizeof(errbuf));
    } else {
      median_tree = true;
      std::vector<uint8_t> axes(nnodes);
      glibc_rand_axes(bvh_seed, nnodes, axes.data());
      bs = gpu_build_bvh((const rt_triangle *)(slab + off_tris), nt, axes.data(), dnodes, st, &sc->build_ms, &depth,
                         errbuf, sizeof(errbuf), test_error_level);
    }
    if (bs != RT_SUCCESS) return abort_upload(fail(ctx, bs, "%s", errbuf));
  }
  d.depth = depth;
  if (depth > 64) return abort_upload(fail(ctx, RT_ERR_INVALID_SCENE, "tree depth %u exceeds 64", depth));
  d.median_tree = median_tree ? 1u : 0u;
  // Traversal layout.
  {
    uint32_t *scratch = nullptr;
    size_t words = 2ull * nnodes + nnodes / 1024 + 2;
    UCK(cudaMallocAsync((void **)&scratch, 4 * words, st), "relayout scratch");
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, st);
    cudaError_t le = launch_relayout(dnodes, nnodes, d.tris, (float4 *)d.bvh2, (float4 *)d.tpre,
                                     (int32_t *)d.leaf_tri, scratch, st);
    cudaEventRecord(b, st);
    cudaFreeAsync(scratch, st);
    if (le != cudaSuccess) {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      return abort_upload(cuda_fail(ctx, le, "relayout"));
    }
    rt_bvh_node root;
    UCK(cudaMemcpyAsync(&root, dnodes, sizeof(root), cudaMemcpyDeviceToHost, st), "read root");
    UCK(cudaStreamSynchronize(st), "upload");
    cudaEventElapsedTime(&sc->relayout_ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    for (int k = 0; k < 3; k++) {
      d.root_lo[k] = root.min[k];
      d.root_hi[k] = root.max[k];
    }
    d.root_ref = (root.left != -1) ? 0 : ~0;
  }
  // The 8-wide fold of the same tree.
  {
    bool sah = true;
    {
      std::lock_guard<std::mutex> g(ctx->mu);
      sah = ctx->build_opts.collapse != 0;
    }
    char errbuf[128] = {0};
    cudaError_t be = build_bvh8(d, sah, slab + off_bvh8, bvh8_capacity(nt), &d.n8, &d.levels8, &d.root8, errbuf,
                                sizeof(errbuf), st);
    if (be != cudaSuccess && errbuf[0]) return abort_upload(fail(ctx, RT_ERR_INTERNAL, "%s", errbuf));
    UCK(be, "bvh8");
    d.bvh8 = (const float4 *)(slab + off_bvh8);
  }
#undef UCK
  std::lock_guard<std::mutex> g(ctx->mu);
  uint32_t id = ctx->next_id++;
  sc->last_use = ++ctx->tick;
  ctx->scenes[id] = sc;
  *out = id;
  return RT_SUCCESS;
}

rt_status rtReleaseScene(rt_ctx *ctx, rt_scene_id id) {
  if (!ctx) return RT_ERR_INVALID_ARGUMENT;
  Scene *sc = nullptr;
  {
    std::lock_guard<std::mutex> g(ctx->mu);
    auto it = ctx->scenes.find(id);
    if (it == ctx->scenes.end()) return RT_ERR_NOT_FOUND;
    sc = it->second;
    ctx->scenes.erase(it);
    ctx->used -= sc->bytes;
  }
  // Work already queued on any stream may still read the scene.
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  cudaFree(sc->slab);
  delete sc;
  return RT_SUCCESS;
}

rt_status rtGetSceneInfo(rt_ctx *ctx, rt_scene_id id, rt_scene_info *out) {
  if (!ctx || !out) return RT_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> g(ctx->mu);
  Scene *sc = find_scene(ctx, id);
  if (!sc) return RT_ERR_NOT_FOUND;
  out->triangles = sc->dev.ntris;
  out->materials = sc->dev.nmats;
  out->lights = sc->dev.nlights;
  out->spheres = sc->dev.nspheres;
  out->nodes = sc->dev.nnodes;
  out->depth = sc->dev.depth;
  out->device_bytes = sc->bytes;
  out->build_ms = sc->build_ms;
  out->relayout_ms = sc->relayout_ms;
  return RT_SUCCESS;
}

rt_status rtDownloadBvh(rt_ctx *ctx, rt_scene_id id, rt_bvh_node *host_out, uint32_t n) {
  if (!ctx || !host_out) return RT_ERR_INVALID_ARGUMENT;
  DevScene d;
  {
    std::lock_guard<std::mutex> g(ctx->mu);
    Scene *sc = find_scene(ctx, id);
    if (!sc) return RT_ERR_NOT_FOUND;
    d = sc->dev;
  }
  if (n != d.nnodes) return fail(ctx, RT_ERR_INVALID_ARGUMENT, "expected %u nodes", d.nnodes);
  CK(cudaMemcpyAsync(host_out, d.nodes, sizeof(rt_bvh_node) * n, cudaMemcpyDeviceToHost, ctx->stream), "download");
  CK(cudaStreamSynchronize(ctx->stream), "download");
  return RT_SUCCESS;
}

rt_status rtDownloadLights(rt_ctx *ctx, rt_scene_id id, rt_light *host_out, uint32_t n) {
  if (!ctx || (!host_out && n)) return RT_ERR_INVALID_ARGUMENT;
  DevScene d;
  {
    std::lock_guard<std::mutex> g(ctx->mu);
    Scene *sc = find_scene(ctx, id);
    if (!sc) return RT_ERR_NOT_FOUND;
    d = sc->dev;
  }
  if (n != d.nlights) return fail(ctx, RT_ERR_INVALID_ARGUMENT, "expected %u lights", d.nlights);
  if (n == 0) return RT_SUCCESS;
  CK(cudaMemcpyAsync(host_out, d.lights, sizeof(rt_light) * n, cudaMemcpyDeviceToHost, ctx->stream), "download");
  CK(cudaStreamSynchronize(ctx->stream), "download");
  return RT_SUCCESS;
}

rt_status rtSetCamera(rt_ctx *ctx, rt_scene_id id, const rt_camera *cam) {
  if (!ctx || !cam) return RT_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> g(ctx->mu);
  Scene *sc = find_scene(ctx, id);
  if (!sc) return RT_ERR_NOT_FOUND;
  sc->camera = *cam;
  sc->has_camera = true;
  return RT_SUCCESS;
}

rt_status rtTraceClosestEx(rt_ctx *ctx, rt_scene_id id, const rt_ray *rays, uint32_t n, rt_hit *hits, uint32_t flags,
                           void *stream);

rt_status rtTraceClosest(rt_ctx *ctx, rt_scene_id id, const rt_ray *rays, uint32_t n, rt_hit *hits, void *stream) {
  return rtTraceClosestEx(ctx, id, rays, n, hits, 0, stream);
}

rt_status rtTraceClosestEx(rt_ctx *ctx, rt_scene_id id, const rt_ray *rays, uint32_t n, rt_hit *hits, uint32_t flags,
                           void *stream) {
  if (!ctx || (n && (!rays || !hits))) return RT_ERR_INVALID_ARGUMENT;
  if ((uintptr_t)rays % 16 || (uintptr_t)hits % 16)
    return fail(ctx, RT_ERR_INVALID_ARGUMENT, "ray and hit arrays must be 16-byte aligned");
  if (flags & ~(uint32_t)(RT_COMPAT_STACK16 | RT_HIT_FP32))
    return fail(ctx, RT_ERR_INVALID_ARGUMENT, "unsupported trace flags");
  DevScene d;
  {
    std::lock_guard<std::mutex> g(ctx->mu);
    Scene *sc = find_scene(ctx, id);
    if (!sc) return RT_ERR_NOT_FOUND;
    d = sc->dev;
  }
  if (n == 0) return RT_SUCCESS;
  cudaStream_t st = pick_stream(ctx, stream);
  TraceOpts opts;
  {
    std::lock_guard<std::mutex> g(ctx->mu);
    opts = ctx->trace_opts;
  }
  if (flags & RT_COMPAT_STACK16) {
    cudaError_t e = launch_trace_literal16(d, rays, n, hits, st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "trace launch");
    return RT_SUCCESS;
  }
  const bool refine = (flags & RT_HIT_FP32) == 0;
  const bool use_sort = opts.sort && n >= 65536;
  // Stream-ordered scratch from the device memory pool: the chunk list of
  // the packet pass, then the ray sort's buffers.
  const size_t chunk_bytes = (trace_chunk_scratch_bytes(n) + 255) & ~size_t(255);
  char *scratch = nullptr;
  CK(cudaMallocAsync((void **)&scratch, chunk_bytes + (use_sort ? raysort_scratch_bytes(n) : 0), st),
     "trace scratch");
  uint32_t *perm = nullptr;
  RayCells cells;
  const bool beams = use_sort && opts.packet && opts.beam;
  cudaError_t e = use_sort ? launch_raysort(rays, n, nullptr, scratch + chunk_bytes, &perm, st,
                                            beams ? &cells : nullptr)
                           : cudaSuccess;
  if (e == cudaSuccess)
    e = launch_trace(d, rays, n, hits, next_counter(ctx), ctx->d_err, refine, opts, st, perm,
                     reinterpret_cast<uint32_t *>(scratch), beams ? &cells : nullptr);
  cudaFreeAsync(scratch, st);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "trace launch");
  return RT_SUCCESS;
}

rt_status rtTraceClosestHost(rt_ctx *ctx, rt_scene_id id, const rt_ray *h_rays, uint32_t n, rt_hit *h_hits) {
  if (!ctx || (n && (!h_rays || !h_hits))) return RT_ERR_INVALID_ARGUMENT;
  DevScene d;
  {
    std::lock_guard<std::mutex> g(ctx->mu);
    Scene *sc = find_scene(ctx, id);
    if (!sc) return RT_ERR_NOT_FOUND;
    d = sc->dev;
  }
  if (n == 0) return RT_SUCCESS;
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  TraceOpts opts;
  {
    std::lock_guard<std::mutex> g(ctx->mu);
    opts = ctx->trace_opts;
  }
  // Chunks of trace.host_chunk rays alternate between two streams so the
  // copy of one chunk overlaps the traversal of the other. The streams and
  // buffers are this call's own (a lane of the context's pool), so calls
  // from several host threads run side by side.
  const uint32_t chunk = opts.host_chunk;
  const size_t io_bytes = (size_t)chunk * (sizeof(rt_ray) + sizeof(rt_hit));
  const size_t chunk_bytes = (trace_chunk_scratch_bytes(chunk) + 255) & ~size_t(255);
  const size_t need = io_bytes + chunk_bytes + raysort_scratch_bytes(chunk);
  HostLane *lane = nullptr;
  {
    std::lock_guard<std::mutex> g(ctx->mu);
    if (!ctx->idle_lanes.empty()) {
      lane = ctx->idle_lanes.back();
      ctx->idle_lanes.pop_back();
    } else {
      lane = new HostLane();
      ctx->host_lanes.push_back(lane);
    }
  }
  auto give_back = [&] {
    std::lock_guard<std::mutex> g(ctx->mu);
    ctx->idle_lanes.push_back(lane);
  };
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 2 && e == cudaSuccess; i++)
    if (!lane->st[i]) e = cudaStreamCreateWithFlags(&lane->st[i], cudaStreamNonBlocking);
  if (e == cudaSuccess && lane->bytes < need) {
    for (int i = 0; i < 2 && e == cudaSuccess; i++) {
      if (lane->stage[i]) cudaFree(lane->stage[i]);
      lane->stage[i] = nullptr;
      e = cudaMalloc(&lane->stage[i], need);
    }
    lane->bytes = e == cudaSuccess ? need : 0;
  }
  if (e != cudaSuccess) {
    give_back();
    return cuda_fail(ctx, e, "staging allocation");
  }
  for (uint32_t c = 0, k = 0; c < n && e == cudaSuccess; c += chunk, k++) {
    uint32_t m = std::min(chunk, n - c);
    int s = k & 1;
    cudaStream_t st = lane->st[s];
    rt_ray *dr = (rt_ray *)lane->stage[s];
    rt_hit *dh = (rt_hit *)((char *)lane->stage[s] + (size_t)chunk * sizeof(rt_ray));
    e = cudaMemcpyAsync(dr, h_rays + c, sizeof(rt_ray) * m, cudaMemcpyHostToDevice, st);
    uint32_t *perm = nullptr;
    uint32_t *chunks = (uint32_t *)((char *)lane->stage[s] + io_bytes);
    RayCells cells;
    const bool sorted = opts.sort && m >= 65536, beams = sorted && opts.packet && opts.beam;
    if (e == cudaSuccess && sorted)
      e = launch_raysort(dr, m, nullptr, (char *)lane->stage[s] + io_bytes + chunk_bytes, &perm, st,
                         beams ? &cells : nullptr);
    if (e == cudaSuccess)
      e = launch_trace(d, dr, m, dh, next_counter(ctx), ctx->d_err, true, opts, st, perm, chunks,
                       beams ? &cells : nullptr);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_hits + c, dh, sizeof(rt_hit) * m, cudaMemcpyDeviceToHost, st);
  }
  // Wait for everything queued, also after an error, before the lane is
  // handed to another call.
  const cudaError_t e0 = cudaStreamSynchronize(lane->st[0]), e1 = cudaStreamSynchronize(lane->st[1]);
  give_back();
  if (e == cudaSuccess) e = e0 != cudaSuccess ? e0 : e1;
  if (e != cudaSuccess) return cuda_fail(ctx, e, "trace");
  return rtSynchronize(ctx, nullptr);
}

rt_status rtRender(rt_ctx *ctx, rt_scene_id id, const rt_render_params *p, float *accum, void *stream) {
  if (!ctx || !p || !accum) return RT_ERR_INVALID_ARGUMENT;
  if ((uintptr_t)accum % 16) return fail(ctx, RT_ERR_INVALID_ARGUMENT, "image must be 16-byte aligned");
  if (p->width == 0 || p->height == 0 || p->width > 65536 || p->height > 65536)
    return fail(ctx, RT_ERR_INVALID_ARGUMENT, "bad image size %ux%u", p->width, p->height);
  DevScene d;
  rt_camera cam;
  {
    std::lock_guard<std::mutex> g(ctx->mu);
    Scene *sc = find_scene(ctx, id);
    if (!sc) return RT_ERR_NOT_FOUND;
    if (!sc->has_camera) {
      ctx->last_error = "rtRender: no camera set for this scene (rtSetCamera)";
      return RT_ERR_INVALID_ARGUMENT;
    }
    d = sc->dev;
    cam = sc->camera;
  }
  cudaStream_t st = pick_stream(ctx, stream);
  RenderOpts ropts;
  TraceOpts topts;
  {
    std::lock_guard<std::mutex> g(ctx->mu);
    ropts = ctx->render_opts;
    topts = ctx->trace_opts;
  }
  const uint64_t pixels = (uint64_t)p->width * p->height;
  if (use_wavefront(ropts, *p)) {
    void *scratch = nullptr;
    CK(cudaMallocAsync(&scratch, wavefront_scratch_bytes((uint32_t)pixels), st), "wavefront scratch");
    cudaError_t e = launch_render_wavefront(d, cam, *p, accum, ctx->d_segments, next_counter(ctx), ctx->d_err, scratch,
                                            ropts.sort != 0, use_wide(topts, d), st);
    cudaFreeAsync(scratch, st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "render launch");
    return RT_SUCCESS;
  }
  cudaError_t e = launch_render(d, cam, *p, accum, ctx->d_segments, ctx->d_err, st);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "render launch");
  return RT_SUCCESS;
}

// Number of ray segments traced by render calls since the last reset
// (waits for the context stream).
rt_status rtReadSegmentCounter(rt_ctx *ctx, uint64_t *out, int reset) {
  if (!ctx || !out) return RT_ERR_INVALID_ARGUMENT;
  unsigned long long v = 0;
  CK(cudaDeviceSynchronize(), "synchronize");
  CK(cudaMemcpy(&v, ctx->d_segments, sizeof(v), cudaMemcpyDeviceToHost), "read counter");
  if (reset) CK(cudaMemset(ctx->d_segments, 0, sizeof(v)), "reset counter");
  *out = v;
  return RT_SUCCESS;
}

rt_status rtSetTuning(rt_ctx *ctx, const char *key, int64_t value) {
  if (!ctx || !key) return RT_ERR_INVALID_ARGUMENT;
  std::string k(key);
  std::lock_guard<std::mutex> g(ctx->mu);
  if (k == "trace.refill") {
    if (value < 1 || value > 32) return RT_ERR_INVALID_ARGUMENT;
    ctx->trace_opts.refill = (int)value;
    return RT_SUCCESS;
  }
  if (k == "trace.sort") {
    if (value < 0 || value > 1) return RT_ERR_INVALID_ARGUMENT;
    ctx->trace_opts.sort = (int)value;
    return RT_SUCCESS;
  }
  if (k == "trace.packet") {
    if (value < 0 || value > 1) return RT_ERR_INVALID_ARGUMENT;
    ctx->trace_opts.packet = (int)value;
    return RT_SUCCESS;
  }
  if (k == "trace.beam") {
    if (value < 0 || value > 2) return RT_ERR_INVALID_ARGUMENT;
    ctx->trace_opts.beam = (int)value;
    return RT_SUCCESS;
  }
  if (k == "trace.beam_round") {
    if (value < 16 || value > 256) return RT_ERR_INVALID_ARGUMENT;
    ctx->trace_opts.beam_round = (int)value;
    return RT_SUCCESS;
  }
  if (k == "trace.spec") {
    if (value < 0 || value > 1) return RT_ERR_INVALID_ARGUMENT;
    ctx->trace_opts.spec = (int)value;
    return RT_SUCCESS;
  }
  if (k == "trace.minblocks") {
    if (value != 16 && value != 12 && value != 10) return RT_ERR_INVALID_ARGUMENT;
    ctx->trace_opts.minblocks = (int)value;
    return RT_SUCCESS;
  }
  if (k == "trace.packet_minblocks") {
    if (value != 16 && value != 12 && value != 10) return RT_ERR_INVALID_ARGUMENT;
    ctx->trace_opts.packet_minblocks = (int)value;
    return RT_SUCCESS;
  }
  if (k == "trace.host_chunk") {
    if (value < 65536 || value > (1 << 26)) return RT_ERR_INVALID_ARGUMENT;
    ctx->trace_opts.host_chunk = (uint32_t)value;
    return RT_SUCCESS;
  }
  if (k == "trace.defer") {
    if (value < 0 || value > 1) return RT_ERR_INVALID_ARGUMENT;
    ctx->trace_opts.defer = (int)value;
    return RT_SUCCESS;
  }
  if (k == "trace.wide") {
    if (value < 0 || value > 1) return RT_ERR_INVALID_ARGUMENT;
    ctx->trace_opts.wide = (int)value;
    return RT_SUCCESS;
  }
  if (k == "trace.wide_minblocks") {
    if (value < 5 || value > 8) return RT_ERR_INVALID_ARGUMENT;
    ctx->trace_opts.wide_minblocks = (int)value;
    return RT_SUCCESS;
  }
  if (k == "trace.wide_min_tris") {
    if (value < 0 || value > 0xffffffffll) return RT_ERR_INVALID_ARGUMENT;
    ctx->trace_opts.wide_min_tris = (uint32_t)value;
    return RT_SUCCESS;
  }
  if (k == "trace.wide_refill") {
    if (value < 1 || value > 32) return RT_ERR_INVALID_ARGUMENT;
    ctx->trace_opts.wide_refill = (int)value;
    return RT_SUCCESS;
  }
  if (k == "trace.wide_visits") {
    if (value < 1 || value > 3) return RT_ERR_INVALID_ARGUMENT;
    ctx->trace_opts.wide_visits = (int)value;
    return RT_SUCCESS;
  }
  if (k == "render.batch_streams") {
    if (value < 1 || value > 16) return RT_ERR_INVALID_ARGUMENT;
    ctx->render_opts.batch_streams = (int)value;
    return RT_SUCCESS;
  }
  if (k == "render.batch_wavefront_pixels") {
    if (value < 1 || value > (1ll << 31)) return RT_ERR_INVALID_ARGUMENT;
    ctx->render_opts.batch_wavefront_pixels = (uint64_t)value;
    return RT_SUCCESS;
  }
  if (k == "trace.block") {
    if (value != 64 && value != 128 && value != 256) return RT_ERR_INVALID_ARGUMENT;
    ctx->trace_opts.block = (int)value;
    return RT_SUCCESS;
  }
  if (k == "trace.stack") {
    if (value != 0 && value != 16 && value != 32 && value != 64) return RT_ERR_INVALID_ARGUMENT;
    ctx->trace_opts.stack = (int)value;
    return RT_SUCCESS;
  }
  if (k == "render.wavefront_pixels") {
    if (value < 1 || value > (1ll << 31)) return RT_ERR_INVALID_ARGUMENT;
    ctx->render_opts.wavefront_pixels = (uint64_t)value;
    return RT_SUCCESS;
  }
  if (k == "render.mode") {
    if (value < 0 || value > 2) return RT_ERR_INVALID_ARGUMENT;
    ctx->render_opts.mode = (int)value;
    return RT_SUCCESS;
  }
  if (k == "render.sort") {
    if (value < 0 || value > 1) return RT_ERR_INVALID_ARGUMENT;
    ctx->render_opts.sort = (int)value;
    return RT_SUCCESS;
  }
  if (k == "bvh.builder") {
    if (value < 0 || value > 2) return RT_ERR_INVALID_ARGUMENT;
    ctx->build_opts.builder = (int)value;
    return RT_SUCCESS;
  }
  if (k == "bvh.ploc_radius") {
    if (value < 1 || value > 256) return RT_ERR_INVALID_ARGUMENT;
    ctx->build_opts.ploc_radius = (int)value;
    return RT_SUCCESS;
  }
  if (k == "bvh8.collapse") {
    if (value < 0 || value > 1) return RT_ERR_INVALID_ARGUMENT;
    ctx->build_opts.collapse = (int)value;
    return RT_SUCCESS;
  }
  if (k == "bvh.test_error_level") {
    if (value < -1 || value > 64) return RT_ERR_INVALID_ARGUMENT;
    ctx->build_opts.test_error_level = (int)value;
    return RT_SUCCESS;
  }
  ctx->last_error = "rtSetTuning: unknown key " + k;
  return RT_ERR_INVALID_ARGUMENT;
}

rt_status rtGetTuning(rt_ctx *ctx, const char *key, int64_t *value) {
  if (!ctx || !key || !value) return RT_ERR_INVALID_ARGUMENT;
  std::string k(key);
  std::lock_guard<std::mutex> g(ctx->mu);
  if (k == "trace.refill") {
    *value = ctx->trace_opts.refill;
    return RT_SUCCESS;
  }
  if (k == "trace.sort") {
    *value = ctx->trace_opts.sort;
    return RT_SUCCESS;
  }
  if (k == "trace.packet") {
    *value = ctx->trace_opts.packet;
    return RT_SUCCESS;
  }
  if (k == "trace.beam") {
    *value = ctx->trace_opts.beam;
    return RT_SUCCESS;
  }
  if (k == "trace.beam_round") {
    *value = ctx->trace_opts.beam_round;
    return RT_SUCCESS;
  }
  if (k == "trace.spec") {
    *value = ctx->trace_opts.spec;
    return RT_SUCCESS;
  }
  if (k == "trace.minblocks") {
    *value = ctx->trace_opts.minblocks;
    return RT_SUCCESS;
  }
  if (k == "trace.packet_minblocks") {
    *value = ctx->trace_opts.packet_minblocks;
    return RT_SUCCESS;
  }
  if (k == "trace.defer") {
    *value = ctx->trace_opts.defer;
    return RT_SUCCESS;
  }
  if (k == "trace.wide") {
    *value = ctx->trace_opts.wide;
    return RT_SUCCESS;
  }
  if (k == "trace.wide_minblocks") {
    *value = ctx->trace_opts.wide_minblocks;
    return RT_SUCCESS;
  }
  if (k == "trace.wide_min_tris") {
    *value = ctx->trace_opts.wide_min_tris;
    return RT_SUCCESS;
  }
  if (k == "trace.wide_refill") {
    *value = ctx->trace_opts.wide_refill;
    return RT_SUCCESS;
  }
  if (k == "trace.host_chunk") {
    *value = ctx->trace_opts.host_chunk;
    return RT_SUCCESS;
  }
  if (k == "render.mode") {
    *value = ctx->render_opts.mode;
    return RT_SUCCESS;
  }
  if (k == "render.sort") {
    *value = ctx->render_opts.sort;
    return RT_SUCCESS;
  }
  if (k == "trace.block") {
    *value = ctx->trace_opts.block;
    return RT_SUCCESS;
  }
  if (k == "trace.wide_visits") {
    *value = ctx->trace_opts.wide_visits;
    return RT_SUCCESS;
  }
  if (k == "render.batch_streams") {
    *value = ctx->render_opts.batch_streams;
    return RT_SUCCESS;
  }
  if (k == "render.batch_wavefront_pixels") {
    *value = (int64_t)ctx->render_opts.batch_wavefront_pixels;
    return RT_SUCCESS;
  }
  if (k == "trace.stack") {
    *value = ctx->trace_opts.stack;
    return RT_SUCCESS;
  }
  if (k == "render.wavefront_pixels") {
    *value = (int64_t)ctx->render_opts.wavefront_pixels;
    return RT_SUCCESS;
  }
  if (k == "bvh.builder") {
    *value = ctx->build_opts.builder;
    return RT_SUCCESS;
  }
  if (k == "bvh8.collapse") {
    *value = ctx->build_opts.collapse;
    return RT_SUCCESS;
  }
  if (k == "bvh.ploc_radius") {
    *value = ctx->build_opts.ploc_radius;
    return RT_SUCCESS;
  }
  if (k == "bvh.test_error_level") {
    *value = ctx->build_opts.test_error_level;
    return RT_SUCCESS;
  }
  return RT_ERR_INVALID_ARGUMENT;
}

rt_status rtExportImage(rt_ctx *ctx, const float *d_rgba32f, uint32_t width, uint32_t height, float gamma,
                        uint8_t *d_rgba8, void *stream) {
  if (!ctx || !d_rgba32f || !d_rgba8 || !(gamma > 0.0f) || (uintptr_t)d_rgba32f % 16 || (uintptr_t)d_rgba8 % 4)
    return RT_ERR_INVALID_ARGUMENT;
  uint64_t n = (uint64_t)width * height;
  if (n >= (1ull << 32)) return RT_ERR_INVALID_ARGUMENT;
  CK(launch_export(d_rgba32f, (uint32_t)n, gamma, d_rgba8, pick_stream(ctx, stream)), "export");
  return RT_SUCCESS;
}

rt_status rtDenoiseImage(rt_ctx *ctx, const float *d_in, uint32_t width, uint32_t height, float sigma,
                         float ksigma, float threshold, float mix, float *d_out, void *stream) {
  if (!ctx || !d_in || !d_out || d_in == d_out || (uintptr_t)d_in % 16 || (uintptr_t)d_out % 16)
    return RT_ERR_INVALID_ARGUMENT;
  if (!(sigma > 0.0f) || !(ksigma >= 0.0f) || !(threshold > 0.0f) || !(mix >= 0.0f && mix <= 1.0f))
    return fail(ctx, RT_ERR_INVALID_ARGUMENT, "denoise: sigma > 0, kSigma >= 0, threshold > 0, mix in [0,1]");
  if (std::round(ksigma * sigma) > 64.0f) return fail(ctx, RT_ERR_INVALID_ARGUMENT, "denoise: radius above 64");
  if (width > 65536 || height > 65536) return RT_ERR_INVALID_ARGUMENT;
  CK(launch_denoise(d_in, width, height, sigma, ksigma, threshold, mix, d_out, pick_stream(ctx, stream)),
     "denoise");
  return RT_SUCCESS;
}

rt_status rtSynchronize(rt_ctx *ctx, void *stream) {
  if (!ctx) return RT_ERR_INVALID_ARGUMENT;
  CK(cudaStreamSynchronize(pick_stream(ctx, stream)), "synchronize");
  uint32_t bits = 0;
  CK(cudaMemcpy(&bits, ctx->d_err, sizeof(bits), cudaMemcpyDeviceToHost), "read error word");
  if (bits) {
    CK(cudaMemset(ctx->d_err, 0, sizeof(bits)), "reset error word");
    if (bits & KERR_STACK_OVERFLOW) return fail(ctx, RT_ERR_STACK_OVERFLOW, "traversal stack overflow");
    if (bits & KERR_TIMEOUT) return fail(ctx, RT_ERR_TIMEOUT, "device wait timed out");
    return fail(ctx, RT_ERR_INTERNAL, "kernel error bits 0x%x", bits);
  }
  return RT_SUCCESS;
}

}  // extern "C"

namespace rtgb {

bool ctx_scene_dev(rt_ctx *ctx, rt_scene_id id, DevScene *out) {
  std::lock_guard<std::mutex> g(ctx->mu);
  Scene *sc = find_scene(ctx, id);
  if (!sc) return false;
  *out = sc->dev;
  return true;
}
unsigned long long *ctx_segments(rt_ctx *ctx) { return ctx->d_segments; }
uint32_t *ctx_err(rt_ctx *ctx) { return ctx->d_err; }
uint64_t ctx_budget(rt_ctx *ctx) { return ctx->budget; }
int ctx_device(rt_ctx *ctx) { return ctx->device; }
cudaStream_t ctx_stream(rt_ctx *ctx) { return ctx->stream; }
bool ctx_wavefront_render(rt_ctx *ctx, const rt_render_params &p, bool *sort, bool *wide, uint32_t *min_tris) {
  std::lock_guard<std::mutex> g(ctx->mu);
  if (sort) *sort = ctx->render_opts.sort != 0;
  if (wide) *wide = ctx->trace_opts.wide != 0;
  if (min_tris) *min_tris = ctx->trace_opts.wide_min_tris;
  return use_wavefront_batched(ctx->render_opts, p);
}
uint64_t scene_device_bytes(uint32_t nt, uint32_t nm, uint32_t nl, uint32_t ns) {
  return nt ? slab_layout(nt, nm, nl, ns).total : 0;
}

}  // namespace rtgb

// A batch is split by image size: jobs from render.batch_wavefront_pixels up
// (render.mode 2; every job in mode 1, none in mode 0; by default every job)
// run through the wavefront path, spread over side streams, while one
// persistent launch covers the tiles of all other jobs on the caller's
// stream. The two overlap: the small jobs fill the SMs that the wavefront's
// later, shorter bounces leave idle. Every image equals rtRender of its job
// alone.
struct rt_batch {
  BatchJob *d_jobs = nullptr;  // persistent-launch jobs
  uint32_t n = 0, total_tiles = 0, max_depth = 0;
  std::vector<BatchJob> wf;    // wavefront jobs (host copies)
  BatchJob *d_wf = nullptr;    // their device copies: sample_index advances there
  // Wavefront jobs alternate between `sides` side streams (render.batch_streams,
  // at most kSides), each with its own scratch and work counter
  // (counter[64 * (1 + k)]).
  static constexpr int kSides = 16;
  int sides = 0;
  void *wf_scratch[kSides] = {};
  bool wf_sort = false;
  bool wf_wide = true;
  uint32_t wf_wide_min = 0;
  uint32_t *counter = nullptr; // [0] tile counter
  cudaStream_t side[kSides] = {}, capture = nullptr;
  cudaEvent_t fork = nullptr, join[kSides] = {};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

// Validates the jobs and lays out their tiles; fills host BatchJob records.
rt_status make_jobs(rt_ctx *ctx, const rt_render_job *jobs, uint32_t n, std::vector<BatchJob> &out,
                    uint32_t &total_tiles, uint32_t &max_depth) {
  out.resize(n);
  uint64_t tiles = 0;
  max_depth = 1;
  std::lock_guard<std::mutex> g(ctx->mu);
  for (uint32_t j = 0; j < n; j++) {
    const rt_render_job &J = jobs[j];
    Scene *sc = find_scene(ctx, J.scene);
    if (!sc) {
      ctx->last_error = "batch job " + std::to_string(j) + ": scene not found";
      return RT_ERR_NOT_FOUND;
    }
    const rt_render_params &p = J.params;
    if (!J.d_rgba32f || (uintptr_t)J.d_rgba32f % 16 || p.width == 0 || p.height == 0 || p.width > 65536 ||
        p.height > 65536) {
      ctx->last_error = "batch job " + std::to_string(j) + ": bad image or size";
      return RT_ERR_INVALID_ARGUMENT;
    }
    BatchJob &B = out[j];
    B.sc = sc->dev;
    B.cam = J.camera;
    B.p = p;
    B.accum = J.d_rgba32f;
    B.tile_begin = (uint32_t)tiles;
    B.tiles_x = batch_tiles_x(p.width);
    tiles += batch_tiles(p.width, p.height);
    max_depth = std::max(max_depth, sc->dev.depth);
  }
  if (tiles >= (1ull << 32)) {
    ctx->last_error = "batch has too many tiles";
    return RT_ERR_INVALID_ARGUMENT;
  }
  total_tiles = (uint32_t)tiles;
  return RT_SUCCESS;
}

bool wavefront_job(const RenderOpts &o, const rt_render_params &p) { return use_wavefront_batched(o, p); }

cudaError_t batch_enqueue(rt_ctx *ctx, rt_batch *b, cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  const int sides = b->sides;
  if (sides) {
    if ((e = cudaEventRecord(b->fork, st)) != cudaSuccess) return e;
    for (int k = 0; k < sides; k++)
      if ((e = cudaStreamWaitEvent(b->side[k], b->fork, 0)) != cudaSuccess) return e;
    for (size_t j = 0; j < b->wf.size() && e == cudaSuccess; j++) {
      const BatchJob &J = b->wf[j];
      const int k = (int)(j % (size_t)sides);
      e = launch_render_wavefront(J.sc, J.cam, J.p, J.accum, ctx->d_segments, b->counter + 64 * (1 + k), ctx->d_err,
                                  b->wf_scratch[k], b->wf_sort, b->wf_wide && J.sc.ntris >= b->wf_wide_min,
                                  b->side[k], &b->d_wf[j].p.sample_index);
    }
    for (int k = 0; k < sides && e == cudaSuccess; k++) e = cudaEventRecord(b->join[k], b->side[k]);
  }
  if (e == cudaSuccess && b->n)
    e = launch_render_batch(b->d_jobs, b->n, b->total_tiles, b->max_depth, b->counter, ctx->d_segments, ctx->d_err,
                            st);
  for (int k = 0; k < sides && e == cudaSuccess; k++) e = cudaStreamWaitEvent(st, b->join[k], 0);
  return e;
}

cudaError_t batch_advance(rt_batch *b, cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  if (b->n) e = launch_batch_advance(b->d_jobs, b->n, st);
  if (e == cudaSuccess && !b->wf.empty()) e = launch_batch_advance(b->d_wf, (uint32_t)b->wf.size(), st);
  return e;
}

}  // namespace

extern "C" {

rt_status rtBatchCreate(rt_ctx *ctx, const rt_render_job *jobs, uint32_t n_jobs, rt_batch **out) {
  if (!ctx || !out || (n_jobs && !jobs)) return RT_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  std::vector<BatchJob> host;
  uint32_t total = 0, depth = 1;
  rt_status s = make_jobs(ctx, jobs, n_jobs, host, total, depth);
  if (s != RT_SUCCESS) return s;
  RenderOpts ropts;
  TraceOpts topts;
  {
    std::lock_guard<std::mutex> g(ctx->mu);
    ropts = ctx->render_opts;
    topts = ctx->trace_opts;
  }
  // Split, then lay the persistent jobs' tiles out again without the others.
  std::vector<BatchJob> tiles_jobs;
  rt_batch *b = new rt_batch();
  uint64_t tiles = 0;
  uint32_t max_wf = 0;
  b->max_depth = 1;
  for (const BatchJob &J : host) {
    if (wavefront_job(ropts, J.p)) {
      b->wf.push_back(J);
      max_wf = std::max(max_wf, J.p.width * J.p.height);
    } else {
      BatchJob T = J;
      T.tile_begin = (uint32_t)tiles;
      tiles += batch_tiles(J.p.width, J.p.height);
      b->max_depth = std::max(b->max_depth, J.sc.depth);
      tiles_jobs.push_back(T);
    }
  }
  (void)total;
  (void)depth;
  b->n = (uint32_t)tiles_jobs.size();
  b->total_tiles = (uint32_t)tiles;
  b->wf_sort = ropts.sort != 0;
  b->wf_wide = topts.wide != 0;
  b->wf_wide_min = topts.wide_min_tris;
  cudaError_t e = cudaMalloc((void **)&b->d_jobs, sizeof(BatchJob) * std::max(b->n, 1u));
  if (e == cudaSuccess) e = cudaMalloc((void **)&b->counter, 256 * (1 + rt_batch::kSides));
  if (e == cudaSuccess && b->n)
    e = cudaMemcpy(b->d_jobs, tiles_jobs.data(), sizeof(BatchJob) * b->n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !b->wf.empty()) {
    e = cudaMalloc((void **)&b->d_wf, sizeof(BatchJob) * b->wf.size());
    if (e == cudaSuccess)
      e = cudaMemcpy(b->d_wf, b->wf.data(), sizeof(BatchJob) * b->wf.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    const int sides =
        (int)std::min<size_t>(b->wf.size(), (size_t)std::clamp(ropts.batch_streams, 1, rt_batch::kSides));
    b->sides = sides;
    for (int k = 0; k < sides && e == cudaSuccess; k++) {
      e = cudaMalloc(&b->wf_scratch[k], wavefront_scratch_bytes(max_wf));
      if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->side[k], cudaStreamNonBlocking);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming);
    }
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    rtBatchDestroy(ctx, b);
    return cuda_fail(ctx, e, "batch creation");
  }
  *out = b;
  return RT_SUCCESS;
}

rt_status rtBatchDestroy(rt_ctx *ctx, rt_batch *b) {
  if (!ctx || !b) return RT_ERR_INVALID_ARGUMENT;
  cudaDeviceSynchronize();
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->capture) cudaStreamDestroy(b->capture);
  for (int k = 0; k < rt_batch::kSides; k++) {
    if (b->side[k]) cudaStreamDestroy(b->side[k]);
    if (b->join[k]) cudaEventDestroy(b->join[k]);
    if (b->wf_scratch[k]) cudaFree(b->wf_scratch[k]);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->d_jobs) cudaFree(b->d_jobs);
  if (b->d_wf) cudaFree(b->d_wf);
  if (b->counter) cudaFree(b->counter);
  delete b;
  return RT_SUCCESS;
}

rt_status rtBatchLaunch(rt_ctx *ctx, rt_batch *b, void *stream) {
  if (!ctx || !b) return RT_ERR_INVALID_ARGUMENT;
  CK(batch_enqueue(ctx, b, pick_stream(ctx, stream)), "batch launch");
  return RT_SUCCESS;
}

rt_status rtBatchAdvance(rt_ctx *ctx, rt_batch *b, void *stream) {
  if (!ctx || !b) return RT_ERR_INVALID_ARGUMENT;
  CK(batch_advance(b, pick_stream(ctx, stream)), "batch advance");
  return RT_SUCCESS;
}

rt_status rtBatchLaunchGraph(rt_ctx *ctx, rt_batch *b, void *stream) {
  if (!ctx || !b) return RT_ERR_INVALID_ARGUMENT;
  if (!b->exec) {
    CK(cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal), "graph capture");
    cudaError_t e = batch_enqueue(ctx, b, b->capture);
    if (e == cudaSuccess) e = batch_advance(b, b->capture);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(b->capture, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return cuda_fail(ctx, e != cudaSuccess ? e : e2, "graph capture");
    }
    b->graph = g;
    CK(cudaGraphInstantiate(&b->exec, b->graph, 0), "graph instantiate");
  }
  CK(cudaGraphLaunch(b->exec, pick_stream(ctx, stream)), "graph launch");
  return RT_SUCCESS;
}

rt_status rtRenderBatch(rt_ctx *ctx, const rt_render_job *jobs, uint32_t n_jobs, void *stream) {
  if (!ctx || (n_jobs && !jobs)) return RT_ERR_INVALID_ARGUMENT;
  if (n_jobs == 0) return RT_SUCCESS;
  rt_batch *b = nullptr;
  rt_status s = rtBatchCreate(ctx, jobs, n_jobs, &b);
  if (s != RT_SUCCESS) return s;
  cudaStream_t st = pick_stream(ctx, stream);
  cudaError_t e = batch_enqueue(ctx, b, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  rtBatchDestroy(ctx, b);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "batch launch");
  return RT_SUCCESS;
}

}  // extern "C"
