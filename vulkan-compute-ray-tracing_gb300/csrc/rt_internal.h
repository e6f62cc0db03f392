// Internal declarations shared by the host runtime (api.cpp) and the kernel
// translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "rtgb/rt_api.h"
#include "rtgb/rt_types.h"

namespace rtgb {

// Error bits kernels record in the context's device error word.
enum : uint32_t {
  KERR_STACK_OVERFLOW = 1u,
  KERR_BAD_INDEX = 2u,
  KERR_TIMEOUT = 4u,
};

// Device-resident scene, as the kernels see it.
//
// Reference layout (kept for parity downloads, light sampling and materials):
//   tris    rt_triangle[ntris]   48 B
//   nodes   rt_bvh_node[nnodes]  48 B, nnodes = 2*ntris - 1
// Traversal layout (derived on the GPU from `nodes`):
//   bvh2    4 x float4 per inner node (64 B): one 32-byte record per
//           child, (lo.x, lo.y, hi.x, hi.y) then (lo.z, hi.z, ref, order)
//           (pairs for the packed slab FMAs). ref >= 0 is an inner node,
//           ref < 0 is the leaf ~k whose triangle is tpre[k]; bit o of
//           `order` (the same in both records) set: child 1 is visited
//           first by rays of sign octant o.
//   tpre    3 x float4 per triangle in leaf order (48 B): v0, n = cross(b, a),
//           a = v0 - v1, b = v2 - v0 — the per-triangle terms of triIntersect
//           (ray-trace-compute.comp:157-173), computed once with the same
//           rounding.
//   leaf_tri  original triangle index of leaf k.
//   bvh8    the same tree with levels folded into nodes of up to eight
//           children (bvh8.cu), 96 B per node: origin, per-axis exponents
//           and the filled-slot mask, 8-bit child bounds rounded outward,
//           child refs; slots assigned by octant so that a ray meets the
//           children in about the order s ^ (its direction's sign bits);
//           breadth-first numbered, root node 0; inner refs are node
//           numbers, leaf refs the bvh2 ones (~k). Used by the per-lane
//           8-wide caster.
struct DevScene {
  const rt_triangle *tris;
  const rt_material *mats;
  const rt_light *lights;
  const rt_sphere *spheres;
  const rt_bvh_node *nodes;
  const float4 *bvh2;
  const float4 *tpre;
  const int32_t *leaf_tri;
  float root_lo[3];
  float root_hi[3];
  int32_t root_ref;
  uint32_t ntris, nmats, nlights, nspheres, nnodes;
  uint32_t depth;
  const float4 *bvh8;
  uint32_t n8, levels8;  // bvh8 nodes and levels (0 when absent)
  int32_t root8;         // the bvh8 root node (0)
  // 1 when the tree is Bvh.h's median-split tree (built here or given by
  // the caller), whose overlapping boxes favour beams (trace.beam 2).
  uint32_t median_tree;
};

// ---------------------------------------------------------------- bvh8.cu
// Node capacity the collapse may need for `ntris` leaves: (4n - 1) / 7 + 1.
uint32_t bvh8_capacity(uint32_t ntris);
// Folds d.bvh2 into quantized bvh8 nodes (96 B each, capacity `cap`
// nodes), choosing the folded pairs by the SAH (`sah`) or largest child
// first; synchronises `st`.
constexpr size_t kBvh8NodeBytes = 96;
cudaError_t build_bvh8(const DevScene &d, bool sah, void *bvh8q, uint32_t cap, uint32_t *n8_out,
                       uint32_t *levels_out, int32_t *root_out, char *errbuf, size_t errlen, cudaStream_t st);

// ---------------------------------------------------------------- relayout.cu
// Exclusive scan of n words (in may equal out); `sums` needs ceil(n/1024).
cudaError_t exclusive_scan_u32(const uint32_t *in, uint32_t *out, uint32_t *sums, uint32_t n, cudaStream_t st);
// Derives bvh2 / tpre / leaf_tri from the reference node array. `scratch`
// holds 2*nnodes uint32 words.
cudaError_t launch_relayout(const rt_bvh_node *nodes, uint32_t nnodes, const rt_triangle *tris, float4 *bvh2,
                            float4 *tpre, int32_t *leaf_tri, uint32_t *scratch, cudaStream_t st);

// ---------------------------------------------------------------- trace.cu
// Launch-shape knobs of closest-hit casting (rtSetTuning).
struct TraceOpts {
  int refill = 32;  // idle lanes per warp that trigger a fetch of new rays (32: whole-warp batches)
  int sort = 1;     // 1: cast rays in Morton order of origin and direction (raysort.cu)
  int packet = 1;   // 1: warps of coherent rays traverse as one packet (traverse_packet)
  int beam = 0;     // sorted one-origin batches traverse the sort's cell tiles as beams (beam.cuh):
                    // 1 always, 0 never, 2 on Bvh.h's median-split trees (DevScene::median_tree)
  int beam_round = 64;  // leaves a beam round collects before its rays test them (16..256)
  int spec = 1;     // 1: per-lane traversal parks leaves until the whole warp holds one (traverse_spec)
  int minblocks = 12;  // resident 128-thread blocks per SM the per-lane caster is compiled for (16, 12 or 10)
  int packet_minblocks = 12;  // the same for the packet caster
  int defer = 1;    // 1: chunks that fail the packet test go to the per-lane kernel; 0: traced in place
  int wide = 1;     // 1: per-lane chunks are cast over bvh8 with a warp leaf pool (k_trace_wide)
  int wide_minblocks = 6;  // resident 128-thread blocks per SM k_trace_wide is compiled for (8, 6 or 5)
  int wide_refill = 4;     // idle lanes of a k_trace_wide warp that trigger a fetch of new rays (1..32)
  int wide_visits = 3;     // node steps per lane per k_trace_wide loop iteration (1..3)
  uint32_t wide_min_tris = 0;  // scenes from this many triangles up use the 8-wide caster
  uint32_t host_chunk = 1u << 21;  // rays per pipelined chunk of rtTraceClosestHost
  int block = 128;  // threads per block of the casting kernels (64, 128 or 256)
  int stack = 0;    // traversal stack entries (16, 32 or 64; 0: the smallest that holds the tree)
};

// Stack entries a cast of this scene runs with: trace.stack raised to the
// smallest of 16, 32, 64 that holds the tree (binary depth for the packet
// and per-lane kernels; the 8-wide caster's group stack needs its levels).
inline int trace_stack_entries(const TraceOpts &o, const DevScene &sc) {
  const int need = sc.depth <= 16 ? 16 : (sc.depth <= 32 ? 32 : 64);
  return o.stack > need ? (o.stack <= 32 ? 32 : 64) : need;
}

// `counter` is a device word private to this launch (work distribution);
// `refine` recomputes t, u, v of the winning triangle in fp64.
// `perm` (may be NULL) gives the order rays are cast in; hits always land
// at their ray's input index.
// chunk_scratch holds trace_chunk_scratch_bytes(n) (the packet pass's list of
// chunks left for the per-lane pass); without it packets are not used.
// `cells` (with perm, from the same sort) lets one-origin batches be cast
// as beams over the sort's cell tiles (trace.beam).
struct RayCells;
cudaError_t launch_trace(const DevScene &sc, const rt_ray *rays, uint32_t n, rt_hit *hits, uint32_t *counter,
                         uint32_t *err, bool refine, const TraceOpts &opts, cudaStream_t st,
                         const uint32_t *perm = nullptr, uint32_t *chunk_scratch = nullptr,
                         const RayCells *cells = nullptr);
size_t trace_chunk_scratch_bytes(uint32_t n);
// The 8-wide caster over listed 32-ray chunks of a device-sized queue
// (*d_n rays, at most cap), writing (leaf k, t) hits; wide_ok tells whether
// the scene's bvh8 can take it.
bool wide_ok(const DevScene &sc);
inline bool use_wide(const TraceOpts &o, const DevScene &sc) {
  return o.wide && sc.ntris >= o.wide_min_tris && wide_ok(sc);
}
cudaError_t launch_wide_leaf(const DevScene &sc, const rt_ray *rays, uint32_t cap, const uint32_t *d_n,
                             const uint32_t *perm, const uint32_t *list, const uint32_t *list_count, int2 *hits,
                             uint32_t *counter, uint32_t *err, int minblocks, int refill, cudaStream_t st);
// Morton bucketing of a ray batch (raysort.cu); `scratch` holds
// raysort_scratch_bytes(n); *perm_out points into it.
size_t raysort_scratch_bytes(uint32_t n);
// The sorted batch cut at cells of 64 Morton buckets (8 x 8 direction
// buckets when the batch has one origin), each cell into tiles of at most
// 256 rays: tiles[2t], tiles[2t + 1] = first and one-past-last sorted
// position of tile t, t < *count. ext[0..4] / ext[5..9]: ordered minima /
// maxima of the key coordinates (origin x, y, z, octahedral u, v) over the
// sampled rays. All device pointers into the sort's scratch.
struct RayCells {
  const uint32_t *ext = nullptr;
  const uint32_t *tiles = nullptr;
  const uint32_t *count = nullptr;
};
// With d_n != NULL only the first *d_n of the n rays are sorted. With
// `cells`, the cell tiles are listed too (not with d_n).
cudaError_t launch_raysort(const rt_ray *rays, uint32_t n, const uint32_t *d_n, void *scratch, uint32_t **perm_out,
                           cudaStream_t st, RayCells *cells = nullptr);
// The shader-literal 16-entry-stack traversal over the Bvh.h node array.
cudaError_t launch_trace_literal16(const DevScene &sc, const rt_ray *rays, uint32_t n, rt_hit *hits,
                                   cudaStream_t st);

// ---------------------------------------------------------------- render.cu
// `segments` (may be NULL) accumulates the number of traced ray segments.
cudaError_t launch_render(const DevScene &sc, const rt_camera &cam, const rt_render_params &p, float *accum,
                          unsigned long long *segments, uint32_t *err, cudaStream_t st);

// Wavefront render (wavefront.cu): same images as launch_render; `scratch`
// holds wavefront_scratch_bytes(width*height); `counter` is a launch-private
// device word. With d_sample_index the kernels read the first sample index
// from the device at run time instead of p.sample_index.
size_t wavefront_scratch_bytes(uint32_t cap);
// `wide`: bounce rays that fail the packet test are cast by the 8-wide
// caster (launch_wide_leaf) instead of in place.
cudaError_t launch_render_wavefront(const DevScene &sc, const rt_camera &cam, const rt_render_params &p, float *accum,
                                    unsigned long long *segments, uint32_t *counter, uint32_t *err, void *scratch,
                                    bool sort, bool wide, cudaStream_t st,
                                    const uint32_t *d_sample_index = nullptr);

// Render launch-shape knobs (rtSetTuning "render.mode").
struct RenderOpts {
  int mode = 2;                         // 0 megakernel, 1 wavefront, 2 choose by image size
  uint64_t wavefront_pixels = 1u << 18;  // mode 2: wavefront from this many pixels up
  int batch_streams = 16;                // side streams a batch spreads its wavefront jobs over (1..16)
  // Batches and the render server: jobs from this many pixels up run as
  // wavefronts on side streams (the rest in the persistent tile launch).
  // Jobs that run side by side keep the GPU busy at any size, and queued
  // bounce rays in the 8-wide caster beat the megakernel's diverged lanes,
  // so all of them do by default; a render alone keeps wavefront_pixels.
  uint64_t batch_wavefront_pixels = 1;
  // Wavefront renders: reorder each bounce's rays by Morton key of origin and
  // direction before casting them (1) or cast them in queue order (0). The
  // queue keeps the shading warps' order, which is close to the camera
  // tiles' order, and the 8-wide caster takes them faster unsorted; the
  // closest-hit entry points keep trace.sort.
  int sort = 0;
};
// True when a render of these params goes to the wavefront kernels.
inline bool use_wavefront(const RenderOpts &o, const rt_render_params &p) {
  if (p.flags & RT_COMPAT_STACK16) return false;  // the literal 16-entry traversal is megakernel-only
  const uint64_t pixels = (uint64_t)p.width * p.height;
  return pixels < (1ull << 31) && (o.mode == 1 || (o.mode == 2 && pixels >= o.wavefront_pixels));
}
// True when a job of a batch or a server step goes to the wavefront kernels.
inline bool use_wavefront_batched(const RenderOpts &o, const rt_render_params &p) {
  RenderOpts b = o;
  b.wavefront_pixels = o.batch_wavefront_pixels;
  return use_wavefront(b, p);
}

// Tree used when a scene is uploaded without nodes (rtSetTuning "bvh.builder").
struct BuildOpts {
  int builder = 0;  // 0 the reference's Bvh.h tree (bit-exact), 1 LBVH, 2 PLOC
  int collapse = 1;  // 8-wide fold: 1 SAH-chosen pairs, 0 largest child first ("bvh8.collapse")
  int ploc_radius = 16;  // PLOC's nearest-neighbour search radius ("bvh.ploc_radius")
  int test_error_level = -1;  // test hook of gpu_build_bvh's error word (-1: off)
};

// One job of a batched render (render.cu: k_render_batch).
struct BatchJob {
  DevScene sc;
  rt_camera cam;
  rt_render_params p;
  float *accum;
  uint32_t tile_begin;  // first tile of this job in the batch's tile space
  uint32_t tiles_x;     // tiles per image row
};
uint32_t batch_tiles_x(uint32_t width);
uint32_t batch_tiles(uint32_t width, uint32_t height);
// d_jobs sorted by tile_begin; max_depth = deepest BVH among the jobs.
cudaError_t launch_render_batch(const BatchJob *d_jobs, uint32_t n_jobs, uint32_t total_tiles, uint32_t max_depth,
                                uint32_t *counter, unsigned long long *segments, uint32_t *err, cudaStream_t st);
// sample_index += spp for every job (the next progressive frame).
cudaError_t launch_batch_advance(BatchJob *d_jobs, uint32_t n_jobs, cudaStream_t st);

// ---------------------------------------------------------------- bvh_build.cu
// Builds the Bvh.h node array on the GPU. `axes` holds rand() % 3 for every
// node in pop order (2*n - 1 values, host-generated from glibc's rand()).
// test_error_level >= 0 (a test hook, "bvh.test_error_level") records an
// error bit after that level's sort, as an overflow would; the build must
// then fail with RT_ERR_INTERNAL.
rt_status gpu_build_bvh(const rt_triangle *d_tris, uint32_t n, const uint8_t *h_axes, rt_bvh_node *d_nodes,
                        cudaStream_t st, float *ms_out, uint32_t *depth_out, char *errbuf, size_t errlen,
                        int test_error_level = -1);

// ---------------------------------------------------------------- export.cu
cudaError_t launch_export(const float *in, uint32_t n, float gamma, uint8_t *out, cudaStream_t st);
// smartDeNoise over an RGBA32F image (denoise.cu); in and out must not alias.
cudaError_t launch_denoise(const float *in, uint32_t W, uint32_t H, float sigma, float ksigma, float threshold,
                           float mix, float *out, cudaStream_t st);

// ---------------------------------------------------------------- api.cpp
// Context internals for the serving layer (serve.cpp).
bool ctx_scene_dev(rt_ctx *ctx, rt_scene_id id, DevScene *out);
unsigned long long *ctx_segments(rt_ctx *ctx);
uint32_t *ctx_err(rt_ctx *ctx);
uint64_t ctx_budget(rt_ctx *ctx);
int ctx_device(rt_ctx *ctx);
cudaStream_t ctx_stream(rt_ctx *ctx);
// True when a batch or a server step gives a job of these params to the
// wavefront kernels (render.mode 1, or 2 and at least
// render.batch_wavefront_pixels; never the 16-entry compat traversal);
// *sort receives render.sort (the per-bounce reordering).
bool ctx_wavefront_render(rt_ctx *ctx, const rt_render_params &p, bool *sort, bool *wide = nullptr,
                          uint32_t *min_tris = nullptr);
// Device bytes rtUploadScene allocates for a scene of these counts.
uint64_t scene_device_bytes(uint32_t n_triangles, uint32_t n_materials, uint32_t n_lights, uint32_t n_spheres);

// ---------------------------------------------------------------- lbvh.cu
// A linear BVH (Morton order) in the Bvh.h node layout; not the reference's
// tree — a separately reported traversal mode.
rt_status gpu_build_lbvh(const rt_triangle *d_tris, uint32_t n, rt_bvh_node *d_nodes, cudaStream_t st, float *ms_out,
                         uint32_t *depth_out, char *errbuf, size_t errlen);
// Morton-sorted triangle centroids (lbvh.cu), shared by the LBVH and PLOC builders.
size_t lbvh_sorted_keys_words(uint32_t n);
cudaError_t lbvh_sorted_keys(const rt_triangle *d_tris, uint32_t n, uint32_t *scratch, uint32_t **codes_out,
                             uint32_t **idx_out, cudaStream_t st);
// Agglomerative-clustering tree (ploc.cu), Bvh.h node layout, root node 0;
// nearest neighbours searched within `radius` (1..256) positions.
rt_status gpu_build_ploc(const rt_triangle *d_tris, uint32_t n, uint32_t radius, rt_bvh_node *d_nodes,
                         cudaStream_t st, float *ms_out, uint32_t *depth_out, char *errbuf, size_t errlen);

// ---------------------------------------------------------------- glibc_rand.cpp
// glibc's TYPE_3 random() (what rand() returns) after srand(seed).
void glibc_rand_axes(uint32_t seed, uint64_t count, uint8_t *out_mod3);
void glibc_rand_values(uint32_t seed, uint64_t count, int32_t *out);

}  // namespace rtgb
