/*
 * rt_api.h — the C ABI of the GB300 ray-trace hot path.
 *
 * In the reference, the path is a Vulkan compute "material": a pipeline plus
 * a descriptor set whose bindings are filled in add-order (UBO, target image,
 * accumulation image, triangles, materials, BVH nodes, lights, spheres;
 * src/main.cpp:144-153), dispatched once per frame
 * (src/scene/ComputeModel.cpp:21-25, src/main.cpp:228) with a UBO update per
 * frame (src/main.cpp:166-183). Errors are C++ exceptions
 * (src/scene/ComputeMaterial.cpp:37,57; caught in src/main.cpp:449-457).
 *
 * Here the same path is a context (device + stream + scene registry), scenes
 * uploaded once and kept resident in HBM, and stream-ordered render / trace
 * calls. Every function returns an rt_status; no C++ exception crosses the
 * ABI. Device pointers are plain CUDA device pointers; `stream` is a
 * cudaStream_t passed as void* (NULL = the context's own stream).
 *
 * Threading: one context may be used from several host threads; the scene
 * registry is locked internally. Calls on one stream execute in order.
 */
#ifndef RTGB_RT_API_H
#define RTGB_RT_API_H

#include <stddef.h>
#include <stdint.h>
#include "rt_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef enum rt_status {
  RT_SUCCESS = 0,
  RT_ERR_INVALID_ARGUMENT = 1,
  RT_ERR_OUT_OF_MEMORY = 2,
  RT_ERR_CUDA = 3,
  RT_ERR_NOT_FOUND = 4,
  RT_ERR_INVALID_SCENE = 5,
  RT_ERR_STACK_OVERFLOW = 6,
  RT_ERR_TIMEOUT = 7,
  RT_ERR_BUDGET = 8,
  RT_ERR_BUSY = 9,
  RT_ERR_INTERNAL = 10
} rt_status;

typedef struct rt_ctx rt_ctx;
typedef uint32_t rt_scene_id;

typedef struct rt_ctx_desc {
  int device;                /* CUDA device ordinal */
  uint64_t hbm_budget_bytes; /* resident-scene budget; 0 = 80% of free HBM */
  uint32_t flags;            /* reserved, 0 */
  uint32_t _reserved;
} rt_ctx_desc;

typedef struct rt_scene_info {
  uint32_t triangles, materials, lights, spheres, nodes;
  uint32_t depth;           /* levels of the BVH (root = 1) */
  uint64_t device_bytes;    /* HBM held by the scene */
  float build_ms;           /* GPU BVH build time (0 when nodes were uploaded) */
  float relayout_ms;        /* traversal-layout build time */
} rt_scene_info;

/* Replaces VulkanApplicationContext + ComputeMaterial::init
 * (src/app-context/VulkanApplicationContext.cpp:7-181,
 *  src/scene/ComputeMaterial.cpp:15-26): device, stream and pipeline state. */
rt_status rtCreate(rt_ctx **ctx, const rt_ctx_desc *desc);
rt_status rtDestroy(rt_ctx *ctx);

/* Last error message of the context (thread-safe copy held by the context);
 * replaces the std::runtime_error text of the reference. */
const char *rtGetLastError(rt_ctx *ctx);
const char *rtStatusString(rt_status s);

/* Replaces GpuModel::Scene (src/ray-tracing/RtScene.h:44-101) plus the five
 * storage-buffer bundles bound at bindings 3-7 (src/main.cpp:88-106,148-152).
 * Host arrays in the reference's std430 layouts are validated (finite
 * vertices, indices in range, material types 0-3), copied to HBM and owned
 * by the context afterwards.
 *   nodes == NULL : the BVH is built on the GPU, node-for-node identical to
 *                   Bvh::createBvh (src/ray-tracing/Bvh.h:141-209) run in a
 *                   fresh process whose rand() was seeded with `bvh_seed`
 *                   (the reference never seeds: 1).
 *   nodes != NULL : a node array in the Bvh.h layout is uploaded as is
 *                   (it must be a full binary tree rooted at node 0).
 *   lights == NULL: the light list is derived from LightSource materials as
 *                   RtScene.h:87-96 does (area = |v0 x v1| / 2).
 * The traversal layout (children-pair nodes and triangles in leaf order) is
 * derived on the GPU. The call returns when the scene is resident. */
rt_status rtUploadScene(rt_ctx *ctx, const rt_triangle *triangles, uint32_t n_triangles,
                        const rt_material *materials, uint32_t n_materials, const rt_bvh_node *nodes,
                        uint32_t n_nodes, const rt_light *lights, uint32_t n_lights, const rt_sphere *spheres,
                        uint32_t n_spheres, uint32_t bvh_seed, rt_scene_id *out);
rt_status rtReleaseScene(rt_ctx *ctx, rt_scene_id scene);
rt_status rtGetSceneInfo(rt_ctx *ctx, rt_scene_id scene, rt_scene_info *out);

/* Copies the scene's BVH back in the Bvh.h node layout (n = 2*triangles-1). */
rt_status rtDownloadBvh(rt_ctx *ctx, rt_scene_id scene, rt_bvh_node *host_out, uint32_t n);
/* Copies the scene's light list back (n = info.lights). */
rt_status rtDownloadLights(rt_ctx *ctx, rt_scene_id scene, rt_light *host_out, uint32_t n);

/* Light list of RtScene.h:87-96 computed on the host (no GPU). Returns the
 * number of lights; `out` may be NULL to count. */
uint32_t rtLightsFromMaterials(const rt_triangle *triangles, uint32_t n, const rt_material *materials,
                               uint32_t n_materials, rt_light *out);

/* The UBO camera (ubo.camPos, src/main.cpp:39-47,174) as the shader turns it
 * into rays (ray-trace-compute.comp:357-372: vfov 30, looks down -z, zxy
 * swizzle). */
rt_status rtCameraFromReference(const float cam_pos[3], uint32_t width, uint32_t height, rt_camera *out);
/* A general pinhole: eye, target, up, vertical field of view in degrees;
 * image row 0 is the top row. */
rt_status rtCameraLookAt(const float eye[3], const float target[3], const float up[3], float vfov_deg,
                         uint32_t width, uint32_t height, rt_camera *out);
/* Stores the camera used by rtRender for this scene (the per-frame UBO
 * write of src/main.cpp:174-180). */
rt_status rtSetCamera(rt_ctx *ctx, rt_scene_id scene, const rt_camera *camera);

/* One progressive render call: replaces ComputeModel::computeCommand
 * (src/scene/ComputeModel.cpp:21-25) and the target->accumulation image copy
 * (src/main.cpp:253-261). Accumulates params->spp samples per pixel into
 * the caller's RGBA32F device image (width*height*4 floats, row-major) as a
 * running mean starting at sample params->sample_index (0 resets), tracing
 * params->max_bounces bounces per path. Stream-ordered. */
rt_status rtRender(rt_ctx *ctx, rt_scene_id scene, const rt_render_params *params, float *d_rgba32f,
                   void *stream);

/* Display epilogue of the reference's post-process shader
 * (resources/shaders/source/post-process-shader.frag:62-68): each pixel of
 * the RGBA32F image becomes pow(rgb, 1/gamma) with alpha 1, rounded to
 * 8 bits per channel (clamped to [0,1]), into a device RGBA8 buffer of
 * width*height*4 bytes. The reference uses gamma 2.2. Stream-ordered. */
rt_status rtExportImage(rt_ctx *ctx, const float *d_rgba32f, uint32_t width, uint32_t height, float gamma,
                        uint8_t *d_rgba8, void *stream);

/* smartDeNoise, the edge-preserving filter the reference's post-process
 * shader defines (post-process-shader.frag:26-68) and leaves switched off
 * (frag:73 would blend it 50/50 with the unfiltered image, sigma 2, kSigma 2,
 * threshold 0.05): out = mix * filtered + (1 - mix) * in, per RGBA32F pixel.
 * Circular kernel of radius round(kSigma * sigma) <= 64 with fractional row
 * offsets, spatial Gaussian (sigma) times range Gaussian (threshold) weights,
 * taps fetched bilinearly with the reference sampler's REPEAT wrap
 * (src/memory/Image.cpp:353-357). d_in and d_out must not alias. */
rt_status rtDenoiseImage(rt_ctx *ctx, const float *d_in, uint32_t width, uint32_t height, float sigma,
                         float ksigma, float threshold, float mix, float *d_out, void *stream);

/* Closest-hit casting for a device batch of rays (the hit_bvh loop of
 * ray-trace-compute.comp:262-311 as a stand-alone query). Stream-ordered. */
rt_status rtTraceClosest(rt_ctx *ctx, rt_scene_id scene, const rt_ray *d_rays, uint32_t n, rt_hit *d_hits,
                         void *stream);
/* rtTraceClosest with flags: RT_COMPAT_STACK16 replays the shader's 16-entry
 * stack (comp:262,280), including its silent truncation; RT_HIT_FP32 returns
 * t, u, v exactly as the fp32 triIntersect computes them instead of the
 * default fp64 re-evaluation of the winning triangle. The hit index is the
 * same either way. */
rt_status rtTraceClosestEx(rt_ctx *ctx, rt_scene_id scene, const rt_ray *d_rays, uint32_t n, rt_hit *d_hits,
                           uint32_t flags, void *stream);
/* The same with host arrays: copies in, traces and copies out in pipelined
 * chunks; returns when h_hits is filled. Pinned host memory gives
 * asynchronous DMA. Each call uses its own streams and device staging
 * (from a pool of the context), so calls from several host threads on one
 * context run side by side. */
rt_status rtTraceClosestHost(rt_ctx *ctx, rt_scene_id scene, const rt_ray *h_rays, uint32_t n, rt_hit *h_hits);

/* Launch-shape knobs of the context (the reference fixes its launch at
 * compile time: local size 32x32, comp:3). Keys:
 *   "trace.refill"  idle lanes of a warp that trigger a fetch of new rays
 *                   in closest-hit casting (1..32; 32 = refill whole warps)
 *   "trace.sort"    1 (default) = cast batches of >= 65536 rays in Morton
 *                   order of origin and direction (hits still land at their
 *                   ray's input index; scratch comes from the stream-ordered
 *                   pool)
 *   "trace.packet"  1 (default) = a warp whose 32 rays share an origin and
 *                   point within ~18 degrees traverses them as one packet
 *                   (one node sequence, every lane busy); 0 = always one
 *                   traversal per lane. Results are identical either way
 *   "trace.beam"    1 = sorted batches of one origin are cast in tiles of up
 *                   to 256 rays (the sort's Morton cells) that walk the tree
 *                   once as a beam: the block expands the tile's cone, the
 *                   rays test the leaves it meets (each with its own slab
 *                   test first); 0 (default) = warp packets; 2 = beams on
 *                   Bvh.h's median-split tree (bvh.builder 0 or the caller's
 *                   nodes), whose overlapping boxes favour them, packets on
 *                   the LBVH and PLOC trees. Results are identical either way
 *   "trace.beam_round"  leaves a beam collects before its rays test them
 *                   (16..256, default 64)
 *   "trace.spec"    1 (default) = per-lane traversal parks the first leaf it
 *                   reaches and keeps descending until every lane of the
 *                   warp holds one, then tests them together; 0 = test each
 *                   leaf when reached. Results are identical either way
 *   "trace.minblocks" 16, 12 (default) or 10: resident 128-thread blocks per
 *                   SM the per-lane caster is compiled for (register budget)
 *   "trace.packet_minblocks"  the same for the packet caster (default 12)
 *   "trace.host_chunk"  rays per pipelined chunk of rtTraceClosestHost
 *                   (65536 .. 2^26, default 2^21)
 *   "trace.defer"   1 (default) = 32-ray chunks that fail the packet test are
 *                   listed and cast by a second, per-lane kernel; 0 = cast
 *                   in place by the packet kernel with plain per-lane
 *                   traversal (no postponed leaves)
 *   "trace.wide"    1 (default) = rays of the per-lane kernel (chunks that
 *                   fail the packet test) are cast over the scene's 8-wide
 *                   fold of the same tree: each step tests all eight child
 *                   boxes of a node, and leaves are tested 32 at a time by
 *                   the whole warp from a shared pool; 0 = the binary layout
 *                   with postponed leaves. Results are identical either way
 *   "trace.wide_minblocks" 8, 7, 6 (default) or 5: resident 128-thread blocks
 *                   per SM the 8-wide caster is compiled for
 *   "trace.wide_refill"  idle lanes of an 8-wide caster warp that trigger
 *                   a fetch of new rays (1..32, default 4)
 *   "trace.wide_visits"  node steps a lane of the 8-wide caster takes per
 *                   loop iteration before the warp's shared leaf pool and
 *                   refill bookkeeping run (1, 2 or 3, default 3)
 *   "trace.wide_min_tris"  scenes with at least this many triangles use
 *                   the 8-wide caster (default 0: every scene; the binary
 *                   layout is then used for packets only); it applies to
 *                   closest-hit casts and to the wavefront render's bounce
 *                   rays alike
 *   "trace.block"   threads per block of the casting kernels: 64, 128
 *                   (default) or 256; the register budget per thread stays
 *                   the one the minblocks keys name
 *   "trace.stack"   traversal stack entries of the casting kernels: 16, 32
 *                   or 64, raised to the smallest of those that holds the
 *                   scene's tree; 0 (default) takes that smallest size (the
 *                   reference fixes 16, ray-trace-compute.comp:262, and
 *                   silently drops what does not fit; an overflow here is
 *                   reported as RT_ERR_STACK_OVERFLOW)
 *   "render.mode"   0 megakernel (one thread runs a pixel's whole path),
 *                   1 wavefront (per-bounce kernels over compacted queues),
 *                   2 (default) wavefront from render.wavefront_pixels up;
 *                   images are identical in every mode
 *   "render.wavefront_pixels"  the mode-2 threshold of rtRender (default
 *                   2^18 pixels: 512 x 512 and up)
 *   "render.batch_wavefront_pixels"  the split of batches and of the
 *                   render server's steps: jobs from this many pixels up run
 *                   as wavefronts side by side on side streams, the rest in
 *                   one persistent tile launch (default 1: every job; jobs
 *                   that run side by side fill the GPU at any size, where a
 *                   render alone keeps render.wavefront_pixels)
 *   "render.batch_streams"  side streams a batch (rtBatchCreate) spreads
 *                   its wavefront jobs over, 1..16 (default 16)
 *   "render.sort"   1 = reorder each bounce's rays of a wavefront render
 *                   (rtRender, batches, the render server) in Morton order
 *                   of origin and direction before casting them; 0 (default)
 *                   = cast them in the order shading queued them, which the
 *                   8-wide caster takes faster. Images are identical either way
 *   "bvh.builder"   tree built by rtUploadScene when no nodes are given:
 *                   0 (default) the reference's Bvh.h tree, node-for-node;
 *                   1 a linear BVH over Morton-ordered centroids,
 *                   2 agglomerative clustering of Morton-ordered triangles
 *                   (PLOC; tighter boxes, slower build). 1 and 2 are not
 *                   the reference's tree, but closest hits are identical
 *                   (equal-t ties go to the lower triangle index in every
 *                   tree); rtDownloadBvh returns the tree that was built
 *   "bvh.ploc_radius"  positions on either side the PLOC builder
 *                   (bvh.builder 2) searches for nearest neighbours, 1..256
 *                   (default 16)
 *   "bvh8.collapse"  how rtUploadScene folds the tree into the 8-wide
 *                   nodes the incoherent caster walks: 1 (default) the
 *                   folded pairs chosen by the surface area heuristic
 *                   (least summed node area: fewer node visits), 0 the
 *                   largest child opened first; the hits are the same
 *   "bvh.test_error_level"  test hook (default -1, off): builder 0 records
 *                   an error bit in its device error word after the sort of
 *                   this tree level, as a sort overflow would, so the upload
 *                   must fail with RT_ERR_INTERNAL
 * Values persist for the context; rtAutotuneTrace / rtAutotuneRender write
 * them. Unknown keys return RT_ERR_INVALID_ARGUMENT. */
rt_status rtSetTuning(rt_ctx *ctx, const char *key, int64_t value);
rt_status rtGetTuning(rt_ctx *ctx, const char *key, int64_t *value);

/* Autotuner (no counterpart in the reference, whose launch shape is fixed at
 * compile time, ray-trace-compute.comp:3, 262). Times the closest-hit
 * launch shapes on the caller's own device rays (coordinate descent over
 * trace.block, trace.stack, trace.wide, trace.wide_minblocks, trace.wide_visits, trace.defer,
 * trace.spec, trace.minblocks, trace.packet_minblocks, trace.sort, trace.beam; `reps` timed casts
 * per candidate after one warm-up) and keeps the fastest. Hits are identical
 * in every shape; d_hits receives them. The rates before and after tuning
 * are returned in Grays/s (either pointer may be NULL). Synchronous. */
rt_status rtAutotuneTrace(rt_ctx *ctx, rt_scene_id scene, const rt_ray *d_rays, uint32_t n, rt_hit *d_hits,
                          uint32_t reps, double *start_grays, double *best_grays);
/* Times megakernel against wavefront renders of the scene (its current
 * camera; spp samples, max_bounces) at square sizes 256, 512, ... up to
 * max_side (256..4096) and sets render.wavefront_pixels to the smallest
 * size from which the wavefront is faster (2^31 when it never is). Images
 * are identical either way. Synchronous; allocates one image of max_side^2
 * pixels for the duration of the call. */
rt_status rtAutotuneRender(rt_ctx *ctx, rt_scene_id scene, uint32_t spp, uint32_t max_bounces, uint32_t max_side,
                           uint64_t *wavefront_pixels);

/* Waits for the stream (NULL: the context stream) and reports any error a
 * kernel recorded since the last call (e.g. RT_ERR_STACK_OVERFLOW). */
rt_status rtSynchronize(rt_ctx *ctx, void *stream);

/* Ray segments (camera rays plus every secondary ray) traced by render calls
 * of this context since the last reset; waits for the device. Replaces the
 * reference's ms/frame print (src/main.cpp:403-412) as the throughput
 * counter. */
rt_status rtReadSegmentCounter(rt_ctx *ctx, uint64_t *out, int reset);

/* Allocation-free BVH build. No counterpart in the reference (which builds
 * its tree on the CPU); this is the same GPU build rtUploadScene runs, for
 * callers that may not allocate device memory — a host application whose
 * device memory is owned by another allocator or runtime, or code running
 * where cudaMalloc is forbidden. It allocates nothing: its scratch is a
 * fixed array inside the library (about 3.9 MB on every GPU that loads the
 * library, held until the process exits) plus static host buffers.
 *   d_triangles  n triangles in device memory (Bvh.h layout); a vertex
 *                coordinate that is NaN or infinite returns
 *                RT_ERR_INVALID_SCENE before any sorting starts
 *   n            1 .. 65536; larger n returns RT_ERR_INVALID_ARGUMENT
 *   bvh_seed     the rand() seed, as in rtUploadScene (the reference: 1)
 *   d_nodes      2n-1 nodes of device memory receiving the Bvh.h node array
 *   stream       cudaStream_t (NULL: the legacy default stream)
 * Returns once the nodes are written, and on every error path only after the
 * work it queued has finished. The first call on each device, with that
 * device current, looks up the array's device address
 * (cudaGetSymbolAddress). Calls share the array, which keeps the last call's contents: they
 * are serialised inside the library, and GPU work that overlaps a call on
 * the same device from outside the library and touches the array races.
 * Both pointers must be 16-byte aligned. */
rt_status rtBuildBvhNoAlloc(const rt_triangle *d_triangles, uint32_t n, uint32_t bvh_seed, rt_bvh_node *d_nodes,
                            void *stream);

/* ------------------------------------------------------------------ batches
 * Many renders of uneven size in one launch. */
typedef struct rt_render_job {
  rt_scene_id scene;
  uint32_t _pad;
  rt_camera camera;
  rt_render_params params;
  float *d_rgba32f;
} rt_render_job;

/* Renders every job; per job the image equals rtRender of that job alone.
 * Jobs from render.batch_wavefront_pixels up (default: all) run as
 * wavefronts spread over render.batch_streams side streams (default 16),
 * while one persistent launch covers the pixel tiles of the others; the two
 * overlap on the GPU. The reference renders one scene per dispatch
 * (src/main.cpp:228); this is the batched form. Returns when the jobs are
 * done. */
rt_status rtRenderBatch(rt_ctx *ctx, const rt_render_job *jobs, uint32_t n_jobs, void *stream);

/* A resident job table for repeated batched launches. Scenes named by the
 * jobs must stay resident while the batch exists. */
typedef struct rt_batch rt_batch;
rt_status rtBatchCreate(rt_ctx *ctx, const rt_render_job *jobs, uint32_t n_jobs, rt_batch **out);
rt_status rtBatchDestroy(rt_ctx *ctx, rt_batch *batch);
/* One launch of the batch (the persistent launch plus the side stream's
 * wavefront jobs, joined back into `stream`); performs no host
 * synchronisation and no allocation, so it can be captured in a CUDA graph.
 * The split between the two paths is fixed when the batch is created. */
rt_status rtBatchLaunch(rt_ctx *ctx, rt_batch *batch, void *stream);
/* Adds each job's spp to its sample_index on the device (the next
 * progressive frame); capturable. */
rt_status rtBatchAdvance(rt_ctx *ctx, rt_batch *batch, void *stream);
/* rtBatchLaunch followed by rtBatchAdvance, replayed from a CUDA graph that
 * the first call captures and instantiates (one graph launch per frame). */
rt_status rtBatchLaunchGraph(rt_ctx *ctx, rt_batch *batch, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* RTGB_RT_API_H */
