/*
 * rt_serve.h — a render server over one context: continuous batching of
 * render requests under an HBM budget.
 *
 * The reference renders one fixed scene per frame in a window loop
 * (src/main.cpp:399-421); there is no request path. Here requests (scene,
 * camera, size, samples, bounces) arrive from any host thread; a scheduler
 * thread keeps scenes, BVHs and accumulation images resident, admits queued
 * requests while the budget allows (evicting least-recently-used scenes that
 * no running request needs), and renders every running request together:
 * each step is one persistent launch that advances every running request by
 * up to `spp_per_step` samples, so requests that arrive while others are on
 * the GPU join at the next step and their work overlaps on the device.
 * Setting max_active = 1 and spp_per_step = 0 gives the plain form (one
 * whole request per launch, first come first served).
 */
#ifndef RTGB_RT_SERVE_H
#define RTGB_RT_SERVE_H

#include <stdint.h>
#include "rt_api.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rt_server rt_server;

typedef struct rt_server_desc {
  uint64_t hbm_budget_bytes; /* scenes + accumulation images; 0 = the context budget */
  uint32_t max_active;       /* requests rendered together (0 = 256) */
  uint32_t spp_per_step;     /* samples per request per step (0 = the whole request) */
  uint32_t _reserved[4];
} rt_server_desc;

typedef struct rt_request {
  uint32_t scene;       /* handle from rtServerAddScene */
  uint32_t width, height, spp, max_bounces, flags;
  rt_camera camera;
  float *host_out;      /* width*height*4 floats receiving the image (may be NULL) */
} rt_request;

enum { RT_REQ_QUEUED = 0, RT_REQ_RUNNING = 1, RT_REQ_DONE = 2, RT_REQ_FAILED = 3 };

typedef struct rt_request_status {
  uint32_t state;
  int32_t error;        /* rt_status of a failed request */
  double submit_ms, start_ms, done_ms; /* server clock */
} rt_request_status;

typedef struct rt_server_stats {
  uint64_t submitted, completed, failed;
  uint64_t steps, scene_uploads, scene_evictions;
  double p50_ms, p99_ms, mean_ms; /* submit -> done latency of completed requests */
  double busy_ms;                 /* time with requests in flight */
  uint64_t resident_bytes;
} rt_server_stats;

rt_status rtServerCreate(rt_ctx *ctx, const rt_server_desc *desc, rt_server **out);
/* Stops the scheduler; requests not yet finished are marked failed. */
rt_status rtServerDestroy(rt_server *server);
/* Registers a scene (host arrays are copied and kept on the host); it is
 * uploaded — BVH built on the GPU — when a request needs it and may be
 * evicted again when the budget is short. */
rt_status rtServerAddScene(rt_server *server, const rt_triangle *triangles, uint32_t n_triangles,
                           const rt_material *materials, uint32_t n_materials, const rt_sphere *spheres,
                           uint32_t n_spheres, uint32_t *scene_handle);
rt_status rtServerSubmit(rt_server *server, const rt_request *request, uint64_t *request_id);
rt_status rtServerPoll(rt_server *server, uint64_t request_id, rt_request_status *out);
/* Waits until the request is done or failed (timeout_ms = 0: no limit);
 * RT_ERR_TIMEOUT when the wait runs out. */
rt_status rtServerWait(rt_server *server, uint64_t request_id, uint32_t timeout_ms, rt_request_status *out);
rt_status rtServerStats(rt_server *server, rt_server_stats *out);
/* Clears the latency record and counters (not the resident scenes). */
rt_status rtServerResetStats(rt_server *server);

#ifdef __cplusplus
}
#endif

#endif /* RTGB_RT_SERVE_H */
