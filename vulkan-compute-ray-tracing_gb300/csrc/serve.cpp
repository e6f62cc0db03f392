// Render server: continuous batching under an HBM budget (rt_serve.h).
//
// One scheduler thread owns the GPU side. Each iteration it
//   1. admits queued requests while fewer than max_active run and their
//      scene plus accumulation image fit the budget, evicting resident
//      scenes that no running request uses, least recently used first;
//   2. uploads the scenes it admitted requests for (BVH built on the GPU);
//   3. renders every running request by up to spp_per_step samples: requests
//      that rtRender would give the wavefront kernels (large images) run on
//      side streams, all others in ONE persistent launch over their tiles
//      (launch_render_batch), the two overlapping on the GPU;
//   4. retires finished requests (image to the caller's host buffer,
//      accumulation image freed, latency recorded).
// Requests that arrive during a step are admitted at the next one, so new
// work joins the running set instead of waiting for it to drain.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "rt_internal.h"
#include "rtgb/rt_serve.h"

using namespace rtgb;

namespace {

using Clock = std::chrono::steady_clock;

struct SrvScene {
  std::vector<rt_triangle> tris;
  std::vector<rt_material> mats;
  std::vector<rt_sphere> sph;
  rt_scene_id resident = 0;
  uint64_t bytes = 0;
  uint64_t last_use = 0;
  int active_refs = 0;
};

struct SrvReq {
  uint64_t id = 0;
  rt_request r{};
  uint32_t done_spp = 0;
  float *d_accum = nullptr;
  uint64_t accum_bytes = 0;
  uint32_t state = RT_REQ_QUEUED;
  int32_t error = 0;
  double submit_ms = 0, start_ms = 0, done_ms = 0;
};

}  // namespace

struct rt_server {
  rt_ctx *ctx = nullptr;
  rt_server_desc desc{};
  uint64_t budget = 0, used = 0, tick = 0;
  std::thread th;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  bool stop = false;
  std::deque<SrvScene> scenes;
  std::deque<uint64_t> queue;
  std::vector<SrvReq *> active;
  std::unordered_map<uint64_t, SrvReq *> reqs;
  uint64_t next_id = 1;
  rt_server_stats stats{};
  std::vector<double> lat;
  Clock::time_point t0;
  double busy_since = -1.0;
  cudaStream_t stream = nullptr;
  BatchJob *d_jobs = nullptr, *h_jobs = nullptr;
  uint32_t *d_counter = nullptr;  // [0] tile counter, [64 * (1 + k)] side k's work counter
  int device = 0;
  // Wavefront side streams, their scratch (grown on demand) and join events.
  static constexpr int kSides = 16;
  cudaStream_t side[kSides] = {};
  cudaEvent_t fork = nullptr, join[kSides] = {};
  void *scratch[kSides] = {};
  size_t scratch_bytes[kSides] = {};
};

namespace {

double now_ms(const rt_server *s) {
  return std::chrono::duration<double, std::milli>(Clock::now() - s->t0).count();
}

void finish(rt_server *s, SrvReq *q, uint32_t state, int32_t err) {
  // Called with the lock held.
  q->state = state;
  q->error = err;
  q->done_ms = now_ms(s);
  if (state == RT_REQ_DONE) {
    s->stats.completed++;
    s->lat.push_back(q->done_ms - q->submit_ms);
  } else {
    s->stats.failed++;
  }
  s->cv_done.notify_all();
}

// Admission: pick requests that fit, reserving their bytes. Lock held.
void admit(rt_server *s, std::vector<SrvReq *> &admitted, std::vector<rt_scene_id> &evict) {
  const uint32_t cap = s->desc.max_active ? s->desc.max_active : 256;
  while (!s->queue.empty() && s->active.size() + admitted.size() < cap) {
    SrvReq *q = s->reqs[s->queue.front()];
    SrvScene &sc = s->scenes[q->r.scene];
    uint64_t need = q->accum_bytes + (sc.resident ? 0 : sc.bytes);
    if (need > s->budget) {
      s->queue.pop_front();
      finish(s, q, RT_REQ_FAILED, RT_ERR_BUDGET);
      continue;
    }
    while (s->used + need > s->budget) {
      // Least recently used resident scene that no running or admitted
      // request needs.
      SrvScene *victim = nullptr;
      for (SrvScene &c : s->scenes)
        if (c.resident && c.active_refs == 0 && &c != &sc && (!victim || c.last_use < victim->last_use))
          victim = &c;
      if (!victim) break;
      evict.push_back(victim->resident);
      victim->resident = 0;
      s->used -= victim->bytes;
      s->stats.scene_evictions++;
    }
    if (s->used + need > s->budget) break;  // wait for running requests to finish
    s->used += need;
    s->queue.pop_front();
    sc.active_refs++;
    sc.last_use = ++s->tick;
    q->state = RT_REQ_RUNNING;
    q->start_ms = now_ms(s);
    admitted.push_back(q);
  }
}

void scheduler(rt_server *s) {
  cudaSetDevice(s->device);
  std::vector<SrvReq *> admitted;
  std::vector<rt_scene_id> evict;
  for (;;) {
    admitted.clear();
    evict.clear();
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] { return s->stop || !s->queue.empty() || !s->active.empty(); });
      if (s->stop) return;
      if (s->busy_since < 0) s->busy_since = now_ms(s);
      admit(s, admitted, evict);
    }
    for (rt_scene_id id : evict) rtReleaseScene(s->ctx, id);
    // Uploads and accumulation images for the admitted requests.
    for (SrvReq *q : admitted) {
      SrvScene &sc = s->scenes[q->r.scene];
      rt_status st = RT_SUCCESS;
      if (!sc.resident) {
        rt_scene_id id = 0;
        st = rtUploadScene(s->ctx, sc.tris.data(), (uint32_t)sc.tris.size(), sc.mats.data(), (uint32_t)sc.mats.size(),
                           nullptr, 0, nullptr, 0, sc.sph.empty() ? nullptr : sc.sph.data(), (uint32_t)sc.sph.size(),
                           1, &id);
        if (st == RT_SUCCESS) {
          rt_scene_info info;
          rtGetSceneInfo(s->ctx, id, &info);
          std::lock_guard<std::mutex> g(s->mu);
          sc.resident = id;
          s->used += info.device_bytes;  // replace the estimate by the real size
          s->used -= sc.bytes;
          sc.bytes = info.device_bytes;
          s->stats.scene_uploads++;
        }
      }
      if (st == RT_SUCCESS) {
        cudaError_t e = cudaMalloc((void **)&q->d_accum, q->accum_bytes);
        if (e == cudaSuccess) e = cudaMemset(q->d_accum, 0, q->accum_bytes);
        if (e != cudaSuccess) st = e == cudaErrorMemoryAllocation ? RT_ERR_OUT_OF_MEMORY : RT_ERR_CUDA;
      }
      std::lock_guard<std::mutex> g(s->mu);
      if (st == RT_SUCCESS) {
        s->active.push_back(q);
      } else {
        if (q->d_accum) cudaFree(q->d_accum);
        q->d_accum = nullptr;
        s->used -= q->accum_bytes;
        sc.active_refs--;
        finish(s, q, RT_REQ_FAILED, st);
      }
    }
    // One step over every running request.
    std::vector<SrvReq *> run;
    {
      std::lock_guard<std::mutex> g(s->mu);
      run = s->active;
    }
    if (run.empty()) continue;
    uint64_t tiles = 0;
    uint32_t depth = 1, nj = 0;
    std::vector<uint32_t> step(run.size(), 0);
    std::vector<char> lost(run.size(), 0);
    std::vector<BatchJob> wf;
    bool sort = true, wide = true;
    uint32_t wide_min = 0;
    for (size_t i = 0; i < run.size(); i++) {
      SrvReq *q = run[i];
      SrvScene &sc = s->scenes[q->r.scene];
      DevScene dev;
      if (!ctx_scene_dev(s->ctx, sc.resident, &dev)) {
        lost[i] = 1;  // cannot happen while the request holds the scene
        continue;
      }
      uint32_t left = q->r.spp - q->done_spp;
      step[i] = s->desc.spp_per_step ? std::min(s->desc.spp_per_step, left) : left;
      BatchJob B;
      B.sc = dev;
      B.cam = q->r.camera;
      B.p = rt_render_params{q->r.width, q->r.height, step[i], q->r.max_bounces, q->done_spp, q->r.flags, {0, 0}};
      B.accum = q->d_accum;
      if (ctx_wavefront_render(s->ctx, B.p, &sort, &wide, &wide_min)) {
        wf.push_back(B);
        continue;
      }
      B.tile_begin = (uint32_t)tiles;
      B.tiles_x = batch_tiles_x(q->r.width);
      tiles += batch_tiles(q->r.width, q->r.height);
      depth = std::max(depth, dev.depth);
      s->h_jobs[nj++] = B;
    }
    cudaError_t e = cudaSuccess;
    const int sides = (int)std::min<size_t>(wf.size(), rt_server::kSides);
    for (int k = 0; k < sides && e == cudaSuccess; k++) {
      size_t need = 0;
      for (size_t j = k; j < wf.size(); j += rt_server::kSides)
        need = std::max(need, wavefront_scratch_bytes(wf[j].p.width * wf[j].p.height));
      if (need > s->scratch_bytes[k]) {
        if (s->scratch[k]) cudaFree(s->scratch[k]);
        s->scratch[k] = nullptr;
        s->scratch_bytes[k] = 0;
        e = cudaMalloc(&s->scratch[k], need);
        if (e == cudaSuccess) s->scratch_bytes[k] = need;
      }
    }
    if (e == cudaSuccess && sides) {
      e = cudaEventRecord(s->fork, s->stream);
      for (int k = 0; k < sides && e == cudaSuccess; k++) e = cudaStreamWaitEvent(s->side[k], s->fork, 0);
      for (size_t j = 0; j < wf.size() && e == cudaSuccess; j++) {
        const int k = (int)(j % rt_server::kSides);
        const BatchJob &J = wf[j];
        e = launch_render_wavefront(J.sc, J.cam, J.p, J.accum, ctx_segments(s->ctx), s->d_counter + 64 * (1 + k),
                                    ctx_err(s->ctx), s->scratch[k], sort, wide && J.sc.ntris >= wide_min,
                                    s->side[k]);
      }
      for (int k = 0; k < sides && e == cudaSuccess; k++) e = cudaEventRecord(s->join[k], s->side[k]);
    }
    if (e == cudaSuccess && nj)
      e = cudaMemcpyAsync(s->d_jobs, s->h_jobs, sizeof(BatchJob) * nj, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess && nj)
      e = launch_render_batch(s->d_jobs, nj, (uint32_t)tiles, depth, s->d_counter, ctx_segments(s->ctx),
                              ctx_err(s->ctx), s->stream);
    for (int k = 0; k < sides && e == cudaSuccess; k++) e = cudaStreamWaitEvent(s->stream, s->join[k], 0);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    // Retire.
    std::vector<SrvReq *> done;
    std::vector<char> ok;
    for (size_t i = 0; i < run.size(); i++) {
      SrvReq *q = run[i];
      q->done_spp += step[i];
      if (e != cudaSuccess || lost[i] || q->done_spp >= q->r.spp) {
        done.push_back(q);
        ok.push_back(e == cudaSuccess && !lost[i]);
      }
    }
    for (size_t i = 0; i < done.size(); i++) {
      SrvReq *q = done[i];
      if (ok[i] && q->r.host_out)
        cudaMemcpy(q->r.host_out, q->d_accum, q->accum_bytes, cudaMemcpyDeviceToHost);
      cudaFree(q->d_accum);
      q->d_accum = nullptr;
    }
    std::lock_guard<std::mutex> g(s->mu);
    s->stats.steps++;
    for (size_t i = 0; i < done.size(); i++) {
      SrvReq *q = done[i];
      s->active.erase(std::find(s->active.begin(), s->active.end(), q));
      s->used -= q->accum_bytes;
      s->scenes[q->r.scene].active_refs--;
      finish(s, q, ok[i] ? RT_REQ_DONE : RT_REQ_FAILED, ok[i] ? RT_SUCCESS : RT_ERR_CUDA);
    }
    if (s->active.empty() && s->queue.empty() && s->busy_since >= 0) {
      s->stats.busy_ms += now_ms(s) - s->busy_since;
      s->busy_since = -1.0;
    }
  }
}

}  // namespace

extern "C" {

rt_status rtServerCreate(rt_ctx *ctx, const rt_server_desc *desc, rt_server **out) {
  if (!ctx || !out) return RT_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  rt_server *s = new rt_server();
  s->ctx = ctx;
  if (desc) s->desc = *desc;
  s->budget = s->desc.hbm_budget_bytes ? s->desc.hbm_budget_bytes : ctx_budget(ctx);
  s->device = ctx_device(ctx);
  s->t0 = Clock::now();
  const uint32_t cap = s->desc.max_active ? s->desc.max_active : 256;
  cudaSetDevice(s->device);
  cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc((void **)&s->d_jobs, sizeof(BatchJob) * cap);
  if (e == cudaSuccess) e = cudaMallocHost((void **)&s->h_jobs, sizeof(BatchJob) * cap);
  if (e == cudaSuccess) e = cudaMalloc((void **)&s->d_counter, 256 * (1 + rt_server::kSides));
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming);
  for (int k = 0; k < rt_server::kSides && e == cudaSuccess; k++) {
    e = cudaStreamCreateWithFlags(&s->side[k], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->join[k], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    for (int k = 0; k < rt_server::kSides; k++) {
      if (s->side[k]) cudaStreamDestroy(s->side[k]);
      if (s->join[k]) cudaEventDestroy(s->join[k]);
    }
    if (s->fork) cudaEventDestroy(s->fork);
    if (s->d_counter) cudaFree(s->d_counter);
    if (s->stream) cudaStreamDestroy(s->stream);
    if (s->d_jobs) cudaFree(s->d_jobs);
    if (s->h_jobs) cudaFreeHost(s->h_jobs);
    delete s;
    return e == cudaErrorMemoryAllocation ? RT_ERR_OUT_OF_MEMORY : RT_ERR_CUDA;
  }
  s->th = std::thread(scheduler, s);
  *out = s;
  return RT_SUCCESS;
}

rt_status rtServerDestroy(rt_server *s) {
  if (!s) return RT_ERR_INVALID_ARGUMENT;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  s->th.join();
  cudaSetDevice(s->device);
  cudaStreamSynchronize(s->stream);
  {
    std::lock_guard<std::mutex> g(s->mu);
    for (auto &kv : s->reqs) {
      SrvReq *q = kv.second;
      if (q->d_accum) cudaFree(q->d_accum);
      if (q->state == RT_REQ_QUEUED || q->state == RT_REQ_RUNNING) finish(s, q, RT_REQ_FAILED, RT_ERR_BUSY);
      delete q;
    }
    for (SrvScene &c : s->scenes)
      if (c.resident) rtReleaseScene(s->ctx, c.resident);
  }
  for (int k = 0; k < rt_server::kSides; k++) {
    if (s->side[k]) cudaStreamSynchronize(s->side[k]);
    if (s->side[k]) cudaStreamDestroy(s->side[k]);
    if (s->join[k]) cudaEventDestroy(s->join[k]);
    if (s->scratch[k]) cudaFree(s->scratch[k]);
  }
  if (s->fork) cudaEventDestroy(s->fork);
  cudaStreamDestroy(s->stream);
  cudaFree(s->d_jobs);
  cudaFreeHost(s->h_jobs);
  cudaFree(s->d_counter);
  delete s;
  return RT_SUCCESS;
}

rt_status rtServerAddScene(rt_server *s, const rt_triangle *tris, uint32_t nt, const rt_material *mats, uint32_t nm,
                           const rt_sphere *sph, uint32_t ns, uint32_t *handle) {
  if (!s || !handle || !tris || !nt || !mats || !nm || (ns && !sph)) return RT_ERR_INVALID_ARGUMENT;
  SrvScene sc;
  sc.tris.assign(tris, tris + nt);
  sc.mats.assign(mats, mats + nm);
  if (ns) sc.sph.assign(sph, sph + ns);
  uint32_t nl = rtLightsFromMaterials(tris, nt, mats, nm, nullptr);
  sc.bytes = scene_device_bytes(nt, nm, nl, ns);
  std::lock_guard<std::mutex> g(s->mu);
  *handle = (uint32_t)s->scenes.size();
  s->scenes.push_back(std::move(sc));
  return RT_SUCCESS;
}

rt_status rtServerSubmit(rt_server *s, const rt_request *r, uint64_t *id) {
  if (!s || !r || !id) return RT_ERR_INVALID_ARGUMENT;
  if (r->width == 0 || r->height == 0 || r->width > 16384 || r->height > 16384 || r->spp == 0)
    return RT_ERR_INVALID_ARGUMENT;
  SrvReq *q = new SrvReq();
  q->r = *r;
  q->accum_bytes = 16ull * r->width * r->height;
  std::lock_guard<std::mutex> g(s->mu);
  if (r->scene >= s->scenes.size()) {
    delete q;
    return RT_ERR_NOT_FOUND;
  }
  q->id = s->next_id++;
  q->submit_ms = now_ms(s);
  s->reqs[q->id] = q;
  s->queue.push_back(q->id);
  s->stats.submitted++;
  *id = q->id;
  s->cv_work.notify_one();
  return RT_SUCCESS;
}

static void fill_status(const SrvReq *q, rt_request_status *out) {
  out->state = q->state;
  out->error = q->error;
  out->submit_ms = q->submit_ms;
  out->start_ms = q->start_ms;
  out->done_ms = q->done_ms;
}

rt_status rtServerPoll(rt_server *s, uint64_t id, rt_request_status *out) {
  if (!s || !out) return RT_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return RT_ERR_NOT_FOUND;
  fill_status(it->second, out);
  return RT_SUCCESS;
}

rt_status rtServerWait(rt_server *s, uint64_t id, uint32_t timeout_ms, rt_request_status *out) {
  if (!s) return RT_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return RT_ERR_NOT_FOUND;
  SrvReq *q = it->second;
  auto done = [&] { return q->state == RT_REQ_DONE || q->state == RT_REQ_FAILED; };
  if (timeout_ms == 0) {
    s->cv_done.wait(lk, done);
  } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done)) {
    if (out) fill_status(q, out);
    return RT_ERR_TIMEOUT;
  }
  if (out) fill_status(q, out);
  return RT_SUCCESS;
}

rt_status rtServerStats(rt_server *s, rt_server_stats *out) {
  if (!s || !out) return RT_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> g(s->mu);
  *out = s->stats;
  if (s->busy_since >= 0) out->busy_ms += now_ms(s) - s->busy_since;
  std::vector<double> v = s->lat;
  if (!v.empty()) {
    std::sort(v.begin(), v.end());
    auto pct = [&](double p) { return v[std::min(v.size() - 1, (size_t)(p * (v.size() - 1) + 0.5))]; };
    out->p50_ms = pct(0.50);
    out->p99_ms = pct(0.99);
    double sum = 0;
    for (double x : v) sum += x;
    out->mean_ms = sum / v.size();
  }
  out->resident_bytes = s->used;
  return RT_SUCCESS;
}

rt_status rtServerResetStats(rt_server *s) {
  if (!s) return RT_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> g(s->mu);
  uint64_t keep_uploads = s->stats.scene_uploads, keep_evictions = s->stats.scene_evictions;
  s->stats = rt_server_stats{};
  s->stats.scene_uploads = keep_uploads;
  s->stats.scene_evictions = keep_evictions;
  s->lat.clear();
  s->busy_since = (s->active.empty() && s->queue.empty()) ? -1.0 : now_ms(s);
  return RT_SUCCESS;
}

}  // extern "C"
