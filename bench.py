"""Benchmark: closest-hit ray casting on the 1.31M-triangle displaced icosphere.

Workload (one step): the two ray batches of the closest-hit configuration,
traced against the mesh through the C ABI —
  * coherent: 4,194,304 primary rays of a 2048x2048 pinhole at (0,0,-3)
    looking +z, vfov 40 degrees;
  * incoherent: 4,194,304 rays, origins U[-1.5,1.5]^3, directions uniform on
    the sphere, tmin 1e-4.
The mesh is the icosahedron subdivided 8 times (1,310,720 triangles), radius
1, vertices displaced radially by 0.05*N(0,1); its BVH is built on the GPU
node-for-node as the reference's Bvh.h builds it. All inputs are seeded
synthetic data.

Reported:
  value      rays/s (Mrays/s) with rays resident in HBM (device API);
  e2e        the same through the host-array entry point (rtTraceClosestHost),
             pinned host rays in and hits out inside the timed region;
  roofline   algorithmic bytes of the culled traversal of the reference tree
             (48 B per node or triangle record fetched + 32 B ray + 16 B hit,
             counted by the oracle) / CUDA-event time of the trace kernel,
             against the measured HBM copy bandwidth;
  cpu_baseline  the oracle (fp32, culled traversal, OpenMP) on a bounded
             sample of the same rays, on this machine's host cores.
`--impl reference` times the reference path's CPU implementation (the
oracle restatement of the shader's hit_bvh; the reference's own GLSL needs a
Vulkan stack that is not available) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "vulkan-compute-ray-tracing_gb300"))

import numpy as np  # noqa: E402

METRIC = "Mrays/s incl. secondary (1 GB300, hit-exact); served renders/s + p50/p99 vs plain"
WORKLOAD = "closest-hit, icosphere L8 (1,310,720 tris), 4,194,304 coherent + 4,194,304 incoherent rays"
# Algorithmic bytes per ray (oracle, culled near-first traversal of the
# reference tree over 1/16 of each batch): 48 * (nodes + triangles) + 48.
ALG_BYTES_COHERENT = 48.0 * (531.24 + 61.47) + 48.0
ALG_BYTES_INCOHERENT = 48.0 * (369.86 + 41.28) + 48.0
RAYS_PER_BATCH = 2048 * 2048


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_from_profile():
    """DRAM bytes per trace launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "trace_closest_icosphere_l8.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.out = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                self.out = ""

    def summary(self):
        if not self.out:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out.strip().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for name, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_workload(rt):
    tris = rt.gen_icosphere(1, 8)
    mats = rt.gen_cornell(1, 0)[1]
    cam = rt.camera_look_at([0, 0, -3], [0, 0, 0], [0, 1, 0], 40.0, 2048, 2048)
    coherent = rt.gen_camera_rays(cam, 2048, 2048)
    incoherent = rt.gen_random_rays(3, RAYS_PER_BATCH)
    return tris, mats, coherent, incoherent


def dist_init():
    from rtgb import replicas
    return replicas.init()


def barrier(world):
    from rtgb import replicas
    replicas.barrier(world)


def max_over_ranks(x: float, world: int) -> float:
    from rtgb import replicas
    return replicas.max_over_ranks(x, world)


def cpu_baseline(tris, coherent, incoherent, nodes, target_s: float = 30.0):
    """The oracle on a bounded sample of both batches, all host threads."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    thr = oracle.max_threads()
    probe = 4096
    t0 = time.perf_counter()
    oracle.trace(tris, nodes, coherent[::1024][:probe // 2], slack=0.0)
    oracle.trace(tris, nodes, incoherent[::1024][:probe // 2], slack=0.0)
    rate = probe / max(time.perf_counter() - t0, 1e-6)
    per_batch = int(min(RAYS_PER_BATCH, max(4096, rate * target_s / 2)))
    stride = max(1, RAYS_PER_BATCH // per_batch)
    a, b = coherent[::stride][:per_batch], incoherent[::stride][:per_batch]
    t0 = time.perf_counter()
    oracle.trace(tris, nodes, a, slack=0.0)
    oracle.trace(tris, nodes, b, slack=0.0)
    dt = time.perf_counter() - t0
    n = len(a) + len(b)
    which = "every ray of both batches" if stride == 1 else f"one ray in {stride} of each batch"
    return {"value": n / dt / 1e6, "unit": "Mrays/s", "cores": thr, "kind": "port",
            "sample": f"{which} ({n} rays), oracle fp32 culled traversal, {thr} OpenMP threads, {dt:.1f} s"}


def run_reference(args):
    """--impl reference: the reference path's CPU implementation, timed."""
    world, rank, _ = dist_init()
    if rank != 0:
        return
    import rtgb
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    tris, mats, coherent, incoherent = make_workload(rtgb)
    nodes, _ = oracle.build_bvh(tris, 1)
    thr = oracle.max_threads()
    # The reference's own traversal where its shader was compiled from source
    # (oracle/_ref: hit_bvh of ray-trace-compute.comp, 16-entry stack), else
    # the oracle's restatement of it.
    if oracle.ref_shader_available():
        kind, what = "reference", "the reference shader's own hit_bvh (compiled from ray-trace-compute.comp)"

        def cast(rays):
            return oracle.ref_shader_trace(tris, nodes, rays)
    else:
        kind, what = "port", "oracle restatement of hit_bvh (culled)"

        def cast(rays):
            return oracle.trace(tris, nodes, rays, slack=0.0)
    # Each step: a fixed sample of both batches sized to ~4 s of CPU work.
    probe = 4096
    t0 = time.perf_counter()
    cast(coherent[::1024][:probe // 2])
    cast(incoherent[::1024][:probe // 2])
    rate = probe / max(time.perf_counter() - t0, 1e-6)
    per_batch = int(min(RAYS_PER_BATCH, max(2048, rate * 4.0 / 2)))
    stride = max(1, RAYS_PER_BATCH // per_batch)
    a, b = coherent[::stride][:per_batch], incoherent[::stride][:per_batch]
    for _ in range(args.warmup):
        cast(a[:256])
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cast(a)
        cast(b)
    dt = time.perf_counter() - t0
    n = (len(a) + len(b)) * args.steps
    value = n / dt / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample_per_step": f"one ray in {stride} of each batch "
                                                            f"({len(a) + len(b)} rays)"},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": thr, "kind": kind,
                         "sample": f"one ray in {stride} of each batch, {what}, {thr} OpenMP threads"},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference GLSL path unavailable on this box (no graphics stack); " +
                ("its own source, rewritten into C++, runs on the host cores" if kind == "reference"
                 else "its CPU restatement is timed"),
    }
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import torch
    world, rank, local = dist_init()
    torch.cuda.set_device(local)
    import rtgb
    tris, mats, coherent, incoherent = make_workload(rtgb)
    ctx = rtgb.Context(local)
    sc = ctx.upload_scene(tris, mats)
    info = sc.info()
    # A dedicated stream: every launch and every CUDA event of the timed
    # region is on it (the legacy default stream would not order against the
    # library's non-blocking streams).
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sptr = stream.cuda_stream
    d_rays = [torch.from_numpy(coherent).cuda(), torch.from_numpy(incoherent).cuda()]
    d_hits = [torch.empty((RAYS_PER_BATCH, 4), dtype=torch.float32, device="cuda") for _ in range(2)]

    def step(events=None):
        for b in range(2):
            if events is not None:
                events[b][0].record(stream)
            sc.trace(d_rays[b], RAYS_PER_BATCH, d_hits[b], stream=sptr)
            if events is not None:
                events[b][1].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ctx.synchronize(sptr)
    ev = [[[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(2)] for _ in range(args.steps)]
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        start.record(stream)
        for k in range(args.steps):
            step(ev[k])
        stop.record(stream)
        torch.cuda.synchronize()
    ctx.synchronize(sptr)
    barrier(world)
    ms = start.elapsed_time(stop)
    ms_max = max_over_ranks(ms, world)
    rays_step = 2 * RAYS_PER_BATCH
    value = rays_step * args.steps * world / (ms_max / 1e3) / 1e6
    kern = [[ev[k][b][0].elapsed_time(ev[k][b][1]) for k in range(args.steps)] for b in range(2)]
    coh_ms, inc_ms = statistics.mean(kern[0]), statistics.mean(kern[1])
    alg = [ALG_BYTES_COHERENT * RAYS_PER_BATCH, ALG_BYTES_INCOHERENT * RAYS_PER_BATCH]
    # Average algorithmic bytes per launch / average launch duration (GB/s).
    achieved = ((alg[0] + alg[1]) / 2) / (((coh_ms + inc_ms) / 2) / 1e3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    traffic = traffic_from_profile()

    # End to end: host arrays (pinned) through rtTraceClosestHost.
    h_rays = [torch.from_numpy(coherent).pin_memory(), torch.from_numpy(incoherent).pin_memory()]
    h_hits = [torch.empty((RAYS_PER_BATCH, 4), dtype=torch.float32).pin_memory() for _ in range(2)]

    def e2e_step():
        for b in range(2):
            rc = rtgb.LIB.rtTraceClosestHost(ctx.handle, sc.id, h_rays[b].data_ptr(), RAYS_PER_BATCH,
                                            h_hits[b].data_ptr())
            ctx.check(rc, "rtTraceClosestHost")

    for _ in range(max(1, args.warmup)):
        e2e_step()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e_value = rays_step * args.steps * world / e2e_s / 1e6
    # Sanity: the e2e hits equal the device-path hits.
    same = all(torch.equal(h_hits[b].view(torch.int32), d_hits[b].cpu().view(torch.int32)) for b in range(2))

    if rank != 0:
        ctx.close()
        return
    line = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "rays_per_step": rays_step, "bvh": "reference Bvh.h tree built on GPU",
                   "l2": "inputs larger than L2 (rays 268 MB + hits 134 MB + scene 147 MB per step)",
                   "parallelism": f"replicas x{world}", "coherent_grays": RAYS_PER_BATCH / coh_ms / 1e6,
                   "incoherent_grays": RAYS_PER_BATCH / inc_ms / 1e6, "bvh_build_ms": info.build_ms,
                   "bvh_depth": info.depth},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": peak_kind,
                     # DRAM bytes per ray actually moved (ncu), beside the
                     # algorithmic bytes: frac > 1 is L1/L2 reuse.
                     "dram_bytes_per_ray": traffic / RAYS_PER_BATCH if traffic else None,
                     "alg_bytes_per_ray": {"coherent": ALG_BYTES_COHERENT, "incoherent": ALG_BYTES_INCOHERENT}},
        "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": rays_step * 32,
                "d2h_bytes_per_step": rays_step * 16, "matches_device_path": bool(same)},
        # Per batch: 7 reordering kernels (extent, histogram, 3-kernel scan,
        # scatter, init) + 2 casting kernels (packets, then the listed
        # chunks per lane); two batches per step.
        "gpu_launches": 18 * args.steps,
        "clocks": clk.summary(),
    }
    # Separately reported: the same workload on trees that are not the
    # reference's (1 a linear BVH, 2 agglomerative clustering); the hits are
    # identical, only the traversal work differs.
    for key, builder in (("lbvh_mode", 1), ("ploc_mode", 2)):
        ctx.set_tuning("bvh.builder", builder)
        sc_l = ctx.upload_scene(tris, mats)
        ctx.set_tuning("bvh.builder", 0)
        alt = {}
        for name, b in (("coherent_grays", 0), ("incoherent_grays", 1)):
            sc_l.trace(d_rays[b], RAYS_PER_BATCH, d_hits[b], stream=sptr)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(max(1, args.steps // 2)):
                sc_l.trace(d_rays[b], RAYS_PER_BATCH, d_hits[b], stream=sptr)
            e1.record(stream)
            torch.cuda.synchronize()
            alt[name] = RAYS_PER_BATCH * max(1, args.steps // 2) / e0.elapsed_time(e1) / 1e6
        alt["bvh_build_ms"] = sc_l.info().build_ms
        alt["bvh_depth"] = sc_l.info().depth
        line[key] = alt
        sc_l.release()
    if not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline(tris, coherent, incoherent, sc.bvh())
    ctx.close()
    print(json.dumps(line), flush=True)


def _line(workload, metric, value, unit, args, extra):
    d = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
         "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
         "data": "synthetic (seeded)", "config": {"workload": workload}}
    d.update(extra)
    print(json.dumps(d), flush=True)


def run_render(args):
    """Config 0: Cornell box + 12,000 soup triangles, 256x256, 1 spp, 8 bounces."""
    import torch
    import rtgb
    ctx = rtgb.Context(0)
    t, m, s = rtgb.gen_cornell(1, 12000, 0)
    sc = ctx.upload_scene(t, m)
    W = H = 256
    sc.set_camera(rtgb.camera_look_at([0, 0, -14], [0, 0, 0], [0, 1, 0], 40.0, W, H))
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    acc = torch.zeros((H, W, 4), device="cuda")
    host = torch.empty((H, W, 4)).pin_memory()
    for k in range(args.warmup):
        sc.render(acc, W, H, spp=1, max_bounces=8, sample_index=k, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    ctx.segments(reset=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(args.steps):
        sc.render(acc, W, H, spp=1, max_bounces=8, sample_index=args.warmup + k, stream=stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    seg = ctx.segments(reset=True)
    t0 = time.perf_counter()
    for k in range(args.steps):
        sc.render(acc, W, H, spp=1, max_bounces=8, sample_index=k, stream=stream.cuda_stream)
        host.copy_(acc, non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    seg2 = ctx.segments(reset=True)
    _line("render 256x256 1spp 8 bounces, Cornell box + 12,000 soup triangles", METRIC, seg / (ms / 1e3) / 1e6,
          "Mrays/s", args, {"ms_per_step": ms / args.steps, "segments_per_step": seg / args.steps,
                            "e2e": {"value": seg2 / e2e_s / 1e6, "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                                    "d2h_bytes_per_step": W * H * 16}})
    ctx.close()


def run_batch(args):
    """Config 2: many scenes of uneven size, batched launch vs one launch per render."""
    import torch
    import rtgb
    from rtgb import workloads as wl
    ctx = rtgb.Context(0)
    specs = wl.batch_scene_specs(args.batch_scenes)
    scenes, jobs, accs = [], [], []
    t0 = time.perf_counter()
    build_ms = 0.0
    tris_total = 0
    for sp in specs:
        t, m, s = wl.make_scene(sp)
        sc = ctx.upload_scene(t, m, spheres=s)
        build_ms += sc.info().build_ms
        tris_total += len(t)
        scenes.append(sc)
        acc = torch.zeros((sp.side, sp.side, 4), device="cuda")
        accs.append(acc)
        jobs.append(rtgb.make_job(sc, wl.default_camera(sp.side), acc, sp.side, sp.side, 4, 8))
    setup_s = time.perf_counter() - t0
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sptr = stream.cuda_stream

    def plain():
        for sc, sp, acc in zip(scenes, specs, accs):
            sc.set_camera(wl.default_camera(sp.side))
            sc.render(acc, sp.side, sp.side, spp=4, max_bounces=8, stream=sptr)

    b = ctx.batch(jobs)
    res = {}
    for name, fn in (("plain", plain), ("batched", lambda: b.launch(sptr)), ("batched_graph", lambda: b.launch_graph(sptr))):
        fn()  # warm-up
        torch.cuda.synchronize()
        ctx.segments(reset=True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        seg = ctx.segments(reset=True) / args.steps
        res[name] = {"ms_per_batch": ms, "mrays_s": seg / (ms / 1e3) / 1e6, "renders_s": len(jobs) / (ms / 1e3)}
    b.destroy()
    _line(f"batched render: {len(jobs)} scenes ({tris_total} triangles), sides 128-1024, 4 spp, 8 bounces",
          METRIC, res["batched_graph"]["mrays_s"], "Mrays/s", args,
          {"modes": res, "speedup_vs_plain": res["batched_graph"]["renders_s"] / res["plain"]["renders_s"],
           "setup_s": setup_s, "bvh_build_ms_total": build_ms})
    ctx.close()


def run_serve(args):
    """Config 3: open-loop Poisson requests over resident scenes; continuous
    batching vs one request per launch."""
    import rtgb
    from rtgb import serve
    from rtgb import workloads as wl
    ctx = rtgb.Context(0)
    specs = wl.batch_scene_specs(args.serve_scenes, base_seed=2000)
    datas = [wl.make_scene(sp) for sp in specs]
    sides = tuple(int(x) for x in args.serve_sides.split(","))
    out = {}
    for rate in [float(x) for x in args.serve_rates.split(",")]:
        reqs = wl.request_stream(args.serve_requests, rate, len(specs), sides=sides, spp_max=args.serve_spp_max)
        for mode, kw in (("continuous", dict(max_active=args.serve_active, spp_per_step=args.serve_step)),
                         ("plain", dict(max_active=1, spp_per_step=0))):
            with serve.Server(ctx, hbm_budget_bytes=150 << 30, **kw) as srv:
                handles = [srv.add_scene(*d) for d in datas]
                warm = [srv.submit(h, wl.default_camera(8), 8, 8, 1, 1, keep_image=False) for h in handles]
                for w in warm:
                    srv.wait(w)
                srv.reset_stats()
                wall, ids = wl.run_stream(srv, handles, reqs)
                st = srv.stats()
                out[f"{mode}@{rate:g}"] = {"renders_s": len(reqs) / wall, "p50_ms": st.p50_ms, "p99_ms": st.p99_ms,
                                           "mean_ms": st.mean_ms, "steps": st.steps, "wall_s": wall,
                                           "uploads": st.scene_uploads, "evictions": st.scene_evictions}
    best = max(v["renders_s"] for k, v in out.items() if k.startswith("continuous"))
    _line(f"served renders: {args.serve_requests} Poisson requests per rate over {len(specs)} resident scenes, "
          f"sides {sides}, spp 1-{args.serve_spp_max}, 8 bounces", METRIC, best, "renders/s", args,
          {"rates": out})
    ctx.close()


def run_large(args):
    """Config 4: ~8M triangles (6x6 grid of flattened displaced level-7
    icospheres + the Cornell box), 1920x1080, 1 spp per frame, 8 bounces."""
    import torch
    import rtgb
    ctx = rtgb.Context(0)
    t, m = rtgb.gen_grid(4, 6, 6, 7, 0.35, 0.05, 222222, 3.0)
    sc = ctx.upload_scene(t, m)
    info = sc.info()
    W, H = 1920, 1080
    sc.set_camera(rtgb.camera_look_at([0, 2, -40], [0, -6, 0], [0, 1, 0], 40.0, W, H))
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    acc = torch.zeros((H, W, 4), device="cuda")
    frames = args.steps
    sc.render(acc, W, H, spp=1, max_bounces=8, sample_index=0, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    ctx.segments(reset=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(frames):
        sc.render(acc, W, H, spp=1, max_bounces=8, sample_index=k, stream=stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    seg = ctx.segments(reset=True)
    _line(f"progressive render 1920x1080, {frames} frames x 1 spp, 8 bounces, {info.triangles} triangles",
          METRIC, seg / (ms / 1e3) / 1e6, "Mrays/s", args,
          {"ms_per_frame": ms / frames, "bvh_build_ms": info.build_ms, "bvh_depth": info.depth,
           "triangles": info.triangles})
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="closest-hit", choices=["closest-hit", "render", "batch", "serve", "large"])
    ap.add_argument("--batch-scenes", type=int, default=256)
    ap.add_argument("--serve-scenes", type=int, default=64)
    ap.add_argument("--serve-requests", type=int, default=60)
    ap.add_argument("--serve-rates", default="1,4,64")
    ap.add_argument("--serve-sides", default="256,512,1024")
    ap.add_argument("--serve-spp-max", type=int, default=64)
    ap.add_argument("--serve-active", type=int, default=64)
    ap.add_argument("--serve-step", type=int, default=4)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "render":
        run_render(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.workload == "large":
        run_large(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
