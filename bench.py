"""Benchmark of the ray-trace hot path on one GB300.

Headline (one step): the two ray batches of the closest-hit configuration,
traced against the mesh through the C ABI —
  * coherent: 4,194,304 primary rays of a 2048x2048 pinhole at (0,0,-3)
    looking +z, vfov 40 degrees;
  * incoherent: 4,194,304 rays, origins U[-1.5,1.5]^3, directions uniform on
    the sphere, tmin 1e-4.
The mesh is the icosahedron subdivided 8 times (1,310,720 triangles), radius
1, vertices displaced radially by 0.05*N(0,1); its BVH is built on the GPU
node-for-node as the reference's Bvh.h builds it. All inputs are seeded
synthetic data (no public dataset is involved).

Reported on the one JSON line:
  value      rays/s (Mrays/s) with rays resident in HBM (device API); the
             two batches of a step are cast side by side on two streams,
             while config.coherent_grays / incoherent_grays time each batch
             cast alone;
  e2e        the same through the host-array entry point (rtTraceClosestHost),
             pinned host rays in and hits out inside the timed region, the
             two batches' calls made from two host threads;
  roofline   the dominant casting kernel: algorithmic bytes of the culled
             traversal of the reference tree (48 B per node or triangle
             record + 32 B ray + 16 B hit, counted by the oracle) over its
             live time against the measured HBM copy bandwidth, plus the
             physical DRAM and issue-slot fractions from the committed ncu
             capture;
  parity     every ray's hit index against the oracle, the tie fraction and
             the largest t/u/v error against the fp64 oracle;
  cpu_baseline  the oracle (fp32, culled traversal, OpenMP) on every ray,
             on this machine's host cores, with the reference's own
             single-threaded Bvh::createBvh time;
  render_configs  the render-side configurations: Cornell 256^2 frames,
             the 8M-triangle 1080p progressive render (64 frames), the
             256-scene batch against one request per launch, and served
             Poisson requests against one request at a time (p50/p99), each
             with its own end-to-end figure.
`--impl reference` times the reference path's CPU implementation (its own
compute shader's hit_bvh, compiled from source; the GLSL itself needs a
Vulkan stack that is not available) on every ray of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "vulkan-compute-ray-tracing_gb300"))

import numpy as np  # noqa: E402

METRIC = "Mrays/s incl. secondary (1 GB300, hit-exact); served renders/s + p50/p99 vs plain"
WORKLOAD = "closest-hit, icosphere L8 (1,310,720 tris), 4,194,304 coherent + 4,194,304 incoherent rays"
# Algorithmic bytes per ray (oracle, culled near-first traversal of the
# reference tree over every ray of each batch): 48 * (nodes + triangles) + 48.
ALG_BYTES_COHERENT = 48.0 * (530.158 + 61.469) + 48.0
ALG_BYTES_INCOHERENT = 48.0 * (370.590 + 41.355) + 48.0
RAYS_PER_BATCH = 2048 * 2048
TUNING_KEYS = ("trace.block", "trace.stack", "trace.sort", "trace.packet", "trace.beam", "trace.packet_minblocks",
               "trace.defer",
               "trace.wide", "trace.wide_minblocks", "trace.wide_visits", "trace.wide_refill", "trace.minblocks",
               "trace.spec", "render.sort")


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def kernel_profiles():
    """Per-kernel figures of the committed ncu capture of this workload
    (profiles/trace_closest_icosphere_l8.md, lines "roofline_kernel: <name>
    key=value ..."): DRAM bytes, warp instructions issued and the ncu
    duration of one launch."""
    p = os.path.join(ROOT, "profiles", "trace_closest_icosphere_l8.md")
    out = {}
    if not os.path.exists(p):
        return out
    for line in open(p):
        if not line.startswith("roofline_kernel:"):
            continue
        parts = line.split(":", 1)[1].split()
        try:
            out[parts[0]] = {k: float(v) for k, v in (x.split("=", 1) for x in parts[1:])}
        except ValueError:
            continue
    return out


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


def cpu_baseline(oracle, tris, coherent, incoherent, nodes, target_s: float = 30.0):
    """The oracle's culled traversal (fp32, OpenMP, every host thread) on a
    bounded sample of both batches — every ray when that fits in about
    `target_s` seconds."""
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
    model = cpu_model()
    which = "every ray of both batches" if stride == 1 else f"one ray in {stride} of each batch"
    return {"value": n / dt / 1e6, "unit": "Mrays/s", "cores": thr, "kind": "port", "cpu_model": model,
            "sample": f"{which} ({n} rays), oracle fp32 culled traversal, {thr} OpenMP threads on {model}, "
                      f"{dt:.1f} s"}


def parity_block(oracle, tris, nodes, batches):
    """Every ray's closest-hit index against the fp32 oracle (rays whose two
    nearest candidates lie within 1e-6 relative t are ties and excluded),
    and t, u, v against the fp64 oracle on one ray in 16 where both pick the
    same triangle. `batches` is [(rays, gpu_hits)]."""
    rays_n = mism = ties_n = f64_n = f64_agree = 0
    err = [0.0, 0.0, 0.0]
    for rays, got in batches:
        want, st = oracle.trace(tris, nodes, rays, stats=True)
        ties = (st[:, 2] & 1) != 0
        gi, wi = got.view(np.int32)[:, 0], want.view(np.int32)[:, 0]
        rays_n += len(rays)
        ties_n += int(ties.sum())
        mism += int(((gi != wi) & ~ties).sum())
        sub = np.arange(0, len(rays), 16)
        tri64, tuv = oracle.trace_f64(tris, nodes, rays[sub])
        gs = got[sub]
        gsi = gs.view(np.int32)[:, 0]
        agree = (gsi == tri64) & (gsi >= 0)
        f64_n += int((gsi >= 0).sum())
        f64_agree += int(agree.sum())
        for c in range(3):
            ref = tuv[agree, c]
            rel = np.abs(gs[agree, 1 + c].astype(np.float64) - ref) / np.maximum(np.abs(ref), 1e-30)
            if len(rel):
                err[c] = max(err[c], float(rel.max()))
    return {"rays": rays_n, "index_mismatch_outside_ties": mism, "tie_fraction": ties_n / max(rays_n, 1),
            "max_rel_err_t": err[0], "max_rel_err_u": err[1], "max_rel_err_v": err[2],
            "fp64_sample": f"one ray in 16 ({rays_n // 16} rays); {f64_agree} of {f64_n} GPU hits pick the fp64 "
                           f"oracle's triangle",
            "bar": "index bit-exact outside ties; t, u, v within 1e-5 relative of fp64"}


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


def reference_bvh(oracle, tris):
    """The reference tree, built by the reference's own Bvh::createBvh where
    it was compiled from its source (single thread, timed), else by the
    oracle's restatement (equal node for node). Returns (nodes, seconds,
    what)."""
    t0 = time.perf_counter()
    if oracle.ref_available():
        nodes = oracle.ref_build_bvh(tris, 1)
        what = "the reference's Bvh::createBvh (src/ray-tracing/Bvh.h, compiled from source), one thread"
    else:
        nodes = oracle.build_bvh(tris, 1)[0]
        what = "the oracle's restatement of Bvh::createBvh, one thread"
    return nodes, time.perf_counter() - t0, what


def run_reference(args):
    """--impl reference: the reference path's CPU implementation, timed on
    this machine's host cores over every ray of both batches per step. Its
    inputs come from the oracle's restatement of the seeded generators (byte
    for byte the product's), so nothing of the product is loaded."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    tris, coherent, incoherent = oracle.closest_hit_workload()
    nodes, build_s, build_what = reference_bvh(oracle, tris)
    thr = oracle.max_threads()
    # The reference's own traversal where its shader was compiled from source
    # (oracle/_ref: hit_bvh of ray-trace-compute.comp, 16-entry stack), else
    # the oracle's literal restatement of the same loop.
    if oracle.ref_shader_available():
        kind, what = "reference", "the reference shader's own hit_bvh (ray-trace-compute.comp compiled from source)"

        def cast(rays):
            return oracle.ref_shader_trace(tris, nodes, rays)
    else:
        kind, what = "port", "the oracle's literal restatement of hit_bvh (16-entry stack, no t-culling)"

        def cast(rays):
            return oracle.trace(tris, nodes, rays, mode=1, stack_size=16, slack=0.0)
    warm = np.concatenate([coherent[::128], incoherent[::128]])
    for _ in range(args.warmup):
        cast(warm)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cast(coherent)
        cast(incoherent)
    dt = time.perf_counter() - t0
    n = 2 * RAYS_PER_BATCH * args.steps
    value = n / dt / 1e6
    model = cpu_model()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "rays_per_step": 2 * RAYS_PER_BATCH,
                   "warmup_sample": f"{len(warm)} rays (one in 128 of each batch) per warm-up step"},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": thr, "kind": kind, "cpu_model": model,
                         "sample": f"every ray of both batches ({2 * RAYS_PER_BATCH} per step), {what}, "
                                   f"{thr} OpenMP threads on {model}"},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "bvh_build_reference": {"seconds": build_s, "what": build_what},
        "note": "the reference's GLSL path is unavailable on this box (no graphics stack); " +
                ("its own source, rewritten into C++, runs on the host cores; its 16-entry stack truncates, "
                 "as in the reference" if kind == "reference" else "its CPU restatement is timed"),
    }
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import torch
    world, rank, local = dist_init()
    torch.cuda.set_device(local)
    import rtgb
    tris, mats, coherent, incoherent = make_workload(rtgb)
    ctx = rtgb.Context(local)
    for kv in args.tuning:
        key, value = kv.split("=", 1)
        ctx.set_tuning(key, int(value))
    sc = ctx.upload_scene(tris, mats)
    info = sc.info()
    # A dedicated stream: every launch and every CUDA event of the timed
    # region is on it (the legacy default stream would not order against the
    # library's non-blocking streams).
    stream = torch.cuda.Stream()
    side = torch.cuda.Stream()  # the incoherent batch's stream in a step
    torch.cuda.set_stream(stream)
    sptr = stream.cuda_stream
    d_rays = [torch.from_numpy(coherent).cuda(), torch.from_numpy(incoherent).cuda()]
    d_hits = [torch.empty((RAYS_PER_BATCH, 4), dtype=torch.float32, device="cuda") for _ in range(2)]

    def step():
        # The step's two independent casts run side by side: the incoherent
        # batch on a second stream forked from and joined back to the timed
        # one, so each cast's tail overlaps the other's work.
        fork = torch.cuda.Event()
        fork.record(stream)
        side.wait_event(fork)
        sc.trace(d_rays[1], RAYS_PER_BATCH, d_hits[1], stream=side.cuda_stream)
        sc.trace(d_rays[0], RAYS_PER_BATCH, d_hits[0], stream=sptr)
        join = torch.cuda.Event()
        join.record(side)
        stream.wait_event(join)

    def step_alone(events):
        # Each batch on its own (the per-batch Grays/s and the roofline's
        # batch times).
        for b in range(2):
            events[b][0].record(stream)
            sc.trace(d_rays[b], RAYS_PER_BATCH, d_hits[b], stream=sptr)
            events[b][1].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ctx.synchronize(sptr)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        start.record(stream)
        for k in range(args.steps):
            step()
        stop.record(stream)
        torch.cuda.synchronize()
    ctx.synchronize(sptr)
    barrier(world)
    ms = start.elapsed_time(stop)
    ms_max = max_over_ranks(ms, world)
    rays_step = 2 * RAYS_PER_BATCH
    value = rays_step * args.steps * world / (ms_max / 1e3) / 1e6
    ev = [[[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(2)] for _ in range(args.steps)]
    for k in range(args.steps):
        step_alone(ev[k])
    torch.cuda.synchronize()
    ctx.synchronize(sptr)
    kern = [[ev[k][b][0].elapsed_time(ev[k][b][1]) for k in range(args.steps)] for b in range(2)]
    coh_ms, inc_ms = statistics.mean(kern[0]), statistics.mean(kern[1])
    peak, peak_kind = measured_peak_hbm()
    prof = kernel_profiles()
    nsm = torch.cuda.get_device_properties(local).multi_processor_count

    def kernel_roofline(name, batch_ms, alg_bytes_per_ray, sm_mhz):
        # Algorithmic bytes of one batch over the batch's live CUDA-event time
        # (the cast is ~97% of it; the rest is ray reordering); the ncu
        # capture's DRAM bytes and issued warp instructions of the same
        # kernel over the same live time give the physical fractions.
        achieved = alg_bytes_per_ray * RAYS_PER_BATCH / (batch_ms / 1e3) / 1e9
        e = {"kernel": name, "batch_ms": batch_ms, "achieved": achieved, "frac": achieved / peak,
             "alg_bytes_per_ray": alg_bytes_per_ray}
        p = prof.get(name)
        if p:
            e["traffic"] = p["dram_bytes"]
            e["dram_bytes_per_ray"] = p["dram_bytes"] / RAYS_PER_BATCH
            e["dram_frac"] = p["dram_bytes"] / (batch_ms / 1e3) / (peak * 1e9)
            e["issue_frac"] = p["inst_issued"] / (batch_ms / 1e3 * sm_mhz * 1e6 * nsm * 4)
            e["ncu_duration_ms"] = p["duration_ms"]
        return e

    # End to end: host arrays (pinned) through rtTraceClosestHost.
    h_rays = [torch.from_numpy(coherent).pin_memory(), torch.from_numpy(incoherent).pin_memory()]
    h_hits = [torch.empty((RAYS_PER_BATCH, 4), dtype=torch.float32).pin_memory() for _ in range(2)]

    def e2e_batch(b, rcs):
        rcs[b] = rtgb.LIB.rtTraceClosestHost(ctx.handle, sc.id, h_rays[b].data_ptr(), RAYS_PER_BATCH,
                                             h_hits[b].data_ptr())

    def e2e_step():
        # The two batches' calls from two host threads, side by side as in
        # the device-path step (the library gives each call its own streams
        # and staging; ctypes releases the GIL during the call).
        rcs = [None, None]
        th = threading.Thread(target=e2e_batch, args=(1, rcs))
        th.start()
        e2e_batch(0, rcs)
        th.join()
        for rc in rcs:
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
    gpu_hits = [d_hits[b].cpu().numpy() for b in range(2)]
    same = all(np.array_equal(h_hits[b].numpy().view(np.int32), gpu_hits[b].view(np.int32)) for b in range(2))

    if rank != 0:
        ctx.close()
        return
    clocks = clk.summary()
    sm_mhz = clocks.get("sm_mhz") or 2070.0
    tuning = {k: ctx.get_tuning(k) for k in TUNING_KEYS}
    per = [kernel_roofline("k_trace_packets", coh_ms, ALG_BYTES_COHERENT, sm_mhz),
           kernel_roofline("k_trace_wide", inc_ms, ALG_BYTES_INCOHERENT, sm_mhz)]
    dom = max(per, key=lambda e: e["batch_ms"])
    roofline = {"bound": "hbm", "kernel": dom["kernel"], "achieved": dom["achieved"], "peak": peak, "unit": "GB/s",
                "frac": dom["frac"], "traffic": dom.get("traffic"), "peak_kind": peak_kind,
                "dram_frac": dom.get("dram_frac"), "issue_frac": dom.get("issue_frac"),
                "note": "achieved/frac: the oracle's algorithmic bytes (48 B per node or triangle record of the "
                        "culled traversal of the reference tree, + 48 B ray and hit) over the live time; "
                        "frac > 1 is L1/L2 reuse. dram_frac: the ncu capture's DRAM bytes over the live time "
                        "against the HBM peak; issue_frac: its issued warp instructions over 4 issue slots per SM "
                        "per cycle at the sampled SM clock — the bound these kernels meet",
                "per_kernel": {e["kernel"]: e for e in per}}
    line = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "rays_per_step": rays_step, "bvh": "reference Bvh.h tree built on GPU",
                   "l2": "inputs larger than L2 (rays 268 MB + hits 134 MB + scene 147 MB per step)",
                   "parallelism": f"replicas x{world}", "coherent_grays": RAYS_PER_BATCH / coh_ms / 1e6,
                   "incoherent_grays": RAYS_PER_BATCH / inc_ms / 1e6, "bvh_build_ms": info.build_ms,
                   "bvh_depth": info.depth,
                   "streams": "a step casts the two batches side by side on two streams (value); "
                              "coherent_grays and incoherent_grays time each batch cast alone"},
        "roofline": roofline,
        "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": rays_step * 32,
                "d2h_bytes_per_step": rays_step * 16, "matches_device_path": bool(same)},
        # Per batch: 7 reordering kernels (extent, histogram, 3-kernel scan,
        # scatter, init) + 2 casting kernels (packets, then the listed
        # chunks per lane); two batches per step.
        # Launch shape the casts ran with (rtSetTuning keys; the defaults,
        # which rtAutotuneTrace keeps on this workload).
        "tuning": tuning,
        "gpu_launches": 18 * args.steps,
        "clocks": clocks,
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
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        # The reference tree from the reference's own builder (one thread,
        # timed); the GPU's tree must equal it node for node.
        ref_nodes, build_s, build_what = reference_bvh(oracle, tris)
        cols = [0, 1, 2, 4, 5, 6, 7, 8, 9]
        line["config"]["bvh_equals_reference"] = bool(
            np.array_equal(sc.bvh().view(np.uint32)[:, cols], ref_nodes.view(np.uint32)[:, cols]))
        line["cpu_baseline"] = cpu_baseline(oracle, tris, coherent, incoherent, ref_nodes)
        line["cpu_baseline"]["bvh_build_reference_s"] = build_s
        line["cpu_baseline"]["bvh_build_reference"] = build_what
        line["parity"] = parity_block(oracle, tris, ref_nodes,
                                      [(coherent, gpu_hits[0]), (incoherent, gpu_hits[1])])
    ctx.close()
    if world == 1 and not args.closest_hit_only:
        # The rest of the metric (Mrays/s including secondary rays; served
        # renders/s with p50/p99 against the plain form), one key per
        # configuration, each with its own end-to-end figure.
        del d_rays, d_hits, h_rays, h_hits
        torch.cuda.empty_cache()
        line["render_configs"] = render_configs(args)
    print(json.dumps(line), flush=True)


def _line(workload, metric, value, unit, args, extra):
    d = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
         "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
         "data": "synthetic (seeded)", "config": {"workload": workload}}
    d.update(extra)
    print(json.dumps(d), flush=True)


def _timed(stream, fn, reps):
    """CUDA-event milliseconds of `reps` calls of fn on `stream`."""
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(reps):
        fn(k)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def render_c0(ctx, steps: int, warmup: int):
    """Cornell box + 12,000 soup triangles, 256x256, 1 spp, 8 bounces: one
    progressive frame per step (the reference's per-frame dispatch)."""
    import torch
    import rtgb
    t, m, _ = rtgb.gen_cornell(1, 12000, 0)
    sc = ctx.upload_scene(t, m)
    W = H = 256
    sc.set_camera(rtgb.camera_look_at([0, 0, -14], [0, 0, 0], [0, 1, 0], 40.0, W, H))
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    acc = torch.zeros((H, W, 4), device="cuda")
    host = torch.empty((H, W, 4)).pin_memory()
    for k in range(warmup):
        sc.render(acc, W, H, spp=1, max_bounces=8, sample_index=k, stream=sp)
    torch.cuda.synchronize()
    ctx.segments(reset=True)
    ms = _timed(stream, lambda k: sc.render(acc, W, H, spp=1, max_bounces=8, sample_index=warmup + k, stream=sp),
                steps)
    seg = ctx.segments(reset=True)
    # End to end: the same frames through rtRender, each image read back to
    # pinned host memory inside the timed region.
    t0 = time.perf_counter()
    for k in range(steps):
        sc.render(acc, W, H, spp=1, max_bounces=8, sample_index=k, stream=sp)
        host.copy_(acc, non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    seg2 = ctx.segments(reset=True)
    sc.release()
    return {"workload": "render 256x256, 1 spp per frame, 8 bounces, Cornell box + 12,000 soup triangles",
            "value": seg / (ms / 1e3) / 1e6, "unit": "Mrays/s", "frames": steps, "ms_per_frame": ms / steps,
            "segments_per_frame": seg / steps,
            "e2e": {"value": seg2 / e2e_s / 1e6, "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": W * H * 16}}


def large_c4(ctx, frames: int):
    """~8M triangles (6x6 grid of flattened displaced level-7 icospheres +
    the Cornell box), 1920x1080, `frames` progressive frames of 1 spp, 8
    bounces."""
    import torch
    import rtgb
    t, m = rtgb.gen_grid(4, 6, 6, 7, 0.35, 0.05, 222222, 3.0)
    sc = ctx.upload_scene(t, m)
    info = sc.info()
    W, H = 1920, 1080
    sc.set_camera(rtgb.camera_look_at([0, 2, -40], [0, -6, 0], [0, 1, 0], 40.0, W, H))
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    acc = torch.zeros((H, W, 4), device="cuda")
    host = torch.empty((H, W, 4)).pin_memory()
    sc.render(acc, W, H, spp=1, max_bounces=8, sample_index=0, stream=sp)
    torch.cuda.synchronize()
    ctx.segments(reset=True)
    ms = _timed(stream, lambda k: sc.render(acc, W, H, spp=1, max_bounces=8, sample_index=k, stream=sp), frames)
    seg = ctx.segments(reset=True)
    # End to end: the final image of the progressive run read back.
    t0 = time.perf_counter()
    for k in range(frames):
        sc.render(acc, W, H, spp=1, max_bounces=8, sample_index=k, stream=sp)
    host.copy_(acc, non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    seg2 = ctx.segments(reset=True)
    sc.release()
    return {"workload": f"progressive render 1920x1080, {frames} frames x 1 spp, 8 bounces, "
                        f"{info.triangles} triangles (6x6 flattened displaced level-7 icospheres + Cornell box)",
            "value": seg / (ms / 1e3) / 1e6, "unit": "Mrays/s", "ms_per_frame": ms / frames,
            "bvh_build_ms": info.build_ms, "bvh_depth": info.depth, "triangles": info.triangles,
            "e2e": {"value": seg2 / e2e_s / 1e6, "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": W * H * 16 // frames}}


def batch_c2(ctx, n_scenes: int, reps: int, modes=("plain_one_launch", "plain", "batched", "batched_graph")):
    """256 scenes of uneven size, 4 spp, 8 bounces: the batched launch (one
    persistent launch over the small jobs plus wavefront side streams, and
    its CUDA-graph replay) against one request per launch."""
    import torch
    import rtgb
    from rtgb import workloads as wl
    specs = wl.batch_scene_specs(n_scenes)
    scenes, jobs, accs = [], [], []
    t0 = time.perf_counter()
    build_ms = 0.0
    tris_total = 0
    for sp_ in specs:
        t, m, s = wl.make_scene(sp_)
        sc = ctx.upload_scene(t, m, spheres=s)
        build_ms += sc.info().build_ms
        tris_total += len(t)
        scenes.append(sc)
        acc = torch.zeros((sp_.side, sp_.side, 4), device="cuda")
        accs.append(acc)
        jobs.append(rtgb.make_job(sc, wl.default_camera(sp_.side), acc, sp_.side, sp_.side, 4, 8))
    setup_s = time.perf_counter() - t0
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream
    for sc, sp_ in zip(scenes, specs):
        sc.set_camera(wl.default_camera(sp_.side))

    def plain(_k):
        for sc, sp_, acc in zip(scenes, specs, accs):
            sc.render(acc, sp_.side, sp_.side, spp=4, max_bounces=8, stream=sptr)

    b = ctx.batch(jobs)
    old_mode = ctx.get_tuning("render.mode")
    res = {}

    def one_launch(k):
        ctx.set_tuning("render.mode", 0)
        plain(k)

    for name, fn in (("plain_one_launch", one_launch), ("plain", plain), ("batched", lambda k: b.launch(sptr)),
                     ("batched_graph", lambda k: b.launch_graph(sptr))):
        if name not in modes:
            continue
        fn(0)  # warm-up
        torch.cuda.synchronize()
        ctx.segments(reset=True)
        ms = _timed(stream, fn, reps) / reps
        ctx.set_tuning("render.mode", old_mode)
        seg = ctx.segments(reset=True) / reps
        res[name] = {"ms_per_batch": ms, "mrays_s": seg / (ms / 1e3) / 1e6, "renders_s": len(jobs) / (ms / 1e3)}
    # End to end: the graph replay plus every image read back to pinned host.
    hosts = [torch.empty_like(a, device="cpu").pin_memory() for a in accs]
    d2h = sum(a.numel() * 4 for a in accs)
    t0 = time.perf_counter()
    for _ in range(reps):
        b.launch_graph(sptr)
        with torch.cuda.stream(stream):
            for h, a in zip(hosts, accs):
                h.copy_(a, non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / reps
    b.destroy()
    for sc in scenes:
        sc.release()
    best = res.get("batched_graph") or res.get("batched") or next(iter(res.values()))
    ratio = (lambda key: best["renders_s"] / res[key]["renders_s"] if key in res else None)
    return {"workload": f"batched render: {len(jobs)} scenes ({tris_total} triangles), sides 128-1024, 4 spp, "
                        f"8 bounces", "value": best["renders_s"], "unit": "renders/s", "mrays_s": best["mrays_s"],
            "modes": res, "speedup_vs_one_launch_per_request": ratio("plain_one_launch"),
            "speedup_vs_rtrender_per_request": ratio("plain"),
            "plain_forms": "plain_one_launch: one k_render launch per request, the reference's one dispatch per "
                           "frame; plain: rtRender per request (megakernel below 2^20 pixels, wavefront above)",
            "setup_s": setup_s, "bvh_build_ms_total": build_ms, "reps": reps,
            "e2e": {"value": len(jobs) / e2e_s, "unit": "renders/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": d2h}}


def serve_c3(ctx, n_scenes: int, n_requests: int, rates, sides=(256, 512, 1024), spp_max: int = 64,
             max_active: int = 64, spp_step: int = 4):
    """Open-loop Poisson requests over resident scenes: continuous batching
    against one request at a time, p50/p99 latency beside renders/s. Every
    request's image is copied back to host memory (end to end)."""
    from rtgb import serve
    from rtgb import workloads as wl
    specs = wl.batch_scene_specs(n_scenes, base_seed=2000)
    datas = [wl.make_scene(sp_) for sp_ in specs]
    out = {}
    for rate in rates:
        reqs = wl.request_stream(n_requests, rate, len(specs), sides=sides, spp_max=spp_max)
        for mode, kw in (("continuous", dict(max_active=max_active, spp_per_step=spp_step)),
                         ("plain", dict(max_active=1, spp_per_step=0)),
                         ("plain_one_launch", dict(max_active=1, spp_per_step=0))):
            # plain: one request at a time with rtRender's split (megakernel
            # below render.wavefront_pixels, wavefront from there up);
            # plain_one_launch: one persistent megakernel launch per request
            # (render.mode 0), the reference's one dispatch per frame.
            old_mode = ctx.get_tuning("render.mode")
            old_split = ctx.get_tuning("render.batch_wavefront_pixels")
            if mode == "plain":
                ctx.set_tuning("render.batch_wavefront_pixels", ctx.get_tuning("render.wavefront_pixels"))
            if mode == "plain_one_launch":
                ctx.set_tuning("render.mode", 0)
            with serve.Server(ctx, hbm_budget_bytes=150 << 30, **kw) as srv:
                handles = [srv.add_scene(*d) for d in datas]
                warm = [srv.submit(h, wl.default_camera(8), 8, 8, 1, 1, keep_image=False) for h in handles]
                for w in warm:
                    srv.wait(w)
                srv.reset_stats()
                wall, ids = wl.run_stream(srv, handles, reqs, keep_image=True)
                st = srv.stats()
                out[f"{mode}@{rate:g}"] = {"renders_s": len(reqs) / wall, "p50_ms": st.p50_ms, "p99_ms": st.p99_ms,
                                           "mean_ms": st.mean_ms, "steps": st.steps, "wall_s": wall,
                                           "uploads": st.scene_uploads, "evictions": st.scene_evictions}
            ctx.set_tuning("render.mode", old_mode)
            ctx.set_tuning("render.batch_wavefront_pixels", old_split)
    ratios = {f"{r:g}": out[f"continuous@{r:g}"]["renders_s"] / out[f"plain@{r:g}"]["renders_s"] for r in rates}
    ratios_one = {f"{r:g}": out[f"continuous@{r:g}"]["renders_s"] / out[f"plain_one_launch@{r:g}"]["renders_s"]
                  for r in rates}
    best = max(v["renders_s"] for k, v in out.items() if k.startswith("continuous"))
    return {"workload": f"served renders: {n_requests} Poisson requests per rate over {len(specs)} resident "
                        f"scenes, sides {tuple(sides)}, spp 1-{spp_max}, 8 bounces, 150 GB budget",
            "value": best, "unit": "renders/s", "rates": out, "speedup_vs_plain": ratios,
            "speedup_vs_one_launch_per_request": ratios_one,
            "plain_forms": "plain: one request at a time with rtRender's split (megakernel below 512^2, wavefront "
                           "from there up); plain_one_launch: one request at a time, one megakernel launch per "
                           "request",
            "e2e": {"value": best, "unit": "renders/s",
                    "note": "requests submitted from the host with each image copied back to host memory; "
                            "wall clock from the first arrival to the last completion"}}


def run_render(args):
    import rtgb
    ctx = rtgb.Context(0)
    r = render_c0(ctx, args.steps, args.warmup)
    _line(r.pop("workload"), METRIC, r.pop("value"), r.pop("unit"), args, r)
    ctx.close()


def run_batch(args):
    import rtgb
    ctx = rtgb.Context(0)
    r = batch_c2(ctx, args.batch_scenes, max(1, args.steps), tuple(args.batch_modes.split(",")))
    _line(r.pop("workload"), METRIC, r.pop("value"), r.pop("unit"), args, r)
    ctx.close()


def run_serve(args):
    import rtgb
    ctx = rtgb.Context(0)
    r = serve_c3(ctx, args.serve_scenes, args.serve_requests, [float(x) for x in args.serve_rates.split(",")],
                 tuple(int(x) for x in args.serve_sides.split(",")), args.serve_spp_max, args.serve_active,
                 args.serve_step)
    _line(r.pop("workload"), METRIC, r.pop("value"), r.pop("unit"), args, r)
    ctx.close()


def run_large(args):
    import rtgb
    ctx = rtgb.Context(0)
    r = large_c4(ctx, args.steps)
    _line(r.pop("workload"), METRIC, r.pop("value"), r.pop("unit"), args, r)
    ctx.close()


def render_configs(args):
    """The render-side configurations, reported as keys of the default line."""
    import rtgb
    out = {}
    ctx = rtgb.Context(0)
    try:
        for key, fn in (("render_cornell_256", lambda: render_c0(ctx, 20, 3)),
                        ("progressive_8m_1080p", lambda: large_c4(ctx, 64)),
                        ("batched_256_scenes", lambda: batch_c2(ctx, args.batch_scenes, 1)),
                        ("served_poisson", lambda: serve_c3(ctx, args.serve_scenes, args.serve_requests,
                                                             [float(x) for x in args.serve_rates.split(",")],
                                                             tuple(int(x) for x in args.serve_sides.split(",")),
                                                             args.serve_spp_max, args.serve_active,
                                                             args.serve_step))):
            t0 = time.perf_counter()
            out[key] = fn()
            out[key]["wall_s"] = time.perf_counter() - t0
    finally:
        ctx.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--closest-hit-only", action="store_true",
                    help="skip the render, batched, served and large-scene configurations of the default line")
    ap.add_argument("--tuning", action="append", default=[], metavar="KEY=VALUE",
                    help="closest-hit workload: set a tuning key (rtSetTuning) before the scene upload; repeatable")
    ap.add_argument("--workload", default="closest-hit", choices=["closest-hit", "render", "batch", "serve", "large"])
    ap.add_argument("--batch-scenes", type=int, default=256)
    ap.add_argument("--batch-modes", default="plain_one_launch,plain,batched,batched_graph",
                    help="forms the batch workload times (a subset narrows a profile to the batched launch)")
    ap.add_argument("--serve-scenes", type=int, default=64)
    ap.add_argument("--serve-requests", type=int, default=40)
    ap.add_argument("--serve-rates", default="10,100,2000")
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
