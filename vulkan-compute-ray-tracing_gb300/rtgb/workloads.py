"""Synthetic workloads of the batched and served render configurations.

Batched (one persistent launch over many scenes): scenes from the Cornell
generator with a soup count log-uniform in [1e3, 5e5] and 0-16 spheres of
radius U[0.2, 1], image side drawn from {128, 256, 512, 1024}, 4 samples per
pixel, 8 bounces. Served: a pool of such scenes, requests with a jittered
camera, side from {256, 512, 1024}, spp uniform in {1..64}, 8 bounces,
arriving as a Poisson stream. All draws come from the library's seeded
SplitMix64 stream (rtgbUniform), so every host generates the same workload.
"""
from __future__ import annotations

import math
import threading
import time
from dataclasses import dataclass

import numpy as np

from . import LIB, camera_look_at, gen_cornell


def uniform(seed: int, index: int) -> float:
    return LIB.rtgbUniform(seed, index)


@dataclass
class SceneSpec:
    seed: int
    n_soup: int
    n_spheres: int
    side: int


def batch_scene_specs(count: int, base_seed: int = 1000, sides=(128, 256, 512, 1024)):
    out = []
    for i in range(count):
        s = base_seed + i
        n_soup = int(round(1e3 * (500.0 ** uniform(s, 0))))
        n_sph = min(16, int(17 * uniform(s, 1)))
        side = sides[min(len(sides) - 1, int(len(sides) * uniform(s, 2)))]
        out.append(SceneSpec(s, n_soup, n_sph, side))
    return out


def make_scene(spec: SceneSpec):
    return gen_cornell(spec.seed, spec.n_soup, spec.n_spheres, 0.2, 1.0)


def default_camera(side: int, jitter_seed: int = -1):
    eye = [0.0, 0.0, -14.0]
    if jitter_seed >= 0:
        eye[0] += 2.0 * uniform(jitter_seed, 10) - 1.0
        eye[1] += 2.0 * uniform(jitter_seed, 11) - 1.0
    return camera_look_at(eye, [0, 0, 0], [0, 1, 0], 40.0, side, side)


@dataclass
class RequestSpec:
    arrival_s: float
    scene: int
    side: int
    spp: int
    jitter_seed: int


def request_stream(n: int, rate_hz: float, n_scenes: int, seed: int = 77, sides=(256, 512, 1024), spp_max: int = 64):
    t = 0.0
    out = []
    for i in range(n):
        s = seed * 1000003 + i
        t += -math.log(max(1e-12, 1.0 - uniform(s, 0))) / rate_hz
        scene = min(n_scenes - 1, int(n_scenes * uniform(s, 1)))
        side = sides[min(len(sides) - 1, int(len(sides) * uniform(s, 2)))]
        spp = 1 + min(spp_max - 1, int(spp_max * uniform(s, 3)))
        out.append(RequestSpec(t, scene, side, spp, s))
    return out


def run_stream(server, handles, reqs, bounces: int = 8, keep_image: bool = False):
    """Submits requests at their arrival times (open loop) and waits for all;
    with keep_image every result is copied back to host memory. Returns
    (wall seconds from first arrival to last completion, ids)."""
    ids = [None] * len(reqs)
    t0 = time.perf_counter()

    def feeder():
        for i, r in enumerate(reqs):
            delay = r.arrival_s - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            cam = default_camera(r.side, r.jitter_seed)
            ids[i] = server.submit(handles[r.scene], cam, r.side, r.side, r.spp, bounces, keep_image=keep_image)

    th = threading.Thread(target=feeder)
    th.start()
    th.join()
    for rid in ids:
        server.wait(rid)
    return time.perf_counter() - t0, ids
