"""CPU tests: the oracle pinned against the reference and the golden fixtures.

The reference ships no tests or known-answer vectors, so the pins are:
  * the reference's own Bvh::createBvh (oracle/_ref, built from the reference
    sources) — live where the checkout exists, and through the node-array
    digests in golden/bvh.json everywhere else;
  * glibc's rand() (the generator the reference's randomAxis draws from);
  * the golden trace/render fixtures written by golden/make_golden.py.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

NODE_COLS = [0, 1, 2, 4, 5, 6, 7, 8, 9]


def node_digest(nodes):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(nodes.view(np.uint32)[:, NODE_COLS]).tobytes()).hexdigest()


def load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def bvh_golden():
    return load("bvh.json")


SCENES = {
    "cornell_1410": lambda rt: rt.gen_cornell(11, 1410)[0],
    "cornell_12000": lambda rt: rt.gen_cornell(1, 12000)[0],
    "icosphere_l5": lambda rt: rt.gen_icosphere(2, 5),
    "icosphere_l6": lambda rt: rt.gen_icosphere(3, 6),
    "tiny_3": lambda rt: rt.gen_cornell(5, 0)[0][:3],
    "tiny_17": lambda rt: rt.gen_cornell(5, 5)[0],
    "icosphere_l8": lambda rt: rt.gen_icosphere(1, 8),
}


@pytest.mark.parametrize("name", list(SCENES))
def test_oracle_bvh_matches_reference_digest(rt, orc, bvh_golden, name):
    tris = SCENES[name](rt)
    g = bvh_golden[name]
    assert len(tris) == g["triangles"]
    nodes, depth = orc.build_bvh(tris, 1)
    assert len(nodes) == g["nodes"]
    for r, words in g["rows"].items():
        assert nodes.view(np.uint32)[int(r), NODE_COLS].tolist() == words
    assert node_digest(nodes) == g["digest"]


def test_oracle_bvh_seed(rt, orc, bvh_golden):
    tris = rt.gen_cornell(1, 12000)[0]
    nodes, _ = orc.build_bvh(tris, 7)
    assert node_digest(nodes) == bvh_golden["cornell_12000_seed7"]["digest"]


def _tie_heavy_scene(seed, n):
    """Triangles on a coarse integer lattice: most sort keys tie."""
    rng = np.random.default_rng(seed)
    t = np.zeros((n, 12), np.float32)
    for k in range(3):
        t[:, 4 * k:4 * k + 3] = rng.integers(-3, 4, size=(n, 3)).astype(np.float32)
    t[:, 3] = 0
    t[:, 7] = 0
    t.view(np.uint32)[:, 11] = 0
    return t


@pytest.mark.parametrize("seed,n", [(0, 2), (1, 5), (2, 33), (3, 100), (4, 1000), (5, 4097), (6, 20000)])
def test_oracle_bvh_matches_reference_live(orc, seed, n):
    if not orc.ref_available():
        pytest.skip("reference checkout not present on this machine (digests cover it)")
    tris = _tie_heavy_scene(seed, n)
    ref = orc.ref_build_bvh(tris, 1 + seed)
    mine, _ = orc.build_bvh(tris, 1 + seed)
    assert np.array_equal(ref.view(np.uint32)[:, NODE_COLS], mine.view(np.uint32)[:, NODE_COLS])


def test_reference_layouts(orc):
    if not orc.ref_available():
        pytest.skip("reference checkout not present on this machine")
    import ctypes
    buf = (ctypes.c_int * 64)()
    n = orc.ref_lib().ref_layout(buf, 64)
    got = list(buf)[:n]
    # Triangle 48 (0,16,32,44); BvhNode 48 (0,16,28,32,36); Material 32 (0,16);
    # Sphere 32 (0,16); Light 8 (0,4) — the offsets rt_types.h declares.
    assert got == [48, 0, 16, 32, 44, 48, 0, 16, 28, 32, 36, 32, 0, 16, 32, 0, 16, 8, 0, 4]


def test_glibc_rand(rt, orc):
    g = load("rand.json")
    for seed, vals in g.items():
        seed = int(seed)
        assert rt.glibc_rand(seed, 64).tolist() == vals
        assert orc.glibc_rand(seed, 64).tolist() == vals
    # Long run against the C library itself.
    for seed in (1, 99, 3000000000):
        assert np.array_equal(rt.glibc_rand(seed, 200000), orc.glibc_rand(seed, 200000))


def test_scene_generators_are_deterministic(rt):
    import hashlib

    def d(a):
        return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()

    g = load("scenes.json")
    t, m, s = rt.gen_cornell(1, 12000, 16, 0.2, 1.0)
    assert (d(t), d(m), d(s)) == (g["cornell_12000_16"]["tris"], g["cornell_12000_16"]["mats"],
                                  g["cornell_12000_16"]["spheres"])
    assert d(rt.gen_icosphere(1, 8)) == g["icosphere_l8"]["tris"]
    cam = rt.camera_look_at([0, 0, -3], [0, 0, 0], [0, 1, 0], 40.0, 2048, 2048)
    assert cam.as_array().tolist() == g["camera_rays_2048"]["camera"]
    assert d(rt.gen_camera_rays(cam, 2048, 2048)) == g["camera_rays_2048"]["rays"]
    assert d(rt.gen_random_rays(3, 4194304)) == g["random_rays_4m"]["rays"]
    gt, gm = rt.gen_grid(9, 2, 2, 3, 0.35, 0.05, 1000, 1.0)
    assert (d(gt), d(gm)) == (g["grid_small"]["tris"], g["grid_small"]["mats"])
    vals = [rt.LIB.rtgbUniform(s_, i) for s_, i in ((1, 0), (1, 1), (123456789, 987654321))]
    assert vals == g["uniform"]


def test_scene_shapes(rt):
    t, m, s = rt.gen_cornell(1, 12000, 3)
    assert t.shape == (12012, 12) and m.shape == (8, 8) and s.shape == (3, 8)
    mat = t.view(np.uint32)[:, 11]
    assert mat.max() <= 7 and (mat[12:] <= 6).all()
    assert (np.abs(t[:12, [0, 1, 2, 4, 5, 6, 8, 9, 10]]) <= 5.0).all()
    types = m.view(np.uint32)[:, 0].tolist()
    assert types == [1, 1, 1, 1, 2, 2, 3, 0]
    assert rt.gen_icosphere(1, 8).shape == (1310720, 12)


def test_oracle_trace_golden(rt, orc):
    tris = rt.gen_icosphere(2, 5)
    nodes, _ = orc.build_bvh(tris, 1)
    cam = rt.camera_look_at([0, 0, -3], [0, 0, 0], [0, 1, 0], 40.0, 64, 64)
    rays = np.concatenate([rt.gen_camera_rays(cam, 64, 64), rt.gen_random_rays(5, 4096)])
    hits = orc.trace(tris, nodes, rays)
    gold = np.load(os.path.join(GOLDEN, "trace_icosphere_l5.npy"))
    assert np.array_equal(hits.view(np.uint32), gold.view(np.uint32))
    lit = orc.trace(tris, nodes, rays, mode=1, stack_size=16)
    gold16 = np.load(os.path.join(GOLDEN, "trace_icosphere_l5_stack16.npy"))
    assert np.array_equal(lit.view(np.uint32), gold16.view(np.uint32))


def test_literal_and_culled_traversals_agree(rt, orc):
    """Q2: t-culling + near-first order give the shader-literal hits (stack
    large enough not to truncate) except where two candidates tie."""
    tris = rt.gen_icosphere(4, 6)
    nodes, depth = orc.build_bvh(tris, 1)
    cam = rt.camera_look_at([0, 0, -3], [0, 0, 0], [0, 1, 0], 40.0, 96, 96)
    rays = np.concatenate([rt.gen_camera_rays(cam, 96, 96), rt.gen_random_rays(9, 8192)])
    culled, st = orc.trace(tris, nodes, rays, mode=0, stats=True)
    lit, st_lit = orc.trace(tris, nodes, rays, mode=1, stack_size=256, stats=True)
    assert not (st_lit[:, 2] & 2).any(), "literal traversal truncated with a 256-entry stack"
    tie = (st[:, 2] & 1) != 0
    same = culled.view(np.int32)[:, 0] == lit.view(np.int32)[:, 0]
    assert same[~tie].all()
    assert np.array_equal(culled[~tie, 1], lit[~tie, 1])
    # The culled traversal fetches far fewer records.
    assert st[:, 0].mean() < 0.5 * st_lit[:, 0].mean()


def test_stack16_truncates_on_deep_trees(rt, orc):
    """Q1: the shader's 16-entry stack drops hits once the tree is deep."""
    tris = rt.gen_icosphere(4, 6)
    nodes, depth = orc.build_bvh(tris, 1)
    assert depth >= 17
    rays = rt.gen_random_rays(9, 4096)
    _, st = orc.trace(tris, nodes, rays, mode=1, stack_size=16, stats=True)
    assert (st[:, 2] & 2).any()


def test_oracle_render_golden(rt, orc):
    t, m, s = rt.gen_cornell(1, 12000, 4, 0.2, 1.0)
    nodes, _ = orc.build_bvh(t, 1)
    lights = orc.lights_from_materials(t, m)
    cam = rt.camera_look_at([0, 0, -14], [0, 0, 0], [0, 1, 0], 40.0, 64, 64).as_array()
    img, seg = orc.render(t, m, nodes, lights, s, cam, 64, 64, spp=1, max_bounces=8)
    gold = np.load(os.path.join(GOLDEN, "render_cornell_64.npy"))
    # libm sin/cos may differ by an ulp between hosts; a flipped path changes
    # one pixel, so compare by mean absolute error per channel.
    assert np.abs(img - gold).mean() <= 1e-4
    assert seg >= 64 * 64
    img, _ = orc.render(t, m, nodes, lights, s, cam, 64, 64, spp=4, max_bounces=8,
                        flags=rt.COMPAT_STACK16 | rt.COMPAT_LEN1 | rt.COMPAT_UNORM8)
    gold = np.load(os.path.join(GOLDEN, "render_cornell_64_compat.npy"))
    assert np.abs(img - gold).mean() <= 1e-4


def test_light_list_and_reference_camera(rt, orc):
    t, m, _ = rt.gen_cornell(3, 500)
    a = rt.lights_from_materials(t, m)
    b = orc.lights_from_materials(t, m)
    assert a.shape == (2, 2) and np.array_equal(a.view(np.uint32), b.view(np.uint32))
    for pos, (W, H) in (([1.8, 8.6, 1.1], (800, 600)), ([0.0, 0.0, 0.0], (256, 256)), ([-3, 2, 7], (1920, 1080))):
        cam = rt.camera_from_reference(pos, W, H).as_array()
        ref = orc.camera_from_reference(pos, W, H)
        assert np.array_equal(cam.view(np.uint32), ref.view(np.uint32))
