"""The reference's own compute shader as the pin for the shader restatement.

ray-trace-compute.comp is compiled on the host from its source
(oracle/glsl2cpp.py + oracle/shim/glsl.h -> oracle/_ref/libref_shader.so)
and driven frame by frame as src/main.cpp drives it: hit_bvh with its
16-entry stack, NUM_BOUNCES 2, no spheres, lights.length() of the bound
range, rgba8 target and accumulation images. The oracle's restatement in the
matching compat mode (RT_COMPAT_STACK16 | LEN1 | NO_SPHERES | UNORM8, two
bounces, rtCameraFromReference) must equal it byte for byte. The committed
ref_shader_*.npy fixtures carry the reference's output to machines without
the checkout, where the oracle is checked against them instead. The same
holds for ray-trace-compute-simple.comp (oracle/_ref/libref_shader_simple.so)
and the RT_SHADE_SIMPLE mode."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

COMPAT = ("COMPAT_STACK16", "COMPAT_LEN1", "COMPAT_NO_SPHERES", "COMPAT_UNORM8")


def fixture_meta():
    with open(os.path.join(GOLDEN, "ref_shader.json")) as f:
        return json.load(f)


def cornell_scene(rt):
    t, m, _ = rt.gen_cornell(3, 3000, 0)
    m = m.copy()
    m[:, 1] = 0.0  # metal fuzz is not part of the reference's material
    return t, m, np.zeros((1, 8), np.float32)


def compat_flags(rt, all_lights, simple=False):
    flags = rt.SHADE_SIMPLE if simple else 0
    for name in COMPAT:
        if name == "COMPAT_LEN1" and all_lights:
            continue
        flags |= getattr(rt, name)
    return flags


def oracle_frames(rt, orc, t, m, nodes, lights, sph, cam_pos, W, H, frames, all_lights, simple=False):
    flags = compat_flags(rt, all_lights, simple)
    cam = rt.camera_from_reference(cam_pos, W, H).as_array()
    acc = np.zeros((H, W, 4), np.float32)
    for s in range(frames):
        acc, _ = orc.render(t, m, nodes, lights, sph, cam, W, H, spp=1, max_bounces=4 if simple else 2,
                            sample_index=s, flags=flags, accum=acc)
    return acc


def as_u8(img):
    return np.rint(np.asarray(img, np.float64) * 255.0).astype(np.uint8)


CORNELL_FIXTURES = ["ref_shader_cornell_96x64", "ref_shader_cornell_96x64_lights", "ref_shader_simple_cornell_96x64"]


@pytest.mark.parametrize("name", CORNELL_FIXTURES)
def test_oracle_equals_reference_shader_fixture(rt, orc, name):
    """Runs everywhere: the restatement against the reference's committed output."""
    meta = fixture_meta()[name]
    simple = meta.get("shader") == "simple"
    assert meta["max_bounces"] == (4 if simple else 2)
    t, m, sph = cornell_scene(rt)
    nodes, _ = orc.build_bvh(t, 1)
    lights = orc.lights_from_materials(t, m)
    got = oracle_frames(rt, orc, t, m, nodes, lights, sph, meta["cam_pos"], meta["width"], meta["height"],
                        meta["frames"], meta["lights"] == "all", simple)
    want = np.load(os.path.join(GOLDEN, name + ".npy"))
    assert np.array_equal(as_u8(got), want)
    assert want[..., :3].mean() > 10  # a lit image, not an empty one


needs_ref_shader = pytest.mark.skipif(
    not os.path.exists(os.path.join(os.path.dirname(__file__), "..", "oracle", "_ref", "libref_shader.so")),
    reason="the reference's shader was not compiled (no reference checkout)")


@needs_ref_shader
@pytest.mark.parametrize("frames,all_lights,first", [(1, False, 0), (3, False, 0), (2, True, 0), (2, False, 5)])
def test_oracle_equals_reference_shader(rt, orc, frames, all_lights, first):
    t, m, sph = cornell_scene(rt)
    nodes = orc.ref_build_bvh(t, 1)
    lights = orc.lights_from_materials(t, m)
    W, H, cam_pos = 64, 64, (0.3, 4.0, -0.2)
    want = orc.ref_shader_render(t, m, nodes, lights, sph, cam_pos, W, H, frames, first_sample=first,
                                 lights_len=len(lights) if all_lights else 1)
    flags = compat_flags(rt, all_lights)
    cam = rt.camera_from_reference(cam_pos, W, H).as_array()
    acc = np.zeros((H, W, 4), np.float32)
    for s in range(first, first + frames):
        acc, _ = orc.render(t, m, nodes, lights, sph, cam, W, H, spp=1, max_bounces=2, sample_index=s, flags=flags,
                            accum=acc)
    assert np.array_equal(as_u8(acc), as_u8(want))


needs_ref_shader_simple = pytest.mark.skipif(
    not os.path.exists(os.path.join(os.path.dirname(__file__), "..", "oracle", "_ref", "libref_shader_simple.so")),
    reason="the reference's simple shader was not compiled (no reference checkout)")


@needs_ref_shader
@needs_ref_shader_simple
def test_reference_shader_fixtures_are_current(rt, orc):
    """The committed fixtures are what the compiled reference shaders make."""
    meta = fixture_meta()
    for name in CORNELL_FIXTURES:
        mt = meta[name]
        t, m, sph = cornell_scene(rt)
        nodes = orc.ref_build_bvh(t, 1)
        lights = orc.lights_from_materials(t, m)
        img = orc.ref_shader_render(t, m, nodes, lights, sph, mt["cam_pos"], mt["width"], mt["height"],
                                    mt["frames"], lights_len=len(lights) if mt["lights"] == "all" else 1,
                                    simple=mt.get("shader") == "simple")
        assert np.array_equal(as_u8(img), np.load(os.path.join(GOLDEN, name + ".npy")))


@needs_ref_shader_simple
@pytest.mark.parametrize("frames,first,cam_pos", [(1, 0, (0.3, 4.0, -0.2)), (3, 2, (0.0, 4.5, 0.0))])
def test_simple_shading_equals_reference_simple_shader(rt, orc, frames, first, cam_pos):
    """ray-trace-compute-simple.comp (hit_bvh, NUM_BOUNCES 4, every bounce
    scatters into the normal's hemisphere with a normalised
    random_in_unit_sphere, emitters end the path) against the restatement's
    RT_SHADE_SIMPLE mode, byte for byte."""
    t, m, sph = cornell_scene(rt)
    nodes = orc.ref_build_bvh(t, 1)
    lights = orc.lights_from_materials(t, m)
    W, H = 64, 48
    want = orc.ref_shader_render(t, m, nodes, lights, sph, cam_pos, W, H, frames, first_sample=first, simple=True)
    cam = rt.camera_from_reference(cam_pos, W, H).as_array()
    acc = np.zeros((H, W, 4), np.float32)
    for s in range(first, first + frames):
        acc, _ = orc.render(t, m, nodes, lights, sph, cam, W, H, spp=1, max_bounces=4, sample_index=s,
                            flags=compat_flags(rt, False, True), accum=acc)
    assert np.array_equal(as_u8(acc), as_u8(want))
    assert as_u8(want)[..., :3].mean() > 5


@needs_ref_shader
@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(__file__), "..", "oracle", "_ref",
                                                    "doge_scene", "buff-doge.obj")),
                    reason="the reference's demo scene was not copied")
def test_oracle_equals_reference_shader_on_its_scene(rt, orc):
    """The reference's own scene, camera and shader against the restatement."""
    tris, mats, sph = rt.load_reference_scene(orc.REF_SCENE_DIR)
    nodes = orc.ref_build_bvh(tris, 1)
    lights = orc.lights_from_materials(tris, mats)
    meta = fixture_meta()["ref_shader_doge_128x96"]
    W, H, F = meta["width"], meta["height"], meta["frames"]
    want = orc.ref_shader_render(tris, mats, nodes, lights, sph, rt.REFERENCE_CAMERA_POS, W, H, F)
    got = oracle_frames(rt, orc, tris, mats, nodes, lights, sph, rt.REFERENCE_CAMERA_POS, W, H, F, False)
    assert np.array_equal(as_u8(got), as_u8(want))
    assert np.array_equal(as_u8(want), np.load(os.path.join(GOLDEN, "ref_shader_doge_128x96.npy")))


@needs_ref_shader
@pytest.mark.parametrize("level,seed", [(5, 2), (6, 3)])
def test_literal_traversal_equals_reference_hit_bvh(rt, orc, level, seed):
    """The shader's own hit_bvh (16-entry stack, both children pushed, t in
    (0.001, 10000)) against the oracle's literal traversal: same hits, same
    t bits, including the rays its stack truncates on these 16- and 18-level
    trees."""
    tris = rt.gen_icosphere(seed, level)
    nodes = orc.ref_build_bvh(tris, 1)
    cam = rt.camera_look_at([0, 0, -3], [0, 0, 0], [0, 1, 0], 40.0, 64, 64)
    rays = np.concatenate([rt.gen_camera_rays(cam, 64, 64), rt.gen_random_rays(5, 8192)])
    rays[:, 3] = 0.001
    rays[:, 7] = 10000.0
    t = orc.ref_shader_trace(tris, nodes, rays)
    lit = orc.trace(tris, nodes, rays, mode=1, stack_size=16)
    hit = lit.view(np.int32)[:, 0] >= 0
    assert np.array_equal(t >= 0, hit)
    assert np.array_equal(t[hit].view(np.uint32), lit[hit, 1].view(np.uint32))


@needs_ref_shader
@pytest.mark.parametrize("seed,n_soup,n_spheres", [(4, 2000, 6), (5, 500, 16), (6, 8000, 3)])
def test_hit_records_equal_reference(rt, orc, seed, n_soup, n_spheres):
    """Full shading hit records (t, p with its 1e-4 offset, normal, material,
    back face) against the shader's own functions:
      * hit_scene (every triangle in index order, then the spheres with
        `closest` reset) = the default culled traversal with
        RT_COMPAT_SPHERE_OVERRIDE: an exact-t tie goes to the lower triangle
        index in both, which the linear loop's strict `t < closest` implies;
      * hit_bvh = the literal 16-entry traversal with RT_COMPAT_NO_SPHERES."""
    t, m, s = rt.gen_cornell(seed, n_soup, n_spheres, 0.2, 1.0)
    nodes = orc.ref_build_bvh(t, 1)
    cam = rt.camera_look_at([0, 0, -14], [0, 0, 0], [0, 1, 0], 40.0, 64, 64)
    rays = np.concatenate([rt.gen_camera_rays(cam, 64, 64), rt.gen_random_rays(7, 8192, -4.0, 4.0)])
    for use_scene, flags in ((True, rt.COMPAT_SPHERE_OVERRIDE), (False, rt.COMPAT_NO_SPHERES | rt.COMPAT_STACK16)):
        ref = orc.ref_shader_hit_records(t, nodes, s, rays, use_scene, len(s))
        got = orc.hit_records(t, nodes, s, rays, flags)
        hit = ref[:, 0] > 0
        assert hit.mean() > 0.5
        assert np.array_equal(ref[:, 0], got[:, 0])
        assert np.array_equal(ref[hit].view(np.uint32), got[hit].view(np.uint32))
