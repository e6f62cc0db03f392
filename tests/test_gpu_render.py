"""GPU render (bounce loop) against the oracle: images within 1e-4 mean
absolute error per channel, using the reference's per-pixel RNG stream."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL = 1e-4  # image MAE per channel


def cornell(rt, ctx, n_soup=12000, n_spheres=4, seed=1):
    t, m, s = rt.gen_cornell(seed, n_soup, n_spheres, 0.2, 1.0)
    sc = ctx.upload_scene(t, m, spheres=s)
    return t, m, s, sc


def gpu_render(sc, cam, W, H, **kw):
    import torch
    accum = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    sc.set_camera(cam)
    sc.render(accum, W, H, **kw)
    sc.ctx.synchronize()
    return accum.cpu().numpy()


def mae(a, b):
    return np.abs(a.astype(np.float64) - b.astype(np.float64)).reshape(-1, 4).mean(axis=0)


def test_render_matches_golden_64(rt, ctx):
    t, m, s, sc = cornell(rt, ctx)
    try:
        cam = rt.camera_look_at([0, 0, -14], [0, 0, 0], [0, 1, 0], 40.0, 64, 64)
        img = gpu_render(sc, cam, 64, 64, spp=1, max_bounces=8)
        gold = np.load(os.path.join(GOLDEN, "render_cornell_64.npy"))
        assert (mae(img, gold) <= TOL).all()
        img = gpu_render(sc, cam, 64, 64, spp=4, max_bounces=8,
                         flags=rt.COMPAT_STACK16 | rt.COMPAT_LEN1 | rt.COMPAT_UNORM8)
        gold = np.load(os.path.join(GOLDEN, "render_cornell_64_compat.npy"))
        assert (mae(img, gold) <= TOL).all()
    finally:
        sc.release()


def test_render_config0_vs_oracle(rt, orc, ctx):
    """Config 0: 256x256, 1 spp, 8 bounces, 12,012 triangles."""
    t, m, s, sc = cornell(rt, ctx, n_spheres=0)
    try:
        cam = rt.camera_look_at([0, 0, -14], [0, 0, 0], [0, 1, 0], 40.0, 256, 256)
        img = gpu_render(sc, cam, 256, 256, spp=1, max_bounces=8)
        want, seg = orc.render(t, m, sc.bvh(), sc.lights(), None, cam.as_array(), 256, 256, spp=1, max_bounces=8)
        err = mae(img, want)
        assert (err <= TOL).all(), err
        assert img[..., 3].min() == 1.0
        # Segment counter = the oracle's count of traced segments.
        ctx.segments(reset=True)
        gpu_render(sc, cam, 256, 256, spp=1, max_bounces=8)
        assert abs(ctx.segments(reset=True) - seg) <= 0.001 * seg
    finally:
        sc.release()


@pytest.mark.parametrize("flags", ["SPHERE_OVERRIDE", "NO_SPHERES", "LEN1", "SHADE_SIMPLE", "UNORM8", "STACK16"])
def test_render_compat_modes(rt, orc, ctx, flags):
    t, m, s, sc = cornell(rt, ctx, n_soup=3000, n_spheres=6, seed=2)
    try:
        f = getattr(rt, "COMPAT_" + flags, None) or getattr(rt, flags)
        cam = rt.camera_look_at([0, 0, -14], [0, 0, 0], [0, 1, 0], 40.0, 96, 80)
        img = gpu_render(sc, cam, 96, 80, spp=2, max_bounces=6, flags=f)
        want, _ = orc.render(t, m, sc.bvh(), sc.lights(), s, cam.as_array(), 96, 80, spp=2, max_bounces=6, flags=f)
        assert (mae(img, want) <= TOL).all()
    finally:
        sc.release()


def test_progressive_accumulation_across_calls(rt, orc, ctx):
    """Two calls of 2 spp (sample_index 0 then 2) equal one 4-spp render."""
    import torch
    t, m, s, sc = cornell(rt, ctx, n_soup=2000, n_spheres=2, seed=3)
    try:
        W, H = 64, 48
        cam = rt.camera_look_at([0, 0, -14], [0, 0, 0], [0, 1, 0], 40.0, W, H)
        sc.set_camera(cam)
        accum = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
        sc.render(accum, W, H, spp=2, max_bounces=8, sample_index=0)
        sc.render(accum, W, H, spp=2, max_bounces=8, sample_index=2)
        ctx.synchronize()
        one = gpu_render(sc, cam, W, H, spp=4, max_bounces=8)
        assert np.array_equal(accum.cpu().numpy(), one)
        want, _ = orc.render(t, m, sc.bvh(), sc.lights(), s, cam.as_array(), W, H, spp=4, max_bounces=8)
        assert (mae(one, want) <= TOL).all()
    finally:
        sc.release()


def test_reference_camera_and_two_bounces(rt, orc, ctx):
    """The reference's own frame setup: UBO camera (comp:357-372), 2 bounces,
    hit_bvh-only path (no spheres), 16-entry stack, lengths of 1."""
    t, m, s, sc = cornell(rt, ctx, n_soup=1410, n_spheres=1, seed=4)
    try:
        W, H = 200, 150
        cam = rt.camera_from_reference([1.8, 8.6, 1.1], W, H)
        f = rt.COMPAT_STACK16 | rt.COMPAT_LEN1 | rt.COMPAT_NO_SPHERES
        img = gpu_render(sc, cam, W, H, spp=3, max_bounces=2, flags=f)
        want, _ = orc.render(t, m, sc.bvh(), sc.lights(), s, cam.as_array(), W, H, spp=3, max_bounces=2, flags=f)
        assert (mae(img, want) <= TOL).all()
    finally:
        sc.release()


def test_render_without_camera_is_an_error(rt, ctx):
    import torch
    t, m, s = rt.gen_cornell(1, 10)
    sc = ctx.upload_scene(t, m)
    try:
        accum = torch.zeros((8, 8, 4), device="cuda")
        with pytest.raises(rt.RtError):
            sc.render(accum, 8, 8)
    finally:
        sc.release()


@pytest.mark.parametrize("flags,spheres,spp", [(0, 6, 3), ("LEN1", 6, 2), ("SPHERE_OVERRIDE", 6, 1),
                                               ("NO_SPHERES", 0, 2), ("UNORM8", 3, 3), ("SHADE_SIMPLE", 3, 1)])
def test_wavefront_equals_megakernel(rt, ctx, flags, spheres, spp):
    """The wavefront split (bounce rays with or without per-bounce Morton
    reordering, cast in place or by the 8-wide caster) gives the
    megakernel's image bit for bit, and counts the same segments."""
    import torch
    f = 0 if flags == 0 else (getattr(rt, "COMPAT_" + flags, None) or getattr(rt, flags))
    t, m, s, sc = cornell(rt, ctx, n_soup=5000, n_spheres=spheres, seed=6)
    keys = ("render.mode", "trace.wide", "trace.wide_min_tris", "render.sort")
    try:
        W, H = 160, 120
        cam = rt.camera_look_at([0, 0, -14], [0, 0, 0], [0, 1, 0], 40.0, W, H)
        out = {}
        old = [ctx.get_tuning(k) for k in keys]
        try:
            for shape in ((0, 0, 0, 0), (1, 0, 0, 1), (1, 1, 0, 1), (1, 0, 0, 0), (1, 1, 0, 0)):
                for k, v in zip(keys, shape):
                    ctx.set_tuning(k, v)
                ctx.segments(reset=True)
                out[shape] = (gpu_render(sc, cam, W, H, spp=spp, max_bounces=7, sample_index=2, flags=f),
                              ctx.segments(reset=True))
        finally:
            for k, v in zip(keys, old):
                ctx.set_tuning(k, v)
        base = out[(0, 0, 0, 0)]
        for shape in ((1, 0, 0, 1), (1, 1, 0, 1), (1, 0, 0, 0), (1, 1, 0, 0)):
            assert np.array_equal(base[0].view(np.uint32), out[shape][0].view(np.uint32)), shape
            assert base[1] == out[shape][1], shape
    finally:
        sc.release()


def test_wavefront_config0_vs_oracle(rt, orc, ctx):
    t, m, s, sc = cornell(rt, ctx, n_spheres=4)
    try:
        old = ctx.get_tuning("render.mode")
        ctx.set_tuning("render.mode", 1)
        try:
            cam = rt.camera_look_at([0, 0, -14], [0, 0, 0], [0, 1, 0], 40.0, 256, 256)
            img = gpu_render(sc, cam, 256, 256, spp=1, max_bounces=8)
        finally:
            ctx.set_tuning("render.mode", old)
        want, _ = orc.render(t, m, sc.bvh(), sc.lights(), s, cam.as_array(), 256, 256, spp=1, max_bounces=8)
        assert (mae(img, want) <= TOL).all()
    finally:
        sc.release()


def test_export_gamma_rgba8(rt, ctx, tmp_path):
    """post-process-shader.frag:67-68: pow(rgb, 1/2.2), alpha 1, 8 bits."""
    import torch
    rng = np.random.default_rng(3)
    img = rng.uniform(-0.2, 1.5, (37, 53, 4)).astype(np.float32)
    img[0, 0, :3] = [0.0, np.nan, np.inf]
    d_in = torch.from_numpy(img).cuda()
    d_out = torch.zeros((37, 53, 4), dtype=torch.uint8, device="cuda")
    rt.export_image(ctx, d_in, 53, 37, d_out, gamma=2.2)
    ctx.synchronize()
    got = d_out.cpu().numpy().astype(np.int32)
    with np.errstate(invalid="ignore"):
        x = np.where(img[..., :3] > 0, np.power(np.maximum(img[..., :3], 0).astype(np.float64), 1 / 2.2), 0.0)
    x = np.nan_to_num(x, nan=0.0, posinf=1.0)
    want = np.rint(np.clip(x, 0, 1) * 255).astype(np.int32)
    assert np.abs(got[..., :3] - want).max() <= 1
    assert (got[..., 3] == 255).all()
    rt.write_ppm(str(tmp_path / "x.ppm"), d_out.cpu().numpy())
    assert (tmp_path / "x.ppm").stat().st_size == 37 * 53 * 3 + len(b"P6\n53 37\n255\n")


@pytest.mark.parametrize("sigma,ksigma,threshold,mix", [(2.0, 2.0, 0.05, 0.5), (1.5, 3.0, 0.2, 1.0),
                                                        (2.0, 0.0, 0.05, 1.0), (0.7, 2.0, 1.0, 1.0)])
def test_denoise_matches_oracle(rt, orc, ctx, sigma, ksigma, threshold, mix):
    """smartDeNoise (post-process-shader.frag:26-68) on a noisy 1-spp render,
    and on a 7x5 image where the radius-4 kernel wraps around every edge
    (REPEAT sampler). Tolerance: libm's and CUDA's expf differ in the last
    ulp, so each weight may differ by ~1e-7 relative."""
    import torch
    t, m, s, sc = cornell(rt, ctx, n_soup=2000, n_spheres=3)
    try:
        cam = rt.camera_look_at([0, 0, -14], [0, 0, 0], [0, 1, 0], 40.0, 64, 48)
        img = gpu_render(sc, cam, 64, 48, spp=1, max_bounces=8)
    finally:
        sc.release()
    small = np.random.default_rng(9).uniform(0, 1, (5, 7, 4)).astype(np.float32)
    for src in (img, small):
        H, W = src.shape[:2]
        d_in = torch.from_numpy(np.ascontiguousarray(src)).cuda()
        d_out = torch.zeros_like(d_in)
        rt.denoise_image(ctx, d_in, W, H, d_out, sigma, ksigma, threshold, mix)
        ctx.synchronize()
        got = d_out.cpu().numpy()
        want = orc.denoise(src, sigma, ksigma, threshold, mix)
        assert np.isfinite(want).all()
        err = np.abs(got.astype(np.float64) - want) / (1.0 + np.abs(want))
        assert err.max() <= 2e-5, err.max()
        if ksigma == 0.0:  # radius 0: the centre tap alone, (w * delta) / delta
            np.testing.assert_allclose(got, src, rtol=1e-6, atol=0)


def test_denoise_rejects_bad_arguments(rt, ctx):
    import torch
    a = torch.zeros((8, 8, 4), device="cuda")
    b = torch.zeros_like(a)
    for args in ((0.0, 2.0, 0.05, 1.0), (2.0, -1.0, 0.05, 1.0), (2.0, 2.0, 0.0, 1.0), (2.0, 2.0, 0.05, 1.5),
                 (10.0, 10.0, 0.05, 1.0)):
        with pytest.raises(rt.RtError):
            rt.denoise_image(ctx, a, 8, 8, b, *args)
    with pytest.raises(rt.RtError):
        rt.denoise_image(ctx, a, 8, 8, a)


def test_autotune_render_sets_split(rt, ctx):
    t, m, s, sc = cornell(rt, ctx, n_soup=3000, n_spheres=2)
    old = (ctx.get_tuning("render.mode"), ctx.get_tuning("render.wavefront_pixels"))
    try:
        sc.set_camera(rt.camera_look_at([0, 0, -14], [0, 0, 0], [0, 1, 0], 40.0, 64, 64))
        px = rt.autotune_render(sc, spp=1, max_bounces=3, max_side=512)
        assert px in (256 * 256, 512 * 512, 1 << 31)
        assert ctx.get_tuning("render.wavefront_pixels") == px
        assert ctx.get_tuning("render.mode") == old[0]
    finally:
        ctx.set_tuning("render.mode", old[0])
        ctx.set_tuning("render.wavefront_pixels", old[1])
        sc.release()


@pytest.mark.parametrize("mode", [0, 1])
def test_partial_tiles_multi_sample_vs_oracle(rt, orc, ctx, mode):
    """A 101x37 image (tiles cut on both axes, so warps hold pixels outside
    the image) with 3 samples per call: the shared camera segment and the
    per-sample bounces match the oracle, megakernel and wavefront alike."""
    t, m, s, sc = cornell(rt, ctx, n_soup=4000, n_spheres=3, seed=4)
    old = ctx.get_tuning("render.mode")
    try:
        ctx.set_tuning("render.mode", mode)
        cam = rt.camera_look_at([0.5, 0.3, -14], [0, 0, 0], [0, 1, 0], 40.0, 101, 37)
        img = gpu_render(sc, cam, 101, 37, spp=3, max_bounces=8, sample_index=1)
        want, _ = orc.render(t, m, sc.bvh(), sc.lights(), s, cam.as_array(), 101, 37, spp=3, max_bounces=8,
                             sample_index=1)
        assert (mae(img, want) <= TOL).all()
    finally:
        ctx.set_tuning("render.mode", old)
        sc.release()


def _ref_fixture(name):
    import json
    with open(os.path.join(GOLDEN, "ref_shader.json")) as f:
        meta = json.load(f)[name]
    return meta, np.load(os.path.join(GOLDEN, name + ".npy"))


def _compat_frames(rt, sc, meta, all_lights):
    """The GPU kernels in the reference's own configuration, frame by frame."""
    import torch
    flags = rt.COMPAT_STACK16 | rt.COMPAT_NO_SPHERES | rt.COMPAT_UNORM8 | (0 if all_lights else rt.COMPAT_LEN1)
    if meta.get("shader") == "simple":
        flags |= rt.SHADE_SIMPLE
    W, H = meta["width"], meta["height"]
    sc.set_camera(rt.camera_from_reference(meta["cam_pos"], W, H))
    acc = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    for s in range(meta["frames"]):
        sc.render(acc, W, H, spp=1, max_bounces=meta["max_bounces"], sample_index=s, flags=flags)
    sc.ctx.synchronize()
    return np.rint(acc.cpu().numpy().astype(np.float64) * 255.0).astype(np.uint8)


@pytest.mark.parametrize("name", ["ref_shader_cornell_96x64", "ref_shader_cornell_96x64_lights",
                                  "ref_shader_simple_cornell_96x64"])
def test_kernels_match_reference_shader(rt, ctx, name):
    """Against images made by the reference's own compute shader (compiled on
    the host from its source): the GPU kernels in compat mode, through the
    GPU-built Bvh.h tree. Tolerance: CUDA's sinf/cosf and libm's differ in
    the last ulp, which can move a bounce direction; pixel values are rgba8."""
    meta, want = _ref_fixture(name)
    t, m, _ = rt.gen_cornell(3, 3000, 0)
    m = m.copy()
    m[:, 1] = 0.0
    sc = ctx.upload_scene(t, m)
    try:
        got = _compat_frames(rt, sc, meta, meta["lights"] == "all")
    finally:
        sc.release()
    exact = (got == want).all(axis=2).mean()
    err = np.abs(got.astype(np.float64) - want) / 255.0
    assert exact >= 0.99, exact
    assert (err.reshape(-1, 4).mean(axis=0) <= TOL).all(), err.reshape(-1, 4).mean(axis=0)


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(__file__), "..", "oracle", "_ref",
                                                    "doge_scene", "buff-doge.obj")),
                    reason="the reference's demo scene was not copied")
def test_kernels_match_reference_shader_on_its_scene(rt, orc, ctx):
    meta, want = _ref_fixture("ref_shader_doge_128x96")
    tris, mats, sph = rt.load_reference_scene(orc.REF_SCENE_DIR)
    sc = ctx.upload_scene(tris, mats, spheres=sph)
    try:
        got = _compat_frames(rt, sc, meta, False)
    finally:
        sc.release()
    exact = (got == want).all(axis=2).mean()
    err = np.abs(got.astype(np.float64) - want) / 255.0
    assert exact >= 0.99, exact
    assert (err.reshape(-1, 4).mean(axis=0) <= TOL).all(), err.reshape(-1, 4).mean(axis=0)


@pytest.mark.parametrize("mode", [1, 0], ids=["wavefront", "megakernel"])
def test_large_scene_8m_vs_oracle(rt, orc, ctx, mode):
    """The progressive 1080p configuration's 8,000,004-triangle scene (6x6
    flattened displaced level-7 icospheres + the Cornell box, 40% glass, 30%
    metal, 30% lambertian) at a 128x72 view of the same camera, 2 spp, 8
    bounces. The wavefront casts its bounce rays with the 8-wide caster
    here (the scene is far above trace.wide_min_tris), so that path is
    checked at scale against the oracle on the GPU-built tree."""
    t, m = rt.gen_grid(4, 6, 6, 7, 0.35, 0.05, 222222, 3.0)
    sc = ctx.upload_scene(t, m)
    old = ctx.get_tuning("render.mode")
    try:
        assert sc.info().triangles == 8000004
        cam = rt.camera_look_at([0, 2, -40], [0, -6, 0], [0, 1, 0], 40.0, 128, 72)
        ctx.set_tuning("render.mode", mode)
        img = gpu_render(sc, cam, 128, 72, spp=2, max_bounces=8)
        want, _ = orc.render(t, m, sc.bvh(), sc.lights(), None, cam.as_array(), 128, 72, spp=2, max_bounces=8)
        err = mae(img, want)
        assert (err <= TOL).all(), err
        assert img[..., :3].max() > 0.0
    finally:
        ctx.set_tuning("render.mode", old)
        sc.release()
