"""Batched rendering: many scenes of uneven size in one persistent launch.
Each job's image must equal the job rendered alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def scenes(rt, ctx, specs):
    out = []
    for seed, n_soup, n_sph in specs:
        t, m, s = rt.gen_cornell(seed, n_soup, n_sph, 0.2, 1.0)
        out.append(ctx.upload_scene(t, m, spheres=s))
    return out


SPECS = [(31, 200, 0), (32, 3000, 4), (33, 20000, 16), (34, 1000, 2), (35, 60000, 8)]
SIZES = [(64, 48), (128, 128), (96, 80), (40, 200), (160, 96)]


@pytest.fixture(params=[(1, 16), (1 << 20, 4)], ids=["all-wavefront", "tiles+sides"])
def batch_split(request, ctx):
    """Both ways a batch can share its jobs out (render.batch_wavefront_pixels,
    render.batch_streams): every job a wavefront on 16 side streams (the
    default), and jobs below 2^20 pixels in the persistent tile launch with
    the rest on 4 side streams."""
    keys = ("render.batch_wavefront_pixels", "render.batch_streams")
    old = [ctx.get_tuning(k) for k in keys]
    for k, v in zip(keys, request.param):
        ctx.set_tuning(k, v)
    yield request.param
    for k, v in zip(keys, old):
        ctx.set_tuning(k, v)


def render_alone(ctx, sc, cam, W, H, spp, bounces, flags=0, sample_index=0):
    import torch
    acc = torch.zeros((H, W, 4), device="cuda")
    sc.set_camera(cam)
    sc.render(acc, W, H, spp=spp, max_bounces=bounces, flags=flags, sample_index=sample_index)
    ctx.synchronize()
    return acc.cpu().numpy()


def test_batch_equals_individual_renders(rt, ctx, batch_split):
    import torch
    scs = scenes(rt, ctx, SPECS)
    try:
        jobs, accs, want = [], [], []
        for i, (sc, (W, H)) in enumerate(zip(scs, SIZES)):
            cam = rt.camera_look_at([0.3 * i, 0.2, -14], [0, 0, 0], [0, 1, 0], 40.0, W, H)
            spp, bounces = 1 + i % 3, 3 + i
            flags = rt.COMPAT_LEN1 if i == 3 else 0
            acc = torch.zeros((H, W, 4), device="cuda")
            accs.append(acc)
            jobs.append(rt.make_job(sc, cam, acc, W, H, spp, bounces, 0, flags))
            want.append(render_alone(ctx, sc, cam, W, H, spp, bounces, flags))
        ctx.segments(reset=True)
        ctx.render_batch(jobs)
        ctx.synchronize()
        assert ctx.segments(reset=True) > 0
        for a, w in zip(accs, want):
            assert np.array_equal(a.cpu().numpy().view(np.uint32), w.view(np.uint32))
    finally:
        for sc in scs:
            sc.release()


def test_batch_graph_progressive_frames(rt, ctx, batch_split):
    """Three graph replays (launch + device-side sample advance) equal one
    render of three times the samples."""
    import torch
    scs = scenes(rt, ctx, SPECS[:3])
    try:
        jobs, accs, want = [], [], []
        for i, (sc, (W, H)) in enumerate(zip(scs, SIZES)):
            cam = rt.camera_look_at([0, 0, -14], [0, 0, 0], [0, 1, 0], 40.0, W, H)
            acc = torch.zeros((H, W, 4), device="cuda")
            accs.append(acc)
            jobs.append(rt.make_job(sc, cam, acc, W, H, 2, 6))
            want.append(render_alone(ctx, sc, cam, W, H, 6, 6))
        b = ctx.batch(jobs)
        try:
            for _ in range(3):
                b.launch_graph()
            ctx.synchronize()
        finally:
            b.destroy()
        for a, w in zip(accs, want):
            assert np.array_equal(a.cpu().numpy().view(np.uint32), w.view(np.uint32))
    finally:
        for sc in scs:
            sc.release()


@pytest.mark.parametrize("mode", [1, 2])
def test_hybrid_batch_with_wavefront_jobs(rt, ctx, mode):
    """With the batch split at 2^20 pixels, the wavefront jobs (all of them
    in render.mode 1; the 1024x1024 one in mode 2) run on side streams next
    to the persistent launch over the others; every image equals the job
    alone, for a direct launch and for three progressive graph replays."""
    import torch
    scs = scenes(rt, ctx, SPECS[:3])
    sizes = [(1024, 1024), (128, 96), (200, 40)]
    old = ctx.get_tuning("render.mode")
    old_split = ctx.get_tuning("render.batch_wavefront_pixels")
    ctx.set_tuning("render.mode", mode)
    ctx.set_tuning("render.batch_wavefront_pixels", 1 << 20)
    try:
        jobs, accs, want, want3 = [], [], [], []
        for i, (sc, (W, H)) in enumerate(zip(scs, sizes)):
            cam = rt.camera_look_at([0.2 * i, 0.1, -14], [0, 0, 0], [0, 1, 0], 40.0, W, H)
            acc = torch.zeros((H, W, 4), device="cuda")
            accs.append(acc)
            jobs.append(rt.make_job(sc, cam, acc, W, H, 1, 5))
            want.append(render_alone(ctx, sc, cam, W, H, 1, 5))
            want3.append(render_alone(ctx, sc, cam, W, H, 3, 5))
        ctx.render_batch(jobs)
        ctx.synchronize()
        for a, w in zip(accs, want):
            assert np.array_equal(a.cpu().numpy().view(np.uint32), w.view(np.uint32))
        for a in accs:
            a.zero_()
        b = ctx.batch(jobs)
        try:
            for _ in range(3):
                b.launch_graph()
            ctx.synchronize()
        finally:
            b.destroy()
        for a, w in zip(accs, want3):
            assert np.array_equal(a.cpu().numpy().view(np.uint32), w.view(np.uint32))
    finally:
        ctx.set_tuning("render.mode", old)
        ctx.set_tuning("render.batch_wavefront_pixels", old_split)
        for sc in scs:
            sc.release()


def test_batch_rejects_bad_jobs(rt, ctx):
    import torch
    t, m, s = rt.gen_cornell(1, 10)
    sc = ctx.upload_scene(t, m)
    try:
        cam = rt.camera_look_at([0, 0, -14], [0, 0, 0], [0, 1, 0], 40.0, 8, 8)
        acc = torch.zeros((8, 8, 4), device="cuda")
        good = rt.make_job(sc, cam, acc, 8, 8)
        bad = rt.RenderJob(9999, 0, cam, rt.RenderParams(8, 8, 1, 8, 0, 0), acc.data_ptr())
        with pytest.raises(rt.RtError):
            ctx.render_batch([good, bad])
        zero = rt.make_job(sc, cam, acc, 0, 8)
        with pytest.raises(rt.RtError):
            ctx.render_batch([zero])
    finally:
        sc.release()
