"""Render server: continuous batching under an HBM budget with LRU
eviction. Every result must equal the same request rendered alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def serve_mod():
    from rtgb import serve
    return serve


def scene_data(rt, seed, n_soup, n_sph):
    return rt.gen_cornell(seed, n_soup, n_sph, 0.2, 1.0)


def alone(rt, ctx, data, cam, W, H, spp, bounces):
    import torch
    t, m, s = data
    sc = ctx.upload_scene(t, m, spheres=s)
    try:
        acc = torch.zeros((H, W, 4), device="cuda")
        sc.set_camera(cam)
        old = ctx.get_tuning("render.mode")
        ctx.set_tuning("render.mode", 0)
        try:
            sc.render(acc, W, H, spp=spp, max_bounces=bounces)
            ctx.synchronize()
        finally:
            ctx.set_tuning("render.mode", old)
        return acc.cpu().numpy()
    finally:
        sc.release()


REQS = [(0, 64, 48, 5, 8), (1, 96, 64, 3, 6), (2, 80, 80, 7, 8), (0, 32, 128, 2, 4), (3, 128, 96, 4, 8),
        (1, 48, 48, 9, 3), (2, 100, 60, 1, 8)]


@pytest.mark.parametrize("max_active,spp_step,mode,split", [(0, 2, 2, 1 << 20), (3, 1, 2, 1 << 20), (1, 0, 2, 1),
                                                            (0, 2, 1, 1), (5, 3, 1, 1), (5, 3, 2, 1)])
def test_results_equal_alone_in_the_mix(rt, ctx, serve_mod, max_active, spp_step, mode, split):
    """The default split (render.batch_wavefront_pixels 1) and render.mode 1
    send every request through the wavefront side streams (several at
    once); a split at 2^20 pixels sends these sizes through the persistent
    launch."""
    datas = [scene_data(rt, 40 + i, n, k) for i, (n, k) in enumerate([(500, 2), (3000, 0), (8000, 5), (1500, 1)])]
    old_mode = ctx.get_tuning("render.mode")
    old_split = ctx.get_tuning("render.batch_wavefront_pixels")
    ctx.set_tuning("render.mode", mode)
    ctx.set_tuning("render.batch_wavefront_pixels", split)
    try:
        run_mix(rt, ctx, serve_mod, datas, max_active, spp_step)
    finally:
        ctx.set_tuning("render.mode", old_mode)
        ctx.set_tuning("render.batch_wavefront_pixels", old_split)


def run_mix(rt, ctx, serve_mod, datas, max_active, spp_step):
    with serve_mod.Server(ctx, max_active=max_active, spp_per_step=spp_step) as srv:
        handles = [srv.add_scene(*d) for d in datas]
        ids, specs = [], []
        for i, (si, W, H, spp, b) in enumerate(REQS):
            cam = rt.camera_look_at([0.5 * i - 1.0, 0.3, -14], [0, 0, 0], [0, 1, 0], 40.0, W, H)
            ids.append(srv.submit(handles[si], cam, W, H, spp, b))
            specs.append((si, cam, W, H, spp, b))
        for rid in ids:
            st = srv.wait(rid, 60000)
            assert st.state == serve_mod.DONE, st.error
            assert st.done_ms >= st.start_ms >= st.submit_ms
        stats = srv.stats()
        assert stats.completed == len(REQS) and stats.failed == 0
        assert stats.p99_ms >= stats.p50_ms > 0
        for rid, (si, cam, W, H, spp, b) in zip(ids, specs):
            want = alone(rt, ctx, datas[si], cam, W, H, spp, b)
            assert np.array_equal(srv.image(rid).view(np.uint32), want.view(np.uint32))


def test_budget_eviction_and_isolation(rt, ctx, serve_mod):
    """A budget that holds about two scenes: requests cycling over four
    scenes force LRU evictions and re-uploads; results stay exact; a request
    larger than the whole budget fails alone."""
    datas = [scene_data(rt, 60 + i, 20000, 0) for i in range(4)]
    one_scene = 20012 * (48 + 48 * 2 + 64 + 48 + 4) + 64 * 1024
    budget = int(2.5 * one_scene)
    with serve_mod.Server(ctx, hbm_budget_bytes=budget, max_active=1, spp_per_step=1) as srv:
        handles = [srv.add_scene(*d) for d in datas]
        cams = [rt.camera_look_at([0, 0, -14], [0, 0, 0], [0, 1, 0], 40.0, 32, 32) for _ in range(4)]
        ids = [srv.submit(handles[i % 4], cams[i % 4], 32, 32, 2, 5) for i in range(8)]
        huge = srv.submit(handles[0], cams[0], 4096, 4096, 1, 1)  # 256 MB image > budget
        for rid in ids:
            assert srv.wait(rid, 60000).state == serve_mod.DONE
        assert srv.wait(huge, 60000).state == serve_mod.FAILED
        st = srv.stats()
        assert st.scene_evictions >= 4 and st.scene_uploads >= 6
        assert st.resident_bytes <= budget
        want = alone(rt, ctx, datas[1], cams[1], 32, 32, 2, 5)
        assert np.array_equal(srv.image(ids[1]).view(np.uint32), want.view(np.uint32))


def test_bad_requests_are_rejected(rt, ctx, serve_mod):
    with serve_mod.Server(ctx) as srv:
        h = srv.add_scene(*scene_data(rt, 1, 100, 0))
        cam = rt.camera_look_at([0, 0, -14], [0, 0, 0], [0, 1, 0], 40.0, 8, 8)
        with pytest.raises(rt.RtError):
            srv.submit(h + 5, cam, 8, 8, 1)
        with pytest.raises(rt.RtError):
            srv.submit(h, cam, 0, 8, 1)
        rid = srv.submit(h, cam, 8, 8, 1)
        assert srv.wait(rid, 30000).state == serve_mod.DONE
