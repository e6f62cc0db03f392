"""The reference's own demo scene (src/ray-tracing/RtScene.h:44-101, 1,422
triangles from its OBJ files, one glass sphere) through the product path:
loaded by rtLoadReferenceScene, its tree built on the GPU node-for-node as
Bvh.h builds it, and rendered from the reference's starting camera
(src/main.cpp:37) within the image tolerance of the oracle. Also an OBJ
written here, loaded and traced, so the loader is covered on every box."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-4


def gpu_render(sc, cam, W, H, **kw):
    import torch
    accum = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    sc.set_camera(cam)
    sc.render(accum, W, H, **kw)
    sc.ctx.synchronize()
    return accum.cpu().numpy()


def mae(a, b):
    return np.abs(a.astype(np.float64) - b.astype(np.float64)).reshape(-1, 4).mean(axis=0)


def test_obj_scene_traces_like_oracle(rt, orc, ctx, tmp_path):
    # An icosphere written as OBJ with shared vertices and mixed index forms.
    tris = rt.gen_icosphere(3, 4)
    verts, index = {}, []
    for row in tris:
        for j in range(3):
            key = tuple(row[4 * j:4 * j + 3].tolist())
            index.append(verts.setdefault(key, len(verts)))
    lines = ["o ico"] + ["v %r %r %r" % k for k in verts]
    forms = ["%d", "%d/1", "%d//1", "%d/1/1"]
    for f in range(len(tris)):
        a, b, c = (index[3 * f + j] + 1 for j in range(3))
        lines.append("f " + " ".join(forms[(f + j) % 4] % v for j, v in enumerate((a, b, c))))
    path = tmp_path / "ico.obj"
    path.write_text("\n".join(lines) + "\n")
    loaded = rt.load_obj(str(path), material=0)
    np.testing.assert_array_equal(loaded.view(np.uint32), tris.view(np.uint32))
    mats = rt.gen_cornell(1, 0)[1]
    sc = ctx.upload_scene(loaded, mats)
    try:
        cam = rt.camera_look_at([0, 0, -3], [0, 0, 0], [0, 1, 0], 40.0, 64, 64)
        rays = np.concatenate([rt.gen_camera_rays(cam, 64, 64), rt.gen_random_rays(3, 4096)])
        got = sc.trace_host(rays)
        want = orc.trace(loaded, sc.bvh(), rays)
        np.testing.assert_array_equal(got.view(np.int32)[:, 0], want.view(np.int32)[:, 0])
        assert (got.view(np.int32)[:, 0] >= 0).mean() > 0.3
    finally:
        sc.release()


needs_scene = pytest.mark.skipif(
    not os.path.exists(os.path.join(os.path.dirname(__file__), "..", "oracle", "_ref", "doge_scene",
                                    "buff-doge.obj")),
    reason="the reference's demo scene was not copied (no reference checkout)")


@needs_scene
def test_reference_scene_tree_and_render(rt, orc, ctx):
    tris, mats, sph = rt.load_reference_scene(orc.REF_SCENE_DIR)
    sc = ctx.upload_scene(tris, mats, spheres=sph)
    try:
        want_nodes, depth = orc.build_bvh(tris, 1)
        got = sc.bvh()
        cols = [0, 1, 2, 4, 5, 6, 7, 8, 9]
        np.testing.assert_array_equal(got.view(np.uint32)[:, cols], want_nodes.view(np.uint32)[:, cols])
        assert sc.info().depth == depth
        np.testing.assert_array_equal(sc.lights().view(np.uint32), orc.lights_from_materials(tris, mats).view(np.uint32))
        W, H = 160, 128
        cam = rt.camera_from_reference(rt.REFERENCE_CAMERA_POS, W, H)
        img = gpu_render(sc, cam, W, H, spp=2, max_bounces=8)
        want, _ = orc.render(tris, mats, want_nodes, sc.lights(), sph, cam.as_array(), W, H, spp=2, max_bounces=8)
        err = mae(img, want)
        assert (err <= TOL).all(), err
        assert img[..., :3].mean() > 0.0  # the camera sees lit geometry
    finally:
        sc.release()
