"""The GPU's 8-wide closest-hit traversal checked on the host.

The oracle restates the fold (oracle_wide_fold: the GPU builder's
largest-first rule and its SAH-chosen nodes) and the traversal (oracle_trace_wide: the kernel's fp32 plane
arithmetic on quantized nodes, near-first order, the triangle-index tie
rule); the nodes are quantized by the library's own host quantizer
(rtgbQuantizeNode8, the function the upload runs on the GPU). The hits
must equal the oracle's culled binary traversal bit for bit: pruning by
8-bit boxes rounded outward never drops the closest hit. Leaves are tested
as soon as they are reached (the kernel collects them in a shared pool
first), which prunes harder and so checks the containment more strictly."""
import numpy as np
import pytest


def quantize_all(rt, boxes, refs, fmask):
    words = np.zeros((len(boxes), 24), np.uint32)
    out = np.zeros(24, np.uint32)
    for i in range(len(boxes)):
        b = np.ascontiguousarray(boxes[i], np.float32)
        r = np.ascontiguousarray(refs[i], np.int32)
        assert rt.LIB.rtgbQuantizeNode8(b.ctypes.data, r.ctypes.data, int(fmask[i]), out.ctypes.data) == 1
        words[i] = out
    return words


def wide_hits(rt, orc, tris, nodes, rays, stats=False, sah=False):
    boxes, refs, fmask, levels = orc.wide_fold(nodes, sah)
    assert levels >= 1 and (fmask >= 1).all() and (fmask <= 255).all()
    # Every triangle sits in exactly one leaf slot; empty slots match the mask.
    empty = refs == np.iinfo(np.int32).min
    bits = (fmask[:, None] >> np.arange(8, dtype=np.uint32)[None, :]) & 1
    assert np.array_equal(empty, bits == 0)
    leaves = refs[(refs < 0) & ~empty]
    assert sorted((~leaves).tolist()) == list(range(len(tris)))
    words = quantize_all(rt, boxes, refs, fmask)
    assert np.array_equal(words[:, 3] >> 24, fmask)
    root_box = np.concatenate([nodes[0, 0:3], nodes[0, 4:7]]).astype(np.float32)
    return orc.trace_wide(tris, words, 0, root_box, rays, stats=stats)


def check(rt, orc, tris, rays):
    """Both folds: largest child first and SAH-chosen nodes."""
    nodes, _ = orc.build_bvh(tris, 1)
    want = orc.trace(tris, nodes, rays)
    for sah in (False, True):
        got = wide_hits(rt, orc, tris, nodes, rays, sah=sah)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), sah
    assert (want.view(np.int32)[:, 0] >= 0).mean() > 0.2


def test_sah_fold_visits_fewer_nodes(rt, orc):
    """The SAH-chosen fold of the closest-hit mesh family has fewer nodes
    and costs incoherent rays fewer node visits than largest-first."""
    tris = rt.gen_icosphere(1, 6)
    nodes, _ = orc.build_bvh(tris, 1)
    rays = rt.gen_random_rays(3, 8192)
    visits = []
    for sah in (False, True):
        boxes, _, _, _ = orc.wide_fold(nodes, sah)
        _, st = wide_hits(rt, orc, tris, nodes, rays, stats=True, sah=sah)
        visits.append((len(boxes), st[:, 0].mean()))
    assert visits[1][0] < visits[0][0]
    assert visits[1][1] < 0.97 * visits[0][1], visits


def test_icosphere_camera_and_random(rt, orc):
    tris = rt.gen_icosphere(2, 5)
    cam = rt.camera_look_at([0, 0, -3], [0, 0, 0], [0, 1, 0], 40.0, 96, 96)
    rays = np.concatenate([rt.gen_camera_rays(cam, 96, 96), rt.gen_random_rays(5, 20000)])
    check(rt, orc, tris, rays)


def test_cornell_rays_from_inside(rt, orc):
    t, _, _ = rt.gen_cornell(3, 4000, 0)
    rays = rt.gen_random_rays(7, 20000, -4.0, 4.0)
    check(rt, orc, t, rays)


@pytest.mark.parametrize("offset,scale", [((1000.0, -2000.0, 500.0), 10.0), ((-3.0e4, 0.0, 7.0), 1.0),
                                          ((0.0, 0.0, 0.0), 1e-3)])
def test_offset_and_scaled_mesh(rt, orc, offset, scale):
    tris = rt.gen_icosphere(4, 4).copy()
    off = np.array(offset, np.float32)
    for v in range(3):
        tris[:, 4 * v:4 * v + 3] = tris[:, 4 * v:4 * v + 3] * np.float32(scale) + off
    rays = rt.gen_random_rays(9, 8000).copy()
    rays[:, 0:3] = rays[:, 0:3] * np.float32(scale) + off
    rays[:, 3] = 0.0
    check(rt, orc, tris, rays)


def test_axis_aligned_rays(rt, orc):
    """Direction components of exactly 0 take the clamped 1/d path."""
    tris = rt.gen_icosphere(6, 4)
    rng = np.random.default_rng(3)
    n = 6000
    rays = np.zeros((n, 8), np.float32)
    axis = rng.integers(0, 3, n)
    sign = rng.choice([-1.0, 1.0], n)
    rays[:, 0:3] = rng.uniform(-0.8, 0.8, (n, 3))
    rays[np.arange(n), axis] = -1.5 * sign
    rays[np.arange(n), 4 + axis] = sign
    rays[:, 3] = 1e-4
    rays[:, 7] = np.inf
    check(rt, orc, tris, rays)


def test_deep_tree_bench_mesh_family(rt, orc):
    """The displaced icosphere of the closest-hit workload at level 7
    (327,680 triangles, a fold of ~11 levels), camera and random rays."""
    tris = rt.gen_icosphere(1, 7)
    cam = rt.camera_look_at([0, 0, -3], [0, 0, 0], [0, 1, 0], 40.0, 64, 64)
    rays = np.concatenate([rt.gen_camera_rays(cam, 64, 64), rt.gen_random_rays(3, 8192)])
    check(rt, orc, tris, rays)


def test_model_detects_shrunk_boxes(rt, orc):
    """Sensitivity: the same traversal over boxes shrunk by one grid step
    (every upper byte lowered by 1, a non-conservative quantization) must
    lose hits; the check above would catch a quantizer that rounds inward."""
    tris = rt.gen_icosphere(2, 5)
    nodes, _ = orc.build_bvh(tris, 1)
    rays = rt.gen_random_rays(5, 20000)
    want = orc.trace(tris, nodes, rays)
    boxes, refs, fmask, _ = orc.wide_fold(nodes)
    words = quantize_all(rt, boxes, refs, fmask)
    for wi in range(10, 16):  # the qhi words
        w = words[:, wi].copy()
        out = np.zeros_like(w)
        for b in range(4):
            byte = (w >> np.uint32(8 * b)) & np.uint32(0xFF)
            byte = np.where(byte > 0, byte - 1, byte)
            out |= byte << np.uint32(8 * b)
        words[:, wi] = out
    root_box = np.concatenate([nodes[0, 0:3], nodes[0, 4:7]]).astype(np.float32)
    got = orc.trace_wide(tris, words, 0, root_box, rays)
    assert not np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_octant_slots_equal_library(rt, orc):
    """The fold's slot placement: the library's host function (the one the
    GPU fold runs) equals the oracle's restatement on random child sets,
    and children go to distinct slots."""
    rng = np.random.default_rng(11)
    got = np.zeros(8, np.int32)
    for trial in range(3000):
        cnt = int(rng.integers(1, 9))
        lo = rng.normal(0, 1, (cnt, 3)).astype(np.float32)
        hi = (lo + rng.uniform(0, 0.5, (cnt, 3))).astype(np.float32)
        if trial % 7 == 0:
            lo[:] = lo[0]  # identical boxes: every cost ties
            hi[:] = hi[0]
        boxes = np.ascontiguousarray(np.concatenate([lo, hi], 1), np.float32)
        want = orc.octant_slots(boxes)
        assert rt.LIB.rtgbAssignOctantSlots(boxes.ctypes.data, cnt, got.ctypes.data) == 1
        assert np.array_equal(got[:cnt], want)
        assert len(set(want.tolist())) == cnt and (want >= 0).all() and (want < 8).all()


def test_octant_order_visits_fewer_nodes_than_slot_order(rt, orc):
    """The octant placement is what makes the rank order near-first: on the
    bench mesh family the model visits no more nodes than with children
    left in fold order would allow (sanity bound on the work, not results)."""
    tris = rt.gen_icosphere(1, 6)
    nodes, _ = orc.build_bvh(tris, 1)
    rays = rt.gen_random_rays(3, 8192)
    got, st = wide_hits(rt, orc, tris, nodes, rays, stats=True)
    want = orc.trace(tris, nodes, rays)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # An 8-wide step replaces about three binary levels.
    _, bst = orc.trace(tris, nodes, rays, slack=0.0, stats=True)
    assert st[:, 0].mean() < 0.5 * bst[:, 0].mean()
