"""GPU closest-hit casting against the oracle.

Bar (stated in the workload spec): closest-hit triangle indices bit-exact
except rays whose two nearest candidates lie within 1e-6 relative t; t and the
barycentrics within 1e-5 relative of the fp64 oracle. By default the library
re-evaluates the winning triangle in fp64, so where the fp64 oracle picks the
same triangle its t, u, v rounded to fp32 are returned exactly; with
RT_HIT_FP32 the values are bit-exact with the fp32 oracle instead.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def gpu_trace(ctx, sc, rays, flags=0):
    import torch
    d_rays = dev(rays)
    d_hits = torch.zeros((len(rays), 4), dtype=torch.float32, device="cuda")
    sc.trace(d_rays, len(rays), d_hits, flags=flags)
    ctx.synchronize()
    return d_hits.cpu().numpy()


def compare_index(gpu, want, ties):
    gi, wi = gpu.view(np.int32)[:, 0], want.view(np.int32)[:, 0]
    ok = ties | (gi == wi)
    assert ok.all(), f"{(~ok).sum()} hit-index mismatches outside ties"


def compare(gpu, want, ties):
    compare_index(gpu, want, ties)
    gi, wi = gpu.view(np.int32)[:, 0], want.view(np.int32)[:, 0]
    same = (~ties) & (gi == wi)
    assert np.array_equal(gpu[same].view(np.uint32), want[same].view(np.uint32)), "t/u/v not bit-exact"


def mesh_scene(rt, ctx, level, seed):
    tris = rt.gen_icosphere(seed, level)
    mats = rt.gen_cornell(1, 0)[1]
    return tris, ctx.upload_scene(tris, mats)


def test_trace_small_mesh_matches_golden(rt, orc, ctx):
    tris, sc = mesh_scene(rt, ctx, 5, 2)
    try:
        cam = rt.camera_look_at([0, 0, -3], [0, 0, 0], [0, 1, 0], 40.0, 64, 64)
        rays = np.concatenate([rt.gen_camera_rays(cam, 64, 64), rt.gen_random_rays(5, 4096)])
        gold = np.load(os.path.join(GOLDEN, "trace_icosphere_l5.npy"))
        nodes = sc.bvh()
        _, st = orc.trace(tris, nodes, rays, stats=True)
        ties = (st[:, 2] & 1) != 0
        compare(gpu_trace(ctx, sc, rays, flags=rt.HIT_FP32), gold, ties)
        # Default: t, u, v are the fp64 oracle's values rounded to fp32.
        got = gpu_trace(ctx, sc, rays)
        compare_index(got, gold, ties)
        tri64, tuv = orc.trace_f64(tris, nodes, rays)
        gi = got.view(np.int32)[:, 0]
        agree = (gi == tri64) & (gi >= 0)
        assert agree.sum() > 0.9 * (gi >= 0).sum()
        assert np.array_equal(got[agree, 1:4], tuv[agree].astype(np.float32))
        # Host-array entry point gives the same bits.
        host = sc.trace_host(rays)
        assert np.array_equal(host.view(np.uint32), gpu_trace(ctx, sc, rays).view(np.uint32))
    finally:
        sc.release()


def test_trace_stack16_compat(rt, ctx):
    tris, sc = mesh_scene(rt, ctx, 5, 2)
    try:
        cam = rt.camera_look_at([0, 0, -3], [0, 0, 0], [0, 1, 0], 40.0, 64, 64)
        rays = np.concatenate([rt.gen_camera_rays(cam, 64, 64), rt.gen_random_rays(5, 4096)])
        gold = np.load(os.path.join(GOLDEN, "trace_icosphere_l5_stack16.npy"))
        got = gpu_trace(ctx, sc, rays, flags=rt.COMPAT_STACK16)
        assert np.array_equal(got.view(np.uint32), gold.view(np.uint32))
    finally:
        sc.release()


@pytest.fixture(scope="module")
def big_mesh(rt, ctx):
    tris, sc = mesh_scene(rt, ctx, 8, 1)
    yield tris, sc
    sc.release()


@pytest.fixture(scope="module")
def config1_oracle(rt, orc, big_mesh):
    """Both closest-hit batches at full size (2 x 4,194,304 rays) and the
    fp32 oracle's hits for every ray (culled traversal of the reference tree;
    stats flag the rays whose two nearest candidates lie within 1e-6
    relative t)."""
    tris, sc = big_mesh
    cam = rt.camera_look_at([0, 0, -3], [0, 0, 0], [0, 1, 0], 40.0, 2048, 2048)
    batches = {"coherent": rt.gen_camera_rays(cam, 2048, 2048), "incoherent": rt.gen_random_rays(3, 4194304)}
    nodes = sc.bvh()
    out = {}
    for name, rays in batches.items():
        want, st = orc.trace(tris, nodes, rays, stats=True)
        out[name] = (rays, want, (st[:, 2] & 1) != 0)
    return nodes, out


def test_trace_config1_full_batch_vs_oracle(rt, orc, ctx, big_mesh, config1_oracle):
    """Every ray of both batches against the fp32 oracle: hit indices equal
    outside ties (0 mismatches); t, u, v within 1e-5 relative of the fp64
    oracle on one ray in 16; RT_HIT_FP32 bit-exact with the fp32 oracle on
    one ray in 16."""
    tris, sc = big_mesh
    nodes, batches = config1_oracle
    for name, (rays, want, ties) in batches.items():
        got = gpu_trace(ctx, sc, rays)
        gi, wi = got.view(np.int32)[:, 0], want.view(np.int32)[:, 0]
        mismatch = int(((gi != wi) & ~ties).sum())
        print(f"{name}: {len(rays)} rays, {mismatch} index mismatches outside ties, "
              f"tie fraction {ties.mean():.3e}, hit fraction {(gi >= 0).mean():.4f}")
        assert mismatch == 0, f"{name}: {mismatch} hit-index mismatches outside ties"
        assert ties.mean() < 0.01
        # t, u, v against the fp64 oracle where both pick the same triangle.
        sub = np.arange(0, len(rays), 16)
        tri64, tuv = orc.trace_f64(tris, nodes, rays[sub])
        gs = got[sub]
        gsi = gs.view(np.int32)[:, 0]
        agree = (gsi == tri64) & (gsi >= 0)
        assert agree.sum() >= 0.999 * ((gsi >= 0) & ~ties[sub]).sum()
        for col in range(3):
            ref = tuv[agree, col]
            rel = np.abs(gs[agree, 1 + col].astype(np.float64) - ref) / np.maximum(np.abs(ref), 1e-30)
            print(f"{name}: max relative error of {'tuv'[col]} vs fp64: {rel.max():.3e}")
            assert rel.max() <= 1e-5, (name, col, rel.max())
        # The fp32 formula itself (RT_HIT_FP32) is bit-exact with the fp32 oracle.
        raw = gpu_trace(ctx, sc, rays[sub], flags=rt.HIT_FP32)
        compare(raw, want[sub], ties[sub])
        hit = gi >= 0
        assert (got[hit, 1] > 0.999e-4).all() and (got[hit, 1] < 1e4).all()


def test_trace_config1_beams_full_batch(rt, ctx, big_mesh, config1_oracle):
    """Beam casts (trace.beam) of the full coherent batch: every ray's hit
    index equals the oracle's outside ties, and the hits equal the packet
    cast's bit for bit."""
    tris, sc = big_mesh
    _, batches = config1_oracle
    rays, want, ties = batches["coherent"]
    old = ctx.get_tuning("trace.beam")
    try:
        ctx.set_tuning("trace.beam", 0)
        packets = gpu_trace(ctx, sc, rays)
        ctx.set_tuning("trace.beam", 1)
        got = gpu_trace(ctx, sc, rays)
    finally:
        ctx.set_tuning("trace.beam", old)
    gi, wi = got.view(np.int32)[:, 0], want.view(np.int32)[:, 0]
    assert int(((gi != wi) & ~ties).sum()) == 0
    assert np.array_equal(got.view(np.uint32), packets.view(np.uint32))


@pytest.mark.parametrize("builder", [1, 2])
def test_trace_config1_full_batch_other_trees(rt, ctx, big_mesh, config1_oracle, builder):
    """The LBVH and PLOC trees are quoted on this mesh too: every ray's hit
    index equals the oracle's on the reference tree, outside ties."""
    tris, _ = big_mesh
    _, batches = config1_oracle
    ctx.set_tuning("bvh.builder", builder)
    try:
        sc = ctx.upload_scene(tris, rt.gen_cornell(1, 0)[1])
    finally:
        ctx.set_tuning("bvh.builder", 0)
    try:
        for name, (rays, want, ties) in batches.items():
            got = gpu_trace(ctx, sc, rays)
            gi, wi = got.view(np.int32)[:, 0], want.view(np.int32)[:, 0]
            mismatch = int(((gi != wi) & ~ties).sum())
            assert mismatch == 0, f"builder {builder}, {name}: {mismatch} mismatches outside ties"
    finally:
        sc.release()


def test_trace_handles_ragged_and_empty_batches(rt, orc, ctx):
    tris, sc = mesh_scene(rt, ctx, 4, 3)
    try:
        nodes = sc.bvh()
        for n in (1, 31, 33, 1000):
            rays = rt.gen_random_rays(n, n, -1.5, 1.5)
            want = orc.trace(tris, nodes, rays)
            got = gpu_trace(ctx, sc, rays)
            assert np.array_equal(got.view(np.int32)[:, 0], want.view(np.int32)[:, 0])
        import torch
        z = torch.zeros((1, 8), device="cuda")
        sc.trace(z, 0, z)
        ctx.synchronize()
    finally:
        sc.release()


def test_trace_axis_aligned_rays(rt, orc, ctx):
    """Zero direction components (Q5: slab NaN/inf handling)."""
    t, m, _ = rt.gen_cornell(4, 2000)
    sc = ctx.upload_scene(t, m)
    try:
        nodes = sc.bvh()
        rng = np.random.default_rng(1)
        n = 4096
        rays = np.zeros((n, 8), np.float32)
        rays[:, 0:3] = rng.uniform(-4, 4, (n, 3))
        axis = rng.integers(0, 3, n)
        sign = rng.choice([-1.0, 1.0], n)
        rays[np.arange(n), 4 + axis] = sign
        rays[:, 3] = 0.001
        rays[:, 7] = 10000
        # Some origins exactly on a wall plane.
        rays[:64, 0] = -5.0
        want, st = orc.trace(t, nodes, rays, stats=True)
        ties = (st[:, 2] & 1) != 0
        compare(gpu_trace(ctx, sc, rays, flags=rt.HIT_FP32), want, ties)
    finally:
        sc.release()


def test_invalid_scenes_are_rejected(rt, ctx):
    t, m, _ = rt.gen_cornell(1, 10)
    bad = t.copy()
    bad[3, 0] = np.nan
    with pytest.raises(rt.RtError) as e:
        ctx.upload_scene(bad, m)
    assert e.value.status == 5
    bad = t.copy()
    bad.view(np.uint32)[2, 11] = 99
    with pytest.raises(rt.RtError):
        ctx.upload_scene(bad, m)
    badm = m.copy()
    badm.view(np.uint32)[0, 0] = 7
    with pytest.raises(rt.RtError):
        ctx.upload_scene(t, badm)
    with pytest.raises(rt.RtError):
        ctx.upload_scene(t[:0], m)
    # A node array that is not a tree.
    nodes = np.zeros((2 * len(t) - 1, 12), np.float32)
    nodes.view(np.int32)[:, 7:10] = -1
    nodes.view(np.int32)[0, 7] = 0
    nodes.view(np.int32)[0, 8] = 0
    with pytest.raises(rt.RtError):
        ctx.upload_scene(t, m, nodes=nodes)
    # The context stays usable.
    sc = ctx.upload_scene(t, m)
    sc.release()


KEYS = ("trace.refill", "trace.sort", "trace.packet", "trace.spec", "trace.wide", "trace.beam")


@pytest.mark.parametrize("refill,sort,packet,spec,wide,beam", [
    (1, 0, 0, 0, 0, 0), (4, 0, 0, 0, 0, 0), (16, 0, 0, 0, 0, 0), (32, 1, 0, 0, 0, 0), (4, 1, 0, 0, 0, 0),
    (32, 1, 1, 0, 0, 0), (32, 1, 1, 0, 0, 1), (32, 0, 1, 0, 0, 0), (32, 0, 1, 0, 0, 1), (32, 0, 0, 1, 0, 0),
    (32, 1, 0, 1, 0, 0), (32, 1, 1, 1, 0, 1), (32, 0, 0, 0, 1, 0), (32, 1, 0, 0, 1, 0), (32, 0, 1, 0, 1, 0),
    (32, 0, 1, 0, 1, 1), (32, 1, 1, 1, 1, 0), (32, 1, 1, 1, 1, 1)])
def test_trace_launch_shapes_agree(rt, orc, ctx, refill, sort, packet, spec, wide, beam):
    """Every launch shape of the caster (refill threshold, Morton order,
    packet traversal of coherent warps, beams over 256-ray tiles of one
    origin, postponed leaves, the 8-wide tree with the warp leaf pool)
    returns the same results in input order, bit for bit: the visiting order
    differs between shapes, and equal-t candidates are resolved by leaf
    index, not by the order met."""
    tris, sc = mesh_scene(rt, ctx, 6, 7)
    old_min = ctx.get_tuning("trace.wide_min_tris")
    ctx.set_tuning("trace.wide_min_tris", 0)  # this 81,920-triangle mesh takes the 8-wide caster too
    try:
        cam = rt.camera_look_at([0, 0, -3], [0, 0, 0], [0, 1, 0], 40.0, 256, 200)
        rays = np.concatenate([rt.gen_camera_rays(cam, 256, 200), rt.gen_random_rays(11, 40000)])
        old = [ctx.get_tuning(k) for k in KEYS]
        for k, v in zip(KEYS, (32, 0, 0, 0, 0, 0)):
            ctx.set_tuning(k, v)
        base = gpu_trace(ctx, sc, rays, flags=rt.HIT_FP32)
        for k, v in zip(KEYS, (refill, sort, packet, spec, wide, beam)):
            ctx.set_tuning(k, v)
        try:
            got = gpu_trace(ctx, sc, rays, flags=rt.HIT_FP32)
            host = sc.trace_host(rays)
            dev_default = gpu_trace(ctx, sc, rays)
        finally:
            for k, v in zip(KEYS, old):
                ctx.set_tuning(k, v)
        assert np.array_equal(host.view(np.uint32), dev_default.view(np.uint32))
        assert np.array_equal(got.view(np.uint32), base.view(np.uint32))
    finally:
        ctx.set_tuning("trace.wide_min_tris", old_min)
        sc.release()


def beam_ray_sets(rt):
    """Same-origin ray sets that take the beam path (sorted batches of at
    least 65,536 rays), and its edges."""
    def cam(eye, target, up, fov, w, h):
        return rt.gen_camera_rays(rt.camera_look_at(eye, target, up, fov, w, h), w, h)
    axis = cam([0, 0, -3], [0, 0, 0], [0, 1, 0], 30.0, 256, 256)  # centre rays with zero x or y
    neg_x = cam([3, 0.1, 0.2], [0, 0, 0], [0, 1, 0], 35.0, 320, 256)  # dominant axis -x
    inside = cam([0, 0, 0], [0, 1, 0], [0, 0, 1], 60.0, 256, 256)  # origin inside the mesh, +y
    grazing = cam([0, 1.25, -3], [0, 1.0, 0], [0, 1, 0], 6.0, 256, 256)  # the silhouette
    diagonal = cam([2, 2, -2], [0, 0, 0], [0, 1, 0], 70.0, 256, 256)  # dominant axis changes across the image
    tail = np.concatenate([axis, axis[:37]])  # a partial last tile
    bounds = axis.copy()
    bounds[::3, 7] = np.inf  # unbounded rays
    bounds[1::7, 7] = 0.0  # tmax below tmin: no hit
    bounds[2::5, 7] = 3.0  # short rays
    mixed = axis.copy()
    mixed[1::2, :3] += np.float32(1e-3)  # two origins: no beam
    stray = axis.copy()
    stray[5::97, :3] += np.float32(1e-3)  # a few other origins: the sort's sample may miss them
    wide = cam([0, 0, -3], [0, 0, 0], [0, 1, 0], 150.0, 256, 256)  # tiles too wide for a beam
    return {"axis": axis, "neg_x": neg_x, "inside": inside, "grazing": grazing, "diagonal": diagonal, "tail": tail,
            "bounds": bounds, "mixed": mixed, "stray": stray, "wide": wide}


@pytest.mark.parametrize("name", ["axis", "neg_x", "inside", "grazing", "diagonal", "tail", "bounds", "mixed",
                                  "stray", "wide"])
def test_beam_tiles_equal_packets(rt, orc, ctx, name):
    """Beams over the ray sort's cell tiles return the packet and per-lane
    casts' hits bit for bit, on the edges of the beam path: axis-aligned
    and negative dominant directions, an origin inside the tree's boxes,
    rays along the silhouette, a dominant axis that changes across the
    image, a partial last tile, unbounded, empty and short rays, batches
    of two origins or a few stray ones, and tiles too wide for a beam."""
    tris, sc = mesh_scene(rt, ctx, 6, 7)
    rays = beam_ray_sets(rt)[name]
    keys = ("trace.beam", "trace.sort", "trace.packet")
    old = [ctx.get_tuning(k) for k in keys]
    try:
        ctx.set_tuning("trace.packet", 0)
        ctx.set_tuning("trace.beam", 0)
        ctx.set_tuning("trace.sort", 0)
        want = gpu_trace(ctx, sc, rays, flags=rt.HIT_FP32)
        ctx.set_tuning("trace.packet", 1)
        for sort in (0, 1):
            for beam in (0, 1):
                ctx.set_tuning("trace.sort", sort)
                ctx.set_tuning("trace.beam", beam)
                got = gpu_trace(ctx, sc, rays, flags=rt.HIT_FP32)
                assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (sort, beam)
        host = sc.trace_host(rays)
        assert np.array_equal(host.view(np.uint32), gpu_trace(ctx, sc, rays).view(np.uint32))
    finally:
        for k, v in zip(keys, old):
            ctx.set_tuning(k, v)
        sc.release()


def test_beam_tiles_vs_oracle(rt, orc, ctx):
    """Beam casts of camera tiles against the oracle's culled traversal of
    the same tree: hit index equal outside exact t ties, t/u/v bit-exact
    where the index agrees."""
    tris, sc = mesh_scene(rt, ctx, 6, 7)
    old = ctx.get_tuning("trace.beam")
    try:
        ctx.set_tuning("trace.beam", 1)
        sets = beam_ray_sets(rt)
        for name in ("axis", "neg_x", "grazing", "inside"):
            rays = sets[name]
            got = gpu_trace(ctx, sc, rays, flags=rt.HIT_FP32)
            want, st = orc.trace(tris, sc.bvh(), rays, stats=True)
            ties = (st[:, 2] & 1) != 0
            compare(got, want, ties)
    finally:
        ctx.set_tuning("trace.beam", old)
        sc.release()


def test_single_triangle_scene(rt, orc, ctx):
    """A one-triangle scene: the root itself is a leaf, in every traversal."""
    t, m, _ = rt.gen_cornell(1, 0)
    t = t[:1].copy()
    sc = ctx.upload_scene(t, m)
    old = [ctx.get_tuning(k) for k in KEYS]
    old_min = ctx.get_tuning("trace.wide_min_tris")
    ctx.set_tuning("trace.wide_min_tris", 0)
    try:
        # 60 degrees: tiles too wide for a beam; 8 degrees: every tile a beam.
        for fov in (60.0, 8.0):
            cam = rt.camera_look_at([0, 0, -14], [0, -4, 0], [0, 1, 0], fov, 64, 64)
            rays = rt.gen_camera_rays(cam, 64, 64)
            want = orc.trace(t, sc.bvh(), rays)
            for spec, wide, beam in ((0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (0, 1, 1)):
                ctx.set_tuning("trace.spec", spec)
                ctx.set_tuning("trace.wide", wide)
                ctx.set_tuning("trace.beam", beam)
                got = gpu_trace(ctx, sc, rays, flags=rt.HIT_FP32)
                np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    finally:
        for k, v in zip(KEYS, old):
            ctx.set_tuning(k, v)
        ctx.set_tuning("trace.wide_min_tris", old_min)
        sc.release()


def test_tuning_keys(rt, ctx):
    with pytest.raises(rt.RtError):
        ctx.set_tuning("no.such.key", 1)
    with pytest.raises(rt.RtError):
        ctx.set_tuning("trace.refill", 0)
    assert 1 <= ctx.get_tuning("trace.refill") <= 32
    for key, bad in (("trace.beam", 3), ("trace.beam", -1), ("trace.beam_round", 15), ("trace.beam_round", 257)):
        with pytest.raises(rt.RtError):
            ctx.set_tuning(key, bad)
    assert ctx.get_tuning("trace.beam") == 0 and ctx.get_tuning("trace.beam_round") == 64


@pytest.mark.parametrize("builder", [1, 2], ids=["lbvh", "ploc"])
def test_alt_tree_mode_same_hits(rt, orc, ctx, builder):
    """The separately reported trees (1 LBVH, 2 PLOC): valid tree, every
    triangle in one leaf, and the same closest hits as the reference tree."""
    tris = rt.gen_icosphere(5, 6)
    mats = rt.gen_cornell(1, 0)[1]
    ref_sc = ctx.upload_scene(tris, mats)
    old = ctx.get_tuning("bvh.builder")
    ctx.set_tuning("bvh.builder", builder)
    try:
        sc = ctx.upload_scene(tris, mats)
    finally:
        ctx.set_tuning("bvh.builder", old)
    try:
        nodes = sc.bvh()
        objs = nodes.view(np.int32)[:, 9]
        leaves = (nodes.view(np.int32)[:, 7] == -1)
        assert sorted(objs[leaves].tolist()) == list(range(len(tris)))
        # Every inner box contains its children's boxes.
        inner = np.nonzero(~leaves)[0]
        L, R = nodes.view(np.int32)[inner, 7], nodes.view(np.int32)[inner, 8]
        for c in (L, R):
            assert (nodes[inner][:, 0:3] <= nodes[c][:, 0:3]).all() and (nodes[inner][:, 4:7] >= nodes[c][:, 4:7]).all()
        assert sc.info().depth <= 64
        cam = rt.camera_look_at([0, 0, -3], [0, 0, 0], [0, 1, 0], 40.0, 96, 96)
        rays = np.concatenate([rt.gen_camera_rays(cam, 96, 96), rt.gen_random_rays(21, 20000)])
        want, st = orc.trace(tris, ref_sc.bvh(), rays, stats=True)
        ties = (st[:, 2] & 1) != 0
        compare(gpu_trace(ctx, sc, rays, flags=rt.HIT_FP32), want, ties)
        compare(gpu_trace(ctx, ref_sc, rays, flags=rt.HIT_FP32), want, ties)
        # The 8-wide fold of this tree (forced below its size threshold).
        old_min = ctx.get_tuning("trace.wide_min_tris")
        ctx.set_tuning("trace.wide_min_tris", 0)
        try:
            compare(gpu_trace(ctx, sc, rays, flags=rt.HIT_FP32), want, ties)
        finally:
            ctx.set_tuning("trace.wide_min_tris", old_min)
    finally:
        sc.release()
        ref_sc.release()


def test_autotune_trace_keeps_hits(rt, orc, ctx):
    """The autotuner's candidates are timing choices only: after tuning, the
    hits equal the ones cast with the settings it started from."""
    keys = ("trace.block", "trace.stack", "trace.wide", "trace.wide_minblocks", "trace.wide_visits", "trace.defer",
            "trace.spec", "trace.minblocks", "trace.packet_minblocks", "trace.sort", "trace.beam")
    old = [ctx.get_tuning(k) for k in keys]
    tris, sc = mesh_scene(rt, ctx, 6, 3)
    try:
        cam = rt.camera_look_at([0, 0, -3], [0, 0, 0], [0, 1, 0], 40.0, 256, 256)
        rays = np.concatenate([rt.gen_camera_rays(cam, 256, 256), rt.gen_random_rays(8, 1 << 16)])
        want = gpu_trace(ctx, sc, rays, flags=rt.HIT_FP32)
        import torch
        d_rays = dev(rays)
        d_hits = torch.zeros((len(rays), 4), dtype=torch.float32, device="cuda")
        before, after = rt.autotune_trace(sc, d_rays, len(rays), d_hits, reps=1)
        assert before > 0 and after > 0
        allowed = {"trace.wide_minblocks": (8, 7, 6, 5), "trace.minblocks": (16, 12, 10), "trace.wide_visits": (1, 2, 3),
                   "trace.packet_minblocks": (16, 12, 10), "trace.block": (64, 128, 256),
                   "trace.stack": (0, 32, 64)}
        for k in keys:
            assert ctx.get_tuning(k) in allowed.get(k, (0, 1))
        got = gpu_trace(ctx, sc, rays, flags=rt.HIT_FP32)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    finally:
        for k, v in zip(keys, old):
            ctx.set_tuning(k, v)
        sc.release()


@pytest.mark.parametrize("level,wide_min", [(6, 0), (6, 1 << 30), (4, 1 << 30)], ids=["bvh8", "binary", "shallow"])
def test_block_size_and_stack_depth_keep_hits(rt, ctx, level, wide_min):
    """The autotuner's block-size (64/128/256 threads), stack-depth
    (16/32/64 entries, raised to what the tree needs) and 8-wide visits
    axes: every candidate returns the same hits bit for bit, on the 8-wide
    caster and on the binary packet and per-lane kernels, including a tree
    shallow enough for the 16-entry stack."""
    tris, sc = mesh_scene(rt, ctx, level, 4)
    keys = ("trace.block", "trace.stack", "trace.wide_min_tris", "trace.wide_visits")
    old = [ctx.get_tuning(k) for k in keys]
    try:
        ctx.set_tuning("trace.wide_min_tris", wide_min)
        if level == 4:
            assert sc.info().depth <= 16
        cam = rt.camera_look_at([0, 0, -3], [0, 0, 0], [0, 1, 0], 40.0, 128, 96)
        rays = np.concatenate([rt.gen_camera_rays(cam, 128, 96), rt.gen_random_rays(12, 20000)])
        base = gpu_trace(ctx, sc, rays, flags=rt.HIT_FP32)
        refined = gpu_trace(ctx, sc, rays)
        for block in (64, 128, 256):
            for stack in (0, 16, 32, 64):
                ctx.set_tuning("trace.block", block)
                ctx.set_tuning("trace.stack", stack)
                ctx.set_tuning("trace.wide_visits", 1 + (stack // 16) % 3)
                got = gpu_trace(ctx, sc, rays, flags=rt.HIT_FP32)
                assert np.array_equal(got.view(np.uint32), base.view(np.uint32)), (block, stack)
                # The default (fp64 re-evaluated) results agree as well.
                assert np.array_equal(gpu_trace(ctx, sc, rays).view(np.uint32), refined.view(np.uint32))
    finally:
        for k, v in zip(keys, old):
            ctx.set_tuning(k, v)
        sc.release()


@pytest.mark.parametrize("collapse", [0, 1], ids=["largest-first", "sah"])
def test_bvh8_collapse_modes_keep_hits(rt, orc, ctx, collapse):
    """Both 8-wide folds ("bvh8.collapse": SAH-chosen pairs, largest child
    first) give the oracle's hits bit for bit on the 8-wide caster, for
    camera and random rays, on a displaced icosphere and on a Cornell soup
    (long thin triangles, many overlapping boxes)."""
    keys = ("bvh8.collapse", "trace.wide_min_tris")
    old = [ctx.get_tuning(k) for k in keys]
    ctx.set_tuning("bvh8.collapse", collapse)
    ctx.set_tuning("trace.wide_min_tris", 0)
    scs = []
    try:
        t_ico = rt.gen_icosphere(9, 6)
        t_box, m_box, _ = rt.gen_cornell(4, 30000, 0)
        for tris, mats, eye in ((t_ico, rt.gen_cornell(1, 0)[1], [0, 0, -3]), (t_box, m_box, [0, 0, -14])):
            sc = ctx.upload_scene(tris, mats)
            scs.append(sc)
            cam = rt.camera_look_at(eye, [0, 0, 0], [0, 1, 0], 40.0, 96, 64)
            rays = np.concatenate([rt.gen_camera_rays(cam, 96, 64), rt.gen_random_rays(13, 20000)])
            want = orc.trace(tris, sc.bvh(), rays)
            got = gpu_trace(ctx, sc, rays, flags=rt.HIT_FP32)
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    finally:
        for k, v in zip(keys, old):
            ctx.set_tuning(k, v)
        for sc in scs:
            sc.release()


@pytest.mark.parametrize("builder", [0, 1, 2], ids=["reference", "lbvh", "ploc"])
def test_degenerate_geometry_both_folds(rt, orc, ctx, builder):
    """Stacked identical triangles, point-sized (zero-area) triangles and a
    flat grid: every tree and both 8-wide folds give the oracle's hits (the
    lowest index among exactly equal t). Zero-area boxes give the SAH fold
    no preference; where it would need more nodes than the slab reserves,
    the upload takes the largest-first fold."""
    t, m, _ = rt.gen_cornell(5, 600, 0)
    t = t.copy()
    rng = np.random.default_rng(5)
    # 200 copies of one triangle, 300 point triangles, the rest as generated.
    t[12:212, 0:12] = t[12, 0:12]
    p = rng.uniform(-3, 3, (300, 3)).astype(np.float32)
    for v in range(3):
        t[212:512, 4 * v:4 * v + 3] = p
    keys = ("bvh8.collapse", "trace.wide_min_tris", "bvh.builder")
    old = [ctx.get_tuning(k) for k in keys]
    try:
        ctx.set_tuning("trace.wide_min_tris", 0)
        ctx.set_tuning("bvh.builder", builder)
        for collapse in (1, 0):
            ctx.set_tuning("bvh8.collapse", collapse)
            sc = ctx.upload_scene(t, m)
            try:
                cam = rt.camera_look_at([0, 0, -14], [0, 0, 0], [0, 1, 0], 40.0, 64, 48)
                rays = np.concatenate([rt.gen_camera_rays(cam, 64, 48), rt.gen_random_rays(17, 6000, -4.0, 4.0)])
                want = orc.trace(t, sc.bvh(), rays)
                got = gpu_trace(ctx, sc, rays, flags=rt.HIT_FP32)
                assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (builder, collapse)
            finally:
                sc.release()
    finally:
        for k, v in zip(keys, old):
            ctx.set_tuning(k, v)


def test_host_entry_concurrent_calls(rt, ctx):
    """rtTraceClosestHost from four host threads at once (each call takes
    its own streams and staging from the context's pool), with chunks small
    enough that every call pipelines several: every result equals the
    device-path hits of the same rays, bit for bit."""
    import threading
    tris, sc = mesh_scene(rt, ctx, 6, 21)
    old = ctx.get_tuning("trace.host_chunk")
    try:
        ctx.set_tuning("trace.host_chunk", 1 << 16)
        cam = rt.camera_look_at([0, 0, -3], [0, 0, 0], [0, 1, 0], 40.0, 384, 384)
        batches = [rt.gen_camera_rays(cam, 384, 384)] + [rt.gen_random_rays(30 + k, 150000) for k in range(3)]
        want = [gpu_trace(ctx, sc, r) for r in batches]
        got = [None] * len(batches)
        errs = []

        def run(k):
            try:
                got[k] = sc.trace_host(batches[k])
            except Exception as e:  # reported below, on the main thread
                errs.append(e)

        for _ in range(2):
            ths = [threading.Thread(target=run, args=(k,)) for k in range(len(batches))]
            for t in ths:
                t.start()
            for t in ths:
                t.join()
            assert not errs, errs
            for g, w in zip(got, want):
                assert np.array_equal(g.view(np.uint32), w.view(np.uint32))
    finally:
        ctx.set_tuning("trace.host_chunk", old)
        sc.release()
