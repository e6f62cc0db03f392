"""The allocation-free BVH build (rtBuildBvhNoAlloc) against the regular
GPU build behind rtUploadScene.

Callers that may not allocate device memory — for instance a host
application whose device memory belongs to another allocator or runtime —
build their BVH with rtBuildBvhNoAlloc: it runs the same kernels on a fixed
scratch array inside the library. This file is named so that pytest collects
it last; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NODE_COLS = [0, 1, 2, 4, 5, 6, 7, 8, 9]
MAX_TRIANGLES = 65536


def _entry(rt):
    fn = rt.LIB.rtBuildBvhNoAlloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p]
    return fn


def no_alloc_build(rt, tris, seed, stream=None):
    """Builds through rtBuildBvhNoAlloc on `stream` (a torch.cuda.Stream or
    None for the legacy default stream) and returns the nodes."""
    import torch
    fn = _entry(rt)
    d_tris = torch.from_numpy(np.ascontiguousarray(tris)).cuda()
    d_nodes = torch.full((2 * len(tris) - 1, 12), -7.0, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    st = fn(d_tris.data_ptr(), len(tris), seed, d_nodes.data_ptr(), stream.cuda_stream if stream else None)
    assert st == 0, rt.LIB.rtStatusString(st)
    return d_nodes.cpu().numpy()


def regular_build(ctx, tris, mats, seed):
    sc = ctx.upload_scene(tris, mats, bvh_seed=seed)
    try:
        return sc.bvh()
    finally:
        sc.release()


def test_no_alloc_build_matches_regular_build(rt, ctx):
    # Two calls in a row: the largest accepted size, then a smaller scene, so
    # the second call runs on the scratch the first one left behind.
    big = rt.gen_cornell(21, MAX_TRIANGLES - 12)[0]
    small, mats, _ = rt.gen_cornell(22, 1410)
    for tris, seed in ((big, 1), (small, 5)):
        got = no_alloc_build(rt, tris, seed)
        want = regular_build(ctx, tris, mats, seed)
        assert np.array_equal(got.view(np.uint32)[:, NODE_COLS], want.view(np.uint32)[:, NODE_COLS])


def test_no_alloc_build_on_a_side_stream_then_the_default_stream(rt, ctx):
    # Consecutive calls on different streams share the scratch array; each
    # result must still be the regular build's tree.
    import torch
    a, mats, _ = rt.gen_cornell(23, 20000)
    b = rt.gen_cornell(24, 3000)[0]
    side = torch.cuda.Stream()
    got_a = no_alloc_build(rt, a, 1, stream=side)
    got_b = no_alloc_build(rt, b, 1, stream=None)
    for got, tris in ((got_a, a), (got_b, b)):
        want = regular_build(ctx, tris, mats, 1)
        assert np.array_equal(got.view(np.uint32)[:, NODE_COLS], want.view(np.uint32)[:, NODE_COLS])


def test_no_alloc_build_rejects_non_finite_vertices(rt, ctx):
    # Checked on the device before any sort runs; the next call still works.
    import torch
    tris, mats, _ = rt.gen_cornell(25, 500)
    bad = tris.copy()
    bad[77, 5] = np.nan
    fn = _entry(rt)
    d_tris = torch.from_numpy(bad).cuda()
    d_nodes = torch.zeros((2 * len(bad) - 1, 12), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    assert fn(d_tris.data_ptr(), len(bad), 1, d_nodes.data_ptr(), None) == 5  # RT_ERR_INVALID_SCENE
    bad[77, 5] = np.inf
    d_tris = torch.from_numpy(bad).cuda()
    torch.cuda.synchronize()
    assert fn(d_tris.data_ptr(), len(bad), 1, d_nodes.data_ptr(), None) == 5
    got = no_alloc_build(rt, tris, 1)
    want = regular_build(ctx, tris, mats, 1)
    assert np.array_equal(got.view(np.uint32)[:, NODE_COLS], want.view(np.uint32)[:, NODE_COLS])


def test_no_alloc_build_rejects_oversize_and_bad_pointers(rt):
    fn = _entry(rt)
    # Rejected before any device work: the size limit, n == 0, null pointers.
    assert fn(16, MAX_TRIANGLES + 1, 1, 16, None) == 1
    assert fn(16, 0, 1, 16, None) == 1
    assert fn(None, 10, 1, 16, None) == 1
    assert fn(16, 10, 1, None, None) == 1
