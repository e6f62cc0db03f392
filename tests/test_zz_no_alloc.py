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


def no_alloc_build(rt, tris, seed):
    import torch
    fn = rt.LIB.rtBuildBvhNoAlloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p]
    d_tris = torch.from_numpy(np.ascontiguousarray(tris)).cuda()
    d_nodes = torch.full((2 * len(tris) - 1, 12), -7.0, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    st = fn(d_tris.data_ptr(), len(tris), seed, d_nodes.data_ptr(), None)
    assert st == 0, rt.LIB.rtStatusString(st)
    return d_nodes.cpu().numpy()


def test_no_alloc_build_matches_regular_build(rt, ctx):
    # Two calls in a row: the largest accepted size, then a smaller scene, so
    # the second call runs on the scratch the first one left behind.
    big = rt.gen_cornell(21, MAX_TRIANGLES - 12)[0]
    small, mats, _ = rt.gen_cornell(22, 1410)
    for tris, seed in ((big, 1), (small, 5)):
        got = no_alloc_build(rt, tris, seed)
        sc = ctx.upload_scene(tris, mats, bvh_seed=seed)
        try:
            want = sc.bvh()
        finally:
            sc.release()
        assert np.array_equal(got.view(np.uint32)[:, NODE_COLS], want.view(np.uint32)[:, NODE_COLS])


def test_no_alloc_build_rejects_oversize_and_bad_pointers(rt):
    fn = rt.LIB.rtBuildBvhNoAlloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p]
    # Rejected before any device work: the size limit, n == 0, null pointers.
    assert fn(16, MAX_TRIANGLES + 1, 1, 16, None) == 1
    assert fn(16, 0, 1, 16, None) == 1
    assert fn(None, 10, 1, 16, None) == 1
    assert fn(16, 10, 1, None, None) == 1
