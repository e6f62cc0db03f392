"""GPU BVH build: node-for-node identical to the reference's Bvh::createBvh.

Pinned by the reference-generated digests in golden/bvh.json (1.4k to 1.31M
triangles) and, live, by the oracle's restatement on tie-heavy inputs.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from test_oracle_pins import SCENES, node_digest, _tie_heavy_scene

pytestmark = pytest.mark.gpu

NODE_COLS = [0, 1, 2, 4, 5, 6, 7, 8, 9]


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(GOLDEN, "bvh.json")) as f:
        return json.load(f)


def _mats(rt):
    return rt.gen_cornell(1, 0)[1]


@pytest.mark.parametrize("name", list(SCENES))
def test_gpu_build_matches_reference_digest(rt, ctx, golden, name):
    tris = SCENES[name](rt)
    tris.view(np.uint32)[:, 11] = 0
    sc = ctx.upload_scene(tris, _mats(rt))
    try:
        nodes = sc.bvh()
        g = golden[name]
        assert len(nodes) == g["nodes"]
        for r, words in g["rows"].items():
            assert nodes.view(np.uint32)[int(r), NODE_COLS].tolist() == words, f"row {r}"
        assert node_digest(nodes) == g["digest"]
        info = sc.info()
        assert info.nodes == 2 * len(tris) - 1
    finally:
        sc.release()


def test_gpu_build_seed(rt, ctx, golden):
    tris = rt.gen_cornell(1, 12000)[0]
    sc = ctx.upload_scene(tris, _mats(rt), bvh_seed=7)
    try:
        assert node_digest(sc.bvh()) == golden["cornell_12000_seed7"]["digest"]
    finally:
        sc.release()


@pytest.mark.parametrize("seed,n", [(0, 1), (0, 2), (1, 5), (2, 33), (3, 100), (4, 1000), (5, 4097),
                                    (6, 20000), (7, 9000), (8, 70000), (9, 300000)])
def test_gpu_build_matches_oracle_on_ties(rt, orc, ctx, seed, n):
    tris = _tie_heavy_scene(seed, n)
    want, depth = orc.build_bvh(tris, 1 + seed)
    sc = ctx.upload_scene(tris, _mats(rt), bvh_seed=1 + seed)
    try:
        got = sc.bvh()
        assert np.array_equal(got.view(np.uint32)[:, NODE_COLS], want.view(np.uint32)[:, NODE_COLS])
        assert sc.info().depth == depth
    finally:
        sc.release()


def test_uploaded_nodes_are_used_as_is(rt, orc, ctx):
    tris = rt.gen_cornell(2, 3000)[0]
    nodes, _ = orc.build_bvh(tris, 5)
    sc = ctx.upload_scene(tris, _mats(rt), nodes=nodes)
    try:
        assert np.array_equal(sc.bvh().view(np.uint32)[:, NODE_COLS], nodes.view(np.uint32)[:, NODE_COLS])
    finally:
        sc.release()


@pytest.mark.parametrize("level", [0, 3, 9])
def test_error_raised_at_an_early_level_fails_the_upload(rt, ctx, level):
    # The build's error word must survive the later levels: a bit recorded
    # after the sort of `level` (test hook, as an overflow would record it)
    # fails the upload with RT_ERR_INTERNAL, and the next upload succeeds.
    tris = rt.gen_cornell(3, 4000)[0]
    ctx.set_tuning("bvh.test_error_level", level)
    try:
        with pytest.raises(rt.RtError) as ei:
            ctx.upload_scene(tris, _mats(rt))
        assert ei.value.status == 10
    finally:
        ctx.set_tuning("bvh.test_error_level", -1)
    sc = ctx.upload_scene(tris, _mats(rt))
    sc.release()
