"""The oracle's restatement of the seeded workload generators equals the
product library's generators byte for byte (the reference arm of the bench
makes its inputs from the oracle alone)."""
import numpy as np
import pytest


@pytest.mark.parametrize("seed,level,radius,sigma,mat", [(1, 0, 1.0, 0.05, 0), (7, 3, 2.5, 0.2, 3),
                                                         (1, 6, 1.0, 0.05, 0)])
def test_icosphere_equals_library(rt, orc, seed, level, radius, sigma, mat):
    a = rt.gen_icosphere(seed, level, radius, sigma, mat)
    b = orc.gen_icosphere(seed, level, radius, sigma, mat)
    assert a.shape == b.shape
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("eye,target,vfov,w,h", [([0, 0, -3], [0, 0, 0], 40.0, 2048, 2048),
                                                 ([0, 0, -14], [0, 0, 0], 40.0, 256, 256),
                                                 ([1.5, 2, -7], [0.2, -0.3, 1], 65.0, 97, 41)])
def test_camera_and_camera_rays_equal_library(rt, orc, eye, target, vfov, w, h):
    cam = rt.camera_look_at(eye, target, [0, 1, 0], vfov, w, h)
    mine = orc.camera_look_at(eye, target, [0, 1, 0], vfov, w, h)
    assert np.array_equal(cam.as_array().view(np.uint32), mine.view(np.uint32))
    side = min(w, 128)
    a = rt.gen_camera_rays(cam, side, min(h, 128))
    b = orc.gen_camera_rays(mine, side, min(h, 128))
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("seed,n,lo,hi", [(3, 100000, -1.5, 1.5), (11, 777, -4.0, 2.0)])
def test_random_rays_equal_library(rt, orc, seed, n, lo, hi):
    a = rt.gen_random_rays(seed, n, lo, hi)
    b = orc.gen_random_rays(seed, n, lo, hi)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.slow
def test_closest_hit_workload_equals_library(rt, orc):
    # The full measured inputs: 1,310,720 triangles, 2 x 4,194,304 rays.
    tris, coh, inc = orc.closest_hit_workload()
    assert np.array_equal(tris.view(np.uint32), rt.gen_icosphere(1, 8).view(np.uint32))
    cam = rt.camera_look_at([0, 0, -3], [0, 0, 0], [0, 1, 0], 40.0, 2048, 2048)
    assert np.array_equal(coh.view(np.uint32), rt.gen_camera_rays(cam, 2048, 2048).view(np.uint32))
    assert np.array_equal(inc.view(np.uint32), rt.gen_random_rays(3, 2048 * 2048).view(np.uint32))
