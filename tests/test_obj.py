"""OBJ loading (rtLoadObj / rtLoadReferenceScene) on the CPU: the index forms
and statements a Wavefront file mixes, error handling, coordinate parsing
against correctly rounded conversion, and the reference's own demo scene
(src/ray-tracing/RtScene.h:44-101) against the oracle's restatement and the
reference's Bvh.h build."""
import ctypes
import os

import numpy as np
import pytest


def write(tmp_path, name, text, newline="\n"):
    p = tmp_path / name
    p.write_bytes(text.replace("\n", newline).encode())
    return str(p)


SAMPLE = """# comment line
mtllib scene.mtl
o first
v 0.000000 0.000000 0.000000
v 1.000000 0.000000 0.000000
v\t0.000000  1.000000 0.000000
v 1.0 1.0 1.0 1.0
vt 0.5 0.5
vn 0.0 0.0 1.0
usemtl red
s off
f 1 2 3
f 1/1 2/1 4/1
f 2//1 3//1 4//1
f 1/1/1 3/1/1 4/1/1
g second
v +2.5e0 -1.25E-1 3
v 2 2 2
f -3 -2 -1
f 1 2 4 3
l 1 2
"""


def expected_sample():
    V = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (1, 1, 1), (2.5, -0.125, 3.0), (2, 2, 2)]
    faces = [(0, 1, 2), (0, 1, 3), (1, 2, 3), (0, 2, 3), (3, 4, 5), (0, 1, 3), (0, 3, 2)]
    return V, faces


@pytest.mark.parametrize("newline", ["\n", "\r\n"], ids=["lf", "crlf"])
def test_obj_statements_and_index_forms(rt, orc, tmp_path, newline):
    path = write(tmp_path, "sample.obj", SAMPLE, newline)
    tris = rt.load_obj(path, material=7)
    V, faces = expected_sample()
    assert tris.shape == (len(faces), 12)
    for row, f in zip(tris, faces):
        for j in range(3):
            assert tuple(row[4 * j:4 * j + 3]) == tuple(np.float32(V[f[j]]))
    assert (tris.view(np.uint32)[:, 11] == 7).all()
    np.testing.assert_array_equal(tris.view(np.uint32), orc.obj_triangles(path, 7).view(np.uint32))


def test_obj_errors(rt, tmp_path):
    with pytest.raises(rt.RtError) as e:
        rt.load_obj(str(tmp_path / "missing.obj"))
    assert e.value.status == 4  # RT_ERR_NOT_FOUND
    bad0 = write(tmp_path, "zero.obj", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 0 1 2\n")
    with pytest.raises(rt.RtError) as e:
        rt.load_obj(bad0)
    assert e.value.status == 5  # RT_ERR_INVALID_SCENE
    far = write(tmp_path, "far.obj", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 4\n")
    with pytest.raises(rt.RtError) as e:
        rt.load_obj(far)
    assert "outside the 3 vertices" in str(e.value)
    # A relative index may only reach vertices read before the face.
    late = write(tmp_path, "late.obj", "v 0 0 0\nv 1 0 0\nf -1 -2 -3\nv 0 1 0\n")
    with pytest.raises(rt.RtError):
        rt.load_obj(late)
    ok = write(tmp_path, "ok.obj", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\nf 3 2 1\nf 1 2\n")
    n = ctypes.c_uint32()
    buf = np.zeros((1, 12), np.float32)
    st = rt.LIB.rtLoadObj(ok.encode(), 0, buf.ctypes.data, 1, ctypes.byref(n))
    assert st == 1 and n.value == 2  # capacity below the count; a 2-vertex face is skipped
    assert rt.load_obj(ok).shape == (2, 12)
    empty = write(tmp_path, "empty.obj", "# nothing\n")
    assert rt.load_obj(empty).shape == (0, 12)


def test_obj_coordinates_round_like_correct_conversion(rt, tmp_path):
    """Digit-by-digit parsing gives the correctly rounded float for the
    six-decimal coordinates OBJ exporters write, and stays within one float
    ulp of it for long mantissas and exponents."""
    g = np.random.default_rng(5)
    vals = np.concatenate([g.normal(0, 3, 3000), g.uniform(-1e4, 1e4, 600), 10.0 ** g.uniform(-8, 8, 600)])
    for fmt, exact in (("%.6f", True), ("%.4f", True), ("%.9g", False), ("%.17g", False), ("%.7e", False)):
        strs = [fmt % v for v in vals]
        lines = ["v %s %s %s" % (strs[i], strs[i + 1], strs[i + 2]) for i in range(0, len(strs) - 2, 3)]
        n = len(lines)
        lines += ["f %d %d %d" % (i + 1, i + 1, i + 1) for i in range(n)]
        path = write(tmp_path, "num.obj", "\n".join(lines) + "\n")
        tris = rt.load_obj(path)
        got = tris[:, 0:3].reshape(-1)
        want = np.array([float(s) for s in strs[:3 * n]], np.float64).astype(np.float32)
        if exact:
            np.testing.assert_array_equal(got, want)
        else:
            ulp = np.abs(got.view(np.int32).astype(np.int64) - want.view(np.int32).astype(np.int64))
            assert ulp.max() <= 1, fmt
            assert (ulp == 0).mean() > 0.999, fmt


needs_scene = pytest.mark.skipif(
    not os.path.exists(os.path.join(os.path.dirname(__file__), "..", "oracle", "_ref", "doge_scene",
                                    "buff-doge.obj")),
    reason="the reference's demo scene was not copied (no reference checkout)")


@needs_scene
def test_reference_scene_matches_restatement(rt, orc):
    tris, mats, sph = rt.load_reference_scene(orc.REF_SCENE_DIR)
    want_t, want_m, want_s = orc.reference_scene(orc.REF_SCENE_DIR)
    assert len(tris) == 1422  # 916 + 480 + 2 + 2 + 2 + 16 + 2 + 2
    np.testing.assert_array_equal(tris.view(np.uint32), want_t.view(np.uint32))
    np.testing.assert_array_equal(mats.view(np.uint32), want_m.view(np.uint32))
    np.testing.assert_array_equal(sph.view(np.uint32), want_s.view(np.uint32))
    # The light quad is the last object (material 3): two lights.
    lights = rt.lights_from_materials(tris, mats)
    assert lights.view(np.uint32)[:, 0].tolist() == [1420, 1421]
    np.testing.assert_array_equal(lights.view(np.uint32), orc.lights_from_materials(tris, mats).view(np.uint32))


@needs_scene
def test_reference_scene_tree_matches_reference_build(orc):
    if not orc.ref_available():
        pytest.skip("reference Bvh.h not compiled")
    tris, _, _ = orc.reference_scene(orc.REF_SCENE_DIR)
    mine, _ = orc.build_bvh(tris, 1)
    ref = orc.ref_build_bvh(tris, 1)
    np.testing.assert_array_equal(mine.view(np.uint32)[:, [0, 1, 2, 4, 5, 6, 7, 8, 9]],
                                  ref.view(np.uint32)[:, [0, 1, 2, 4, 5, 6, 7, 8, 9]])
