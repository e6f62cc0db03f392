"""Test infrastructure (oracle) — NOT part of the product.

ctypes access to the CPU oracle (liboracle.so, built from rt_oracle.cpp) and,
where they were built, to the reference's own BVH builder (_ref/libref_bvh.so,
built from the reference's src/ray-tracing/Bvh.h) and its own compute shader
(_ref/libref_shader.so, ray-trace-compute.comp rewritten into C++ by
glsl2cpp.py). Only the tests,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this module,
and only as the oracle / the timed CPU baseline.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref_bvh.so")


def build() -> None:
    """Builds liboracle.so (and _ref when the reference checkout exists)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def _load():
    if not os.path.exists(LIB_PATH):
        build()
    lib = ctypes.CDLL(LIB_PATH)
    P, U32, I32, D = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.c_double
    sigs = {
        "oracle_glibc_rand": (None, [U32, U32, P]),
        "oracle_build_bvh": (I32, [P, U32, P, U32, ctypes.POINTER(I32)]),
        "oracle_sort_with_depth": (None, [P, P, U32, I32]),
        "oracle_lights_from_materials": (U32, [P, U32, P, U32, P]),
        "oracle_camera_from_reference": (None, [P, U32, U32, P]),
        "oracle_denoise": (None, [P, U32, U32, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, P]),
        "oracle_hit_records": (None, [P, U32, P, U32, P, U32, P, U32, U32, P]),
        "oracle_trace": (I32, [P, U32, P, U32, P, U32, I32, I32, D, P, P, I32]),
        "oracle_trace_f64": (I32, [P, U32, P, U32, P, U32, P, P, I32]),
        "oracle_render": (I32, [P, U32, P, U32, P, U32, P, U32, P, U32, P, P, P, ctypes.POINTER(ctypes.c_uint64), I32]),
        "oracle_render_f64": (I32, [P, U32, P, U32, P, U32, P, U32, P, U32, P, P, P, ctypes.POINTER(ctypes.c_uint64), I32]),
        "oracle_max_threads": (I32, []),
        "oracle_wide_fold": (I32, [P, U32, U32, P, P, P, ctypes.POINTER(U32), ctypes.POINTER(U32)]),
        "oracle_wide_fold_mode": (I32, [P, U32, U32, ctypes.c_int, P, P, P, ctypes.POINTER(U32),
                                        ctypes.POINTER(U32)]),
        "oracle_octant_slot_assignment": (I32, [P, U32, P]),
        "oracle_trace_wide": (I32, [P, U32, P, U32, I32, P, P, U32, P, P, I32]),
        "oracle_gen_icosphere": (U32, [ctypes.c_uint64, U32, ctypes.c_float, ctypes.c_float, U32, P]),
        "oracle_camera_look_at": (I32, [P, P, P, ctypes.c_float, U32, U32, P]),
        "oracle_gen_camera_rays": (None, [P, U32, U32, ctypes.c_float, ctypes.c_float, P]),
        "oracle_gen_random_rays": (None, [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_float, ctypes.c_float,
                                          ctypes.c_float, ctypes.c_float, P]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


LIB = _load()


def _p(a):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


REF_SHADER_PATH = os.path.join(HERE, "_ref", "libref_shader.so")
REF_SHADER_SIMPLE_PATH = os.path.join(HERE, "_ref", "libref_shader_simple.so")


def ref_shader_available() -> bool:
    """True where the recipe compiled the reference's own compute shader."""
    return os.path.exists(REF_SHADER_PATH)


def ref_shader_render(tris, mats, nodes, lights, spheres, cam_pos, width: int, height: int, frames: int,
                      first_sample: int = 0, lights_len: int = 1, spheres_len: int = 1,
                      threads: int = 0, simple: bool = False) -> np.ndarray:
    """The reference's ray-trace-compute.comp, compiled from its source via
    glsl2cpp.py, driven frame by frame as src/main.cpp drives it: returns the
    rgba8 target image after `frames` dispatches as floats (H, W, 4). The
    bound lengths of the light and sphere arrays default to 1, as the
    reference application binds them. `simple` runs
    ray-trace-compute-simple.comp instead."""
    lib = ctypes.CDLL(REF_SHADER_SIMPLE_PATH if simple else REF_SHADER_PATH)
    P, U32 = ctypes.c_void_p, ctypes.c_uint32
    lib.ref_shader_render.restype = ctypes.c_int
    lib.ref_shader_render.argtypes = [P, U32, P, U32, P, U32, P, U32, U32, P, U32, U32, P, U32, U32, U32, U32, P,
                                      ctypes.c_int]
    tris, mats, nodes = (np.ascontiguousarray(a, np.float32) for a in (tris, mats, nodes))
    lights = np.ascontiguousarray(lights, np.float32).reshape(-1, 2)
    spheres = np.zeros((1, 8), np.float32) if spheres is None or len(spheres) == 0 else \
        np.ascontiguousarray(spheres, np.float32)
    cam = np.ascontiguousarray(cam_pos, np.float32)
    out = np.zeros((height, width, 4), np.float32)
    rc = lib.ref_shader_render(_p(tris), len(tris), _p(mats), len(mats), _p(nodes), len(nodes), _p(lights),
                               len(lights), lights_len, _p(spheres), len(spheres), spheres_len, _p(cam), width,
                               height, first_sample, frames, _p(out), threads)
    if rc != 0:
        raise RuntimeError(f"ref_shader_render failed ({rc})")
    return out


def ref_shader_trace(tris, nodes, rays, threads: int = 0) -> np.ndarray:
    """The reference shader's own hit_bvh for each ray (its 16-entry stack and
    fixed t range): hit distance or -1 per ray."""
    lib = ctypes.CDLL(REF_SHADER_PATH)
    P, U32 = ctypes.c_void_p, ctypes.c_uint32
    lib.ref_shader_trace.restype = ctypes.c_int
    lib.ref_shader_trace.argtypes = [P, U32, P, U32, P, U32, P, ctypes.c_int]
    tris, nodes, rays = (np.ascontiguousarray(a, np.float32) for a in (tris, nodes, rays))
    t = np.zeros(len(rays), np.float32)
    rc = lib.ref_shader_trace(_p(tris), len(tris), _p(nodes), len(nodes), _p(rays), len(rays), _p(t), threads)
    if rc != 0:
        raise RuntimeError(f"ref_shader_trace failed ({rc})")
    return t


def hit_records(tris, nodes, spheres, rays, flags: int = 0) -> np.ndarray:
    """Shading hit records (n, 10): hit, t, p, normal, material (uint bits),
    back face (int bits) — the `closest` step of ray_color under `flags`."""
    tris, nodes, rays = (np.ascontiguousarray(a, np.float32) for a in (tris, nodes, rays))
    sph = np.zeros((1, 8), np.float32) if spheres is None or len(spheres) == 0 else \
        np.ascontiguousarray(spheres, np.float32)
    ns = 0 if spheres is None else len(spheres)
    out = np.zeros((len(rays), 10), np.float32)
    LIB.oracle_hit_records(_p(tris), len(tris), _p(nodes), len(nodes), _p(sph), ns, _p(rays), len(rays), flags,
                           _p(out))
    return out


def ref_shader_hit_records(tris, nodes, spheres, rays, use_scene: bool, spheres_len: int) -> np.ndarray:
    """The reference shader's own hit_scene (use_scene) or hit_bvh records,
    laid out as hit_records()."""
    lib = ctypes.CDLL(REF_SHADER_PATH)
    P, U32 = ctypes.c_void_p, ctypes.c_uint32
    lib.ref_shader_hit_records.restype = ctypes.c_int
    lib.ref_shader_hit_records.argtypes = [P, U32, P, U32, P, U32, U32, P, U32, ctypes.c_int, P, ctypes.c_int]
    tris, nodes, rays = (np.ascontiguousarray(a, np.float32) for a in (tris, nodes, rays))
    sph = np.zeros((1, 8), np.float32) if spheres is None or len(spheres) == 0 else \
        np.ascontiguousarray(spheres, np.float32)
    out = np.zeros((len(rays), 10), np.float32)
    rc = lib.ref_shader_hit_records(_p(tris), len(tris), _p(nodes), len(nodes), _p(sph), len(sph), spheres_len,
                                    _p(rays), len(rays), 1 if use_scene else 0, _p(out), 0)
    if rc != 0:
        raise RuntimeError(f"ref_shader_hit_records failed ({rc})")
    return out


REF_SCENE_DIR = os.path.join(HERE, "_ref", "doge_scene")


def ref_scene_available() -> bool:
    """True where the recipe copied the reference's demo-scene OBJ files."""
    return os.path.exists(os.path.join(REF_SCENE_DIR, "buff-doge.obj"))


def obj_triangles(path: str, material: int = 0) -> np.ndarray:
    """Restatement of the reference's OBJ-to-triangles step
    (src/scene/mesh.cpp:96-139 through tinyobjloader, then
    src/ray-tracing/RtScene.h:13-31): every face's vertex positions in file
    order, polygons fanned from their first vertex. Coordinates go through
    Python's correctly rounded float() and then to float32; the reference
    scene's six-decimal coordinates round the same way through any parser
    that is accurate to double precision."""
    verts, out = [], []
    with open(path, "rb") as f:
        text = f.read().decode("latin-1")
    for line in text.replace("\r\n", "\n").replace("\r", "\n").split("\n"):
        tok = line.split()
        if not tok:
            continue
        if tok[0] == "v":
            xyz = []
            for t in tok[1:4]:
                try:
                    xyz.append(float(t))
                except ValueError:
                    xyz.append(0.0)
            verts.append((xyz + [0.0, 0.0, 0.0])[:3])
        elif tok[0] == "f":
            ids = []
            for t in tok[1:]:
                i = int(t.split("/")[0])
                if i == 0:
                    raise ValueError("face index 0")
                v = i - 1 if i > 0 else len(verts) + i
                if not 0 <= v < len(verts):
                    raise ValueError("face index out of range")
                ids.append(v)
            for k in range(1, len(ids) - 1):
                row = np.zeros(12, np.float32)
                for j, v in enumerate((ids[0], ids[k], ids[k + 1])):
                    row[4 * j:4 * j + 3] = np.asarray(verts[v], np.float64).astype(np.float32)
                row[11] = np.array([material], np.uint32).view(np.float32)[0]
                out.append(row)
    return np.array(out, np.float32).reshape(-1, 12)


def reference_scene(model_dir: str):
    """Restatement of GpuModel::Scene() (src/ray-tracing/RtScene.h:44-101):
    (tris, mats, spheres) as float32 word arrays."""
    objs = [("buff-doge.obj", 0), ("cheems.obj", 0), ("right.obj", 1), ("left.obj", 2), ("back.obj", 0),
            ("ceil.obj", 0), ("floor.obj", 0), ("light.obj", 3)]
    tris = np.concatenate([obj_triangles(os.path.join(model_dir, f), m) for f, m in objs])
    mats = np.zeros((6, 8), np.float32)
    for i, (typ, alb) in enumerate([(1, (0.3, 0.3, 0.3)), (1, (0.9, 0.1, 0.1)), (1, (0.1, 0.9, 0.1)),
                                    (0, (2.0, 2.0, 2.0)), (2, (1.0, 1.0, 1.0)), (3, (1.0, 1.0, 1.0))]):
        mats[i, 0] = np.array([typ], np.uint32).view(np.float32)[0]
        mats[i, 4:7] = alb
    sph = np.zeros((1, 8), np.float32)
    sph[0, :4] = (0.6, 1.0, -1.0, 0.6)
    sph[0, 4] = np.array([5], np.uint32).view(np.float32)[0]
    return tris, mats, sph


def ref_lib():
    lib = ctypes.CDLL(REF_PATH)
    lib.ref_create_bvh.restype = ctypes.c_int
    lib.ref_create_bvh.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32]
    lib.ref_layout.restype = ctypes.c_int
    lib.ref_layout.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.ref_rand_sequence.restype = None
    lib.ref_rand_sequence.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p]
    return lib


def ref_build_bvh(tris: np.ndarray, seed: int = 1) -> np.ndarray:
    """The reference's own Bvh::createBvh (needs the reference checkout)."""
    tris = np.ascontiguousarray(tris, np.float32)
    out = np.zeros((2 * len(tris) - 1, 12), np.float32)
    rc = ref_lib().ref_create_bvh(_p(tris), len(tris), _p(out), seed)
    if rc != 0:
        raise RuntimeError(f"ref_create_bvh failed ({rc})")
    return out


def build_bvh(tris: np.ndarray, seed: int = 1):
    """The oracle's restatement of Bvh::createBvh. Returns (nodes, depth)."""
    tris = np.ascontiguousarray(tris, np.float32)
    out = np.zeros((2 * len(tris) - 1, 12), np.float32)
    depth = ctypes.c_int()
    rc = LIB.oracle_build_bvh(_p(tris), len(tris), _p(out), seed, ctypes.byref(depth))
    if rc != 0:
        raise RuntimeError("oracle_build_bvh failed")
    return out, depth.value


def glibc_rand(seed: int, count: int) -> np.ndarray:
    out = np.zeros(count, np.int32)
    LIB.oracle_glibc_rand(seed, count, _p(out))
    return out


def sort_with_depth(keys: np.ndarray, depth: int):
    keys = np.ascontiguousarray(keys, np.float32).copy()
    idx = np.arange(len(keys), dtype=np.uint32)
    LIB.oracle_sort_with_depth(_p(keys), _p(idx), len(keys), depth)
    return keys, idx


def lights_from_materials(tris, mats) -> np.ndarray:
    n = LIB.oracle_lights_from_materials(_p(tris), len(tris), _p(mats), len(mats), None)
    out = np.zeros((max(n, 1), 2), np.float32)
    LIB.oracle_lights_from_materials(_p(tris), len(tris), _p(mats), len(mats), _p(out))
    return out[:n]


def camera_from_reference(cam_pos, W: int, H: int) -> np.ndarray:
    p = np.asarray(cam_pos, np.float32)
    out = np.zeros(12, np.float32)
    LIB.oracle_camera_from_reference(_p(p), W, H, _p(out))
    return out


def trace(tris, nodes, rays, mode: int = 0, stack_size: int = 16, slack: float = 1e-5, stats: bool = False,
          threads: int = 0):
    """Closest hit per ray. Returns hits (n,4 float32; col 0 is int32 bits) and optionally stats (n,4 uint32)."""
    rays = np.ascontiguousarray(rays, np.float32)
    hits = np.zeros((len(rays), 4), np.float32)
    st = np.zeros((len(rays), 4), np.uint32) if stats else None
    LIB.oracle_trace(_p(tris), len(tris), _p(nodes), len(nodes), _p(rays), len(rays), mode, stack_size, slack,
                     _p(hits), _p(st), threads)
    return (hits, st) if stats else hits


def wide_fold(nodes, sah: bool = False):
    """The GPU builder's 8-wide fold of a reference node array, restated:
    per node 8 child slots placed by octant (boxes lo.xyz, hi.xyz; refs: the
    child node's number for inner children, ~triangle for leaves, INT_MIN
    empty) and the mask of filled slots; the folded nodes opened largest
    child first, or (sah) chosen by the surface area heuristic. Returns
    (boxes (n8, 8, 6), refs (n8, 8), fmask (n8,), levels)."""
    nodes = np.ascontiguousarray(nodes, np.float32)
    ntris = (len(nodes) + 1) // 2
    cap = max(1, ntris if sah else (4 * ntris + 6) // 7 + 1)
    boxes = np.zeros((cap, 8, 6), np.float32)
    refs = np.zeros((cap, 8), np.int32)
    fmask = np.zeros(cap, np.uint32)
    n8, levels = ctypes.c_uint32(0), ctypes.c_uint32(0)
    rc = LIB.oracle_wide_fold_mode(_p(nodes), len(nodes), cap, 1 if sah else 0, _p(boxes), _p(refs), _p(fmask),
                                   ctypes.byref(n8), ctypes.byref(levels))
    if rc != 0:
        raise RuntimeError(f"oracle_wide_fold failed ({rc})")
    n = n8.value
    return boxes[:n], refs[:n], fmask[:n], levels.value


def octant_slots(boxes) -> np.ndarray:
    """Slot of each of 1..8 child boxes (lo.xyz, hi.xyz) under the fold's
    octant rule."""
    b = np.ascontiguousarray(boxes, np.float32).reshape(-1, 6)
    out = np.zeros(len(b), np.int32)
    if LIB.oracle_octant_slot_assignment(_p(b), len(b), _p(out)) != 0:
        raise ValueError("1..8 boxes expected")
    return out


def trace_wide(tris, qwords, root8: int, root_box, rays, threads: int = 0, stats: bool = False):
    """Closest hits through quantized 8-wide nodes (qwords: (n8, 24) uint32;
    root8: the root node's number), with the GPU kernel's plane arithmetic
    and visiting order; hits as oracle `trace`, and with stats=True also
    (n, 2) uint32: nodes visited, triangles tested."""
    tris, rays = np.ascontiguousarray(tris, np.float32), np.ascontiguousarray(rays, np.float32)
    qwords = np.ascontiguousarray(qwords, np.uint32)
    rb = np.ascontiguousarray(root_box, np.float32)
    hits = np.zeros((len(rays), 4), np.float32)
    st = np.zeros((len(rays), 2), np.uint32) if stats else None
    rc = LIB.oracle_trace_wide(_p(tris), len(tris), _p(qwords), len(qwords), root8, _p(rb), _p(rays), len(rays),
                               _p(hits), _p(st), threads)
    if rc != 0:
        raise RuntimeError(f"oracle_trace_wide failed ({rc})")
    return (hits, st) if stats else hits


def trace_f64(tris, nodes, rays, threads: int = 0):
    rays = np.ascontiguousarray(rays, np.float32)
    tri = np.zeros(len(rays), np.int32)
    tuv = np.zeros((len(rays), 3), np.float64)
    LIB.oracle_trace_f64(_p(tris), len(tris), _p(nodes), len(nodes), _p(rays), len(rays), _p(tri), _p(tuv), threads)
    return tri, tuv


class _Params(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("spp", ctypes.c_uint32),
                ("max_bounces", ctypes.c_uint32), ("sample_index", ctypes.c_uint32), ("flags", ctypes.c_uint32),
                ("_reserved", ctypes.c_uint32 * 2)]


def render(tris, mats, nodes, lights, spheres, camera: np.ndarray, width: int, height: int, spp: int = 1,
           max_bounces: int = 8, sample_index: int = 0, flags: int = 0, accum=None, f64: bool = False,
           threads: int = 0):
    """Progressive render (in place on `accum`, W*H*4). Returns (accum, segments)."""
    lights = np.zeros((0, 2), np.float32) if lights is None else np.ascontiguousarray(lights, np.float32)
    spheres = np.zeros((0, 8), np.float32) if spheres is None else np.ascontiguousarray(spheres, np.float32)
    cam = np.ascontiguousarray(camera, np.float32).reshape(12)
    if accum is None:
        accum = np.zeros((height, width, 4), np.float64 if f64 else np.float32)
    p = _Params(width, height, spp, max_bounces, sample_index, flags)
    seg = ctypes.c_uint64()
    fn = LIB.oracle_render_f64 if f64 else LIB.oracle_render
    fn(_p(tris), len(tris), _p(mats), len(mats), _p(nodes), len(nodes), _p(lights) if len(lights) else None,
       len(lights), _p(spheres) if len(spheres) else None, len(spheres), _p(cam), ctypes.addressof(p), _p(accum),
       ctypes.byref(seg), threads)
    return accum, seg.value


def denoise(img: np.ndarray, sigma: float = 2.0, ksigma: float = 2.0, threshold: float = 0.05,
            mix: float = 1.0) -> np.ndarray:
    """smartDeNoise restatement on an (H, W, 4) float32 image."""
    img = np.ascontiguousarray(img, np.float32)
    out = np.zeros_like(img)
    LIB.oracle_denoise(_p(img), img.shape[1], img.shape[0], sigma, ksigma, threshold, mix, _p(out))
    return out


def max_threads() -> int:
    return LIB.oracle_max_threads()


# ------------------------------------------------------------------ workloads
# The seeded inputs of the closest-hit measurement (oracle/workloads.cpp),
# byte-equal to the product library's generators, so that the reference arm
# of the bench makes its inputs without the product library.

def gen_icosphere(seed: int, level: int, radius: float = 1.0, sigma: float = 0.05, material: int = 0):
    n = LIB.oracle_gen_icosphere(seed, level, radius, sigma, material, None)
    out = np.zeros((n, 12), np.float32)
    LIB.oracle_gen_icosphere(seed, level, radius, sigma, material, _p(out))
    return out


def camera_look_at(eye, target, up, vfov_deg: float, width: int, height: int) -> np.ndarray:
    """12 floats: origin, lower-left, horizontal, vertical."""
    e, t, u = (np.ascontiguousarray(x, np.float32) for x in (eye, target, up))
    cam = np.zeros(12, np.float32)
    if not LIB.oracle_camera_look_at(_p(e), _p(t), _p(u), vfov_deg, width, height, _p(cam)):
        raise ValueError("degenerate camera")
    return cam


def gen_camera_rays(cam: np.ndarray, width: int, height: int, tmin: float = 1e-4, tmax: float = 1e4):
    cam = np.ascontiguousarray(cam, np.float32).reshape(12)
    rays = np.zeros((width * height, 8), np.float32)
    LIB.oracle_gen_camera_rays(_p(cam), width, height, tmin, tmax, _p(rays))
    return rays


def gen_random_rays(seed: int, n: int, lo: float = -1.5, hi: float = 1.5, tmin: float = 1e-4, tmax: float = 1e4):
    rays = np.zeros((n, 8), np.float32)
    LIB.oracle_gen_random_rays(seed, n, lo, hi, tmin, tmax, _p(rays))
    return rays


def closest_hit_workload(side: int = 2048, level: int = 8):
    """The closest-hit measurement's inputs: the displaced icosphere (seed 1,
    radius 1, sigma 0.05), side x side primary rays of a pinhole at
    (0, 0, -3) looking at the origin with a 40 degree field of view, and
    side^2 random rays (seed 3, origins in [-1.5, 1.5]^3)."""
    tris = gen_icosphere(1, level)
    cam = camera_look_at([0, 0, -3], [0, 0, 0], [0, 1, 0], 40.0, side, side)
    return tris, gen_camera_rays(cam, side, side), gen_random_rays(3, side * side)
