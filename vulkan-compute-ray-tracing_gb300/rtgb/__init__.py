"""Python mirror of the C ABI in include/rtgb/rt_api.h (ctypes).

The reference drives its ray-trace path from C++: it fills a GpuModel::Scene
(src/ray-tracing/RtScene.h), binds it to a ComputeMaterial
(src/scene/ComputeMaterial.cpp) and dispatches a ComputeModel once per frame
(src/scene/ComputeModel.cpp:21-25). Here the same steps are ``Context``
(device + stream), ``Context.upload_scene`` (scene + BVH resident in HBM) and
``Scene.render`` / ``Scene.trace`` (one stream-ordered call each), all thin
wrappers over librtgb.so. Arrays are numpy arrays in the reference's std430
layouts (see ``TRIANGLE_WORDS`` etc.) or torch CUDA tensors for device data.

The library is required: importing this module raises if librtgb.so is
missing or fails to load — there is no fallback implementation.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "librtgb.so")

# Record sizes in 32-bit words (the reference's std430 strides).
TRIANGLE_WORDS = 12  # 48 B: v0@0 v1@16 v2@32 material@44
MATERIAL_WORDS = 8   # 32 B: type@0 fuzz@4 ior@8 albedo@16
NODE_WORDS = 12      # 48 B: min@0 max@16 left@28 right@32 object@36
LIGHT_WORDS = 2      # 8 B: triangle@0 area@4
SPHERE_WORDS = 8     # 32 B: centre+radius@0 material@16
RAY_WORDS = 8        # 32 B: o tmin d tmax
HIT_WORDS = 4        # 16 B: tri t u v

MATERIAL_LIGHT, MATERIAL_LAMBERTIAN, MATERIAL_METAL, MATERIAL_GLASS = 0, 1, 2, 3

COMPAT_STACK16 = 1 << 0
COMPAT_LEN1 = 1 << 1
COMPAT_SPHERE_OVERRIDE = 1 << 2
COMPAT_NO_SPHERES = 1 << 3
COMPAT_UNORM8 = 1 << 4
SHADE_SIMPLE = 1 << 5
HIT_FP32 = 1 << 6

STATUS = {0: "RT_SUCCESS", 1: "RT_ERR_INVALID_ARGUMENT", 2: "RT_ERR_OUT_OF_MEMORY", 3: "RT_ERR_CUDA",
          4: "RT_ERR_NOT_FOUND", 5: "RT_ERR_INVALID_SCENE", 6: "RT_ERR_STACK_OVERFLOW", 7: "RT_ERR_TIMEOUT",
          8: "RT_ERR_BUDGET", 9: "RT_ERR_BUSY", 10: "RT_ERR_INTERNAL"}


class RtError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class Camera(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_float * 3), ("lower_left", ctypes.c_float * 3),
                ("horizontal", ctypes.c_float * 3), ("vertical", ctypes.c_float * 3)]

    def as_array(self) -> np.ndarray:
        return np.ctypeslib.as_array(ctypes.cast(ctypes.pointer(self), ctypes.POINTER(ctypes.c_float)),
                                     shape=(12,)).copy()


class RenderParams(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("spp", ctypes.c_uint32),
                ("max_bounces", ctypes.c_uint32), ("sample_index", ctypes.c_uint32), ("flags", ctypes.c_uint32),
                ("_reserved", ctypes.c_uint32 * 2)]


class CtxDesc(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("hbm_budget_bytes", ctypes.c_uint64), ("flags", ctypes.c_uint32),
                ("_reserved", ctypes.c_uint32)]


class SceneInfo(ctypes.Structure):
    _fields_ = [("triangles", ctypes.c_uint32), ("materials", ctypes.c_uint32), ("lights", ctypes.c_uint32),
                ("spheres", ctypes.c_uint32), ("nodes", ctypes.c_uint32), ("depth", ctypes.c_uint32),
                ("device_bytes", ctypes.c_uint64), ("build_ms", ctypes.c_float), ("relayout_ms", ctypes.c_float)]


class RenderJob(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_uint32), ("_pad", ctypes.c_uint32), ("camera", Camera),
                ("params", RenderParams), ("d_rgba32f", ctypes.c_void_p)]


def _load() -> ctypes.CDLL:
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"librtgb.so not found at {LIB_PATH}: build it with "
                          f"`python vulkan-compute-ray-tracing_gb300/build.py`")
    lib = ctypes.CDLL(LIB_PATH)
    P = ctypes.c_void_p
    U32, U64, I32, F32 = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int, ctypes.c_float
    sigs = {
        "rtCreate": (I32, [ctypes.POINTER(P), ctypes.POINTER(CtxDesc)]),
        "rtDestroy": (I32, [P]),
        "rtGetLastError": (ctypes.c_char_p, [P]),
        "rtStatusString": (ctypes.c_char_p, [I32]),
        "rtUploadScene": (I32, [P, P, U32, P, U32, P, U32, P, U32, P, U32, U32, ctypes.POINTER(U32)]),
        "rtReleaseScene": (I32, [P, U32]),
        "rtGetSceneInfo": (I32, [P, U32, ctypes.POINTER(SceneInfo)]),
        "rtDownloadBvh": (I32, [P, U32, P, U32]),
        "rtDownloadLights": (I32, [P, U32, P, U32]),
        "rtLightsFromMaterials": (U32, [P, U32, P, U32, P]),
        "rtCameraFromReference": (I32, [P, U32, U32, ctypes.POINTER(Camera)]),
        "rtCameraLookAt": (I32, [P, P, P, F32, U32, U32, ctypes.POINTER(Camera)]),
        "rtSetCamera": (I32, [P, U32, ctypes.POINTER(Camera)]),
        "rtRender": (I32, [P, U32, ctypes.POINTER(RenderParams), P, P]),
        "rtTraceClosest": (I32, [P, U32, P, U32, P, P]),
        "rtTraceClosestEx": (I32, [P, U32, P, U32, P, U32, P]),
        "rtTraceClosestHost": (I32, [P, U32, P, U32, P]),
        "rtSynchronize": (I32, [P, P]),
        "rtSetTuning": (I32, [P, ctypes.c_char_p, ctypes.c_int64]),
        "rtGetTuning": (I32, [P, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int64)]),
        "rtReadSegmentCounter": (I32, [P, ctypes.POINTER(U64), I32]),
        "rtRenderBatch": (I32, [P, ctypes.POINTER(RenderJob), U32, P]),
        "rtBatchCreate": (I32, [P, ctypes.POINTER(RenderJob), U32, ctypes.POINTER(P)]),
        "rtBatchDestroy": (I32, [P, P]),
        "rtBatchLaunch": (I32, [P, P, P]),
        "rtBatchAdvance": (I32, [P, P, P]),
        "rtBatchLaunchGraph": (I32, [P, P, P]),
        "rtBuildBvhNoAlloc": (I32, [P, U32, U32, P, P]),
        "rtExportImage": (I32, [P, P, U32, U32, F32, P, P]),
        "rtDenoiseImage": (I32, [P, P, U32, U32, F32, F32, F32, F32, P, P]),
        "rtAutotuneTrace": (I32, [P, U32, P, U32, P, U32, ctypes.POINTER(ctypes.c_double),
                                  ctypes.POINTER(ctypes.c_double)]),
        "rtAutotuneRender": (I32, [P, U32, U32, U32, U32, ctypes.POINTER(U64)]),
        "rtgbGenCornell": (U32, [U64, U32, U32, F32, F32, F32, P, P, P]),
        "rtgbGenIcosphere": (U32, [U64, U32, F32, F32, U32, P]),
        "rtgbGenCameraRays": (None, [ctypes.POINTER(Camera), U32, U32, F32, F32, P]),
        "rtgbGenRandomRays": (None, [U64, U64, F32, F32, F32, F32, P]),
        "rtgbGenGrid": (U32, [U64, U32, U32, U32, F32, F32, U32, F32, P, P]),
        "rtgbUniform": (ctypes.c_double, [U64, U64]),
        "rtgbQuantizeNode8": (ctypes.c_uint32, [P, P, U32, P]),
        "rtgbGlibcRand": (None, [U32, U64, P]),
        "rtLoadObj": (I32, [ctypes.c_char_p, U32, P, U32, ctypes.POINTER(U32)]),
        "rtObjLastError": (ctypes.c_char_p, []),
        "rtLoadReferenceScene": (I32, [ctypes.c_char_p, P, U32, ctypes.POINTER(U32), P, P]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


LIB = _load()


def _ptr(a) -> Optional[int]:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("arrays must be C-contiguous")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):  # torch tensor
        return int(a.data_ptr())
    return int(a)


def _words(a, words: int, name: str) -> np.ndarray:
    a = np.ascontiguousarray(a)
    if a.dtype.itemsize != 4 or a.size % words:
        raise ValueError(f"{name}: expected 32-bit words in records of {words}")
    return a.reshape(-1, words)


# ---------------------------------------------------------------- generators
def gen_cornell(seed: int, n_soup: int, n_spheres: int = 0, r_lo: float = 0.2, r_hi: float = 1.0,
                light_radiance: float = 4.0):
    """Cornell box + soup (see include/rtgb/rt_scenes.h). Returns (tris, mats, spheres)."""
    tris = np.zeros((12 + n_soup, TRIANGLE_WORDS), np.float32)
    mats = np.zeros((8, MATERIAL_WORDS), np.float32)
    sph = np.zeros((max(n_spheres, 1), SPHERE_WORDS), np.float32)
    LIB.rtgbGenCornell(seed, n_soup, n_spheres, r_lo, r_hi, light_radiance, _ptr(tris), _ptr(mats), _ptr(sph))
    return tris, mats, sph[:n_spheres]


def gen_icosphere(seed: int, level: int, radius: float = 1.0, sigma: float = 0.05, material: int = 0):
    n = LIB.rtgbGenIcosphere(seed, level, radius, sigma, material, None)
    tris = np.zeros((n, TRIANGLE_WORDS), np.float32)
    LIB.rtgbGenIcosphere(seed, level, radius, sigma, material, _ptr(tris))
    return tris


def gen_grid(seed: int, gx: int, gz: int, level: int, flatten: float, sigma: float, keep: int, box_scale: float):
    n = LIB.rtgbGenGrid(seed, gx, gz, level, flatten, sigma, keep, box_scale, None, None)
    tris = np.zeros((n, TRIANGLE_WORDS), np.float32)
    mats = np.zeros((8, MATERIAL_WORDS), np.float32)
    LIB.rtgbGenGrid(seed, gx, gz, level, flatten, sigma, keep, box_scale, _ptr(tris), _ptr(mats))
    return tris, mats


def camera_look_at(eye, target, up, vfov_deg: float, width: int, height: int) -> Camera:
    cam = Camera()
    e = np.asarray(eye, np.float32)
    t = np.asarray(target, np.float32)
    u = np.asarray(up, np.float32)
    st = LIB.rtCameraLookAt(_ptr(e), _ptr(t), _ptr(u), vfov_deg, width, height, ctypes.byref(cam))
    if st:
        raise RtError(st, "rtCameraLookAt")
    return cam


def camera_from_reference(cam_pos, width: int, height: int) -> Camera:
    cam = Camera()
    p = np.asarray(cam_pos, np.float32)
    st = LIB.rtCameraFromReference(_ptr(p), width, height, ctypes.byref(cam))
    if st:
        raise RtError(st, "rtCameraFromReference")
    return cam


def gen_camera_rays(cam: Camera, width: int, height: int, tmin: float = 1e-4, tmax: float = 1e4) -> np.ndarray:
    rays = np.zeros((width * height, RAY_WORDS), np.float32)
    LIB.rtgbGenCameraRays(ctypes.byref(cam), width, height, tmin, tmax, _ptr(rays))
    return rays


def gen_random_rays(seed: int, n: int, lo: float = -1.5, hi: float = 1.5, tmin: float = 1e-4,
                    tmax: float = 1e4) -> np.ndarray:
    rays = np.zeros((n, RAY_WORDS), np.float32)
    LIB.rtgbGenRandomRays(seed, n, lo, hi, tmin, tmax, _ptr(rays))
    return rays


def load_obj(path: str, material: int = 0) -> np.ndarray:
    """Triangles of one OBJ file, all with `material` (GpuModel::getTriangles,
    src/ray-tracing/RtScene.h:13-31). Raises RtError on a missing file or a
    bad face index."""
    n = ctypes.c_uint32()
    st = LIB.rtLoadObj(os.fsencode(path), material, None, 0, ctypes.byref(n))
    if st:
        raise RtError(st, LIB.rtObjLastError().decode())
    tris = np.zeros((max(n.value, 1), TRIANGLE_WORDS), np.float32)
    st = LIB.rtLoadObj(os.fsencode(path), material, _ptr(tris), n.value, ctypes.byref(n))
    if st:
        raise RtError(st, LIB.rtObjLastError().decode())
    return tris[:n.value]


def load_reference_scene(model_dir: str):
    """The reference's doge scene (src/ray-tracing/RtScene.h:44-101) from the
    directory holding its OBJ files. Returns (tris, mats, spheres); lights
    are derived by upload_scene (or lights_from_materials)."""
    n = ctypes.c_uint32()
    st = LIB.rtLoadReferenceScene(os.fsencode(model_dir), None, 0, ctypes.byref(n), None, None)
    if st:
        raise RtError(st, LIB.rtObjLastError().decode())
    tris = np.zeros((max(n.value, 1), TRIANGLE_WORDS), np.float32)
    mats = np.zeros((6, MATERIAL_WORDS), np.float32)
    sph = np.zeros((1, SPHERE_WORDS), np.float32)
    st = LIB.rtLoadReferenceScene(os.fsencode(model_dir), _ptr(tris), n.value, ctypes.byref(n), _ptr(mats),
                                  _ptr(sph))
    if st:
        raise RtError(st, LIB.rtObjLastError().decode())
    return tris[:n.value], mats, sph


# The reference's starting camera position (src/main.cpp:37), for
# camera_from_reference.
REFERENCE_CAMERA_POS = (1.8, 8.6, 1.1)


def lights_from_materials(tris: np.ndarray, mats: np.ndarray) -> np.ndarray:
    tris = _words(tris, TRIANGLE_WORDS, "triangles")
    mats = _words(mats, MATERIAL_WORDS, "materials")
    n = LIB.rtLightsFromMaterials(_ptr(tris), len(tris), _ptr(mats), len(mats), None)
    out = np.zeros((max(n, 1), LIGHT_WORDS), np.float32)
    LIB.rtLightsFromMaterials(_ptr(tris), len(tris), _ptr(mats), len(mats), _ptr(out))
    return out[:n]


def glibc_rand(seed: int, count: int) -> np.ndarray:
    out = np.zeros(count, np.int32)
    LIB.rtgbGlibcRand(seed, count, _ptr(out))
    return out


# ---------------------------------------------------------------- runtime
class Context:
    """A device, its stream and the resident scenes (rtCreate / rtDestroy)."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        desc = CtxDesc(device, hbm_budget_bytes, 0, 0)
        h = ctypes.c_void_p()
        st = LIB.rtCreate(ctypes.byref(h), ctypes.byref(desc))
        if st:
            raise RtError(st, "rtCreate failed")
        self.handle = h

    def close(self):
        if self.handle:
            LIB.rtDestroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, st: int, what: str = ""):
        if st:
            msg = LIB.rtGetLastError(self.handle)
            raise RtError(st, f"{what}: {msg.decode() if msg else ''}")

    def upload_scene(self, tris, mats, nodes=None, lights=None, spheres=None, bvh_seed: int = 1) -> "Scene":
        tris = _words(tris, TRIANGLE_WORDS, "triangles")
        mats = _words(mats, MATERIAL_WORDS, "materials")
        nodes = None if nodes is None else _words(nodes, NODE_WORDS, "nodes")
        lights = None if lights is None else _words(lights, LIGHT_WORDS, "lights")
        spheres = None if spheres is None or len(spheres) == 0 else _words(spheres, SPHERE_WORDS, "spheres")
        sid = ctypes.c_uint32()
        st = LIB.rtUploadScene(self.handle, _ptr(tris), len(tris), _ptr(mats), len(mats),
                               _ptr(nodes), 0 if nodes is None else len(nodes),
                               _ptr(lights), 0 if lights is None else len(lights),
                               _ptr(spheres), 0 if spheres is None else len(spheres), bvh_seed, ctypes.byref(sid))
        self.check(st, "rtUploadScene")
        return Scene(self, sid.value)

    def set_tuning(self, key: str, value: int):
        self.check(LIB.rtSetTuning(self.handle, key.encode(), int(value)), "rtSetTuning")

    def get_tuning(self, key: str) -> int:
        v = ctypes.c_int64()
        self.check(LIB.rtGetTuning(self.handle, key.encode(), ctypes.byref(v)), "rtGetTuning")
        return v.value

    def synchronize(self, stream=None):
        self.check(LIB.rtSynchronize(self.handle, stream), "rtSynchronize")

    def segments(self, reset: bool = False) -> int:
        v = ctypes.c_uint64()
        self.check(LIB.rtReadSegmentCounter(self.handle, ctypes.byref(v), int(reset)), "rtReadSegmentCounter")
        return v.value

    def render_batch(self, jobs, stream=None):
        arr = (RenderJob * len(jobs))(*jobs)
        self.check(LIB.rtRenderBatch(self.handle, arr, len(jobs), stream), "rtRenderBatch")

    def batch(self, jobs) -> "Batch":
        arr = (RenderJob * len(jobs))(*jobs)
        h = ctypes.c_void_p()
        self.check(LIB.rtBatchCreate(self.handle, arr, len(jobs), ctypes.byref(h)), "rtBatchCreate")
        return Batch(self, h)


def make_job(scene: "Scene", cam: Camera, accum, width: int, height: int, spp: int = 1, max_bounces: int = 8,
             sample_index: int = 0, flags: int = 0) -> RenderJob:
    return RenderJob(scene.id, 0, cam, RenderParams(width, height, spp, max_bounces, sample_index, flags),
                     _ptr(accum))


class Batch:
    """A resident job table (rtBatchCreate) launched as one persistent kernel."""

    def __init__(self, ctx: "Context", handle):
        self.ctx = ctx
        self.handle = handle

    def launch(self, stream=None):
        self.ctx.check(LIB.rtBatchLaunch(self.ctx.handle, self.handle, stream), "rtBatchLaunch")

    def advance(self, stream=None):
        self.ctx.check(LIB.rtBatchAdvance(self.ctx.handle, self.handle, stream), "rtBatchAdvance")

    def launch_graph(self, stream=None):
        self.ctx.check(LIB.rtBatchLaunchGraph(self.ctx.handle, self.handle, stream), "rtBatchLaunchGraph")

    def destroy(self):
        if self.handle:
            self.ctx.check(LIB.rtBatchDestroy(self.ctx.handle, self.handle), "rtBatchDestroy")
            self.handle = None


class Scene:
    """A resident scene (rtUploadScene result)."""

    def __init__(self, ctx: Context, sid: int):
        self.ctx = ctx
        self.id = sid

    def info(self) -> SceneInfo:
        inf = SceneInfo()
        self.ctx.check(LIB.rtGetSceneInfo(self.ctx.handle, self.id, ctypes.byref(inf)), "rtGetSceneInfo")
        return inf

    def release(self):
        self.ctx.check(LIB.rtReleaseScene(self.ctx.handle, self.id), "rtReleaseScene")

    def bvh(self) -> np.ndarray:
        n = self.info().nodes
        out = np.zeros((n, NODE_WORDS), np.float32)
        self.ctx.check(LIB.rtDownloadBvh(self.ctx.handle, self.id, _ptr(out), n), "rtDownloadBvh")
        return out

    def lights(self) -> np.ndarray:
        n = self.info().lights
        out = np.zeros((max(n, 1), LIGHT_WORDS), np.float32)
        self.ctx.check(LIB.rtDownloadLights(self.ctx.handle, self.id, _ptr(out), n), "rtDownloadLights")
        return out[:n]

    def set_camera(self, cam: Camera):
        self.ctx.check(LIB.rtSetCamera(self.ctx.handle, self.id, ctypes.byref(cam)), "rtSetCamera")

    def render(self, accum, width: int, height: int, spp: int = 1, max_bounces: int = 8, sample_index: int = 0,
               flags: int = 0, stream=None):
        """Accumulate into a device RGBA32F image (torch tensor or device pointer)."""
        p = RenderParams(width, height, spp, max_bounces, sample_index, flags)
        self.ctx.check(LIB.rtRender(self.ctx.handle, self.id, ctypes.byref(p), _ptr(accum), stream), "rtRender")

    def trace(self, d_rays, n: int, d_hits, flags: int = 0, stream=None):
        """Closest hit for n device rays into device hits."""
        self.ctx.check(LIB.rtTraceClosestEx(self.ctx.handle, self.id, _ptr(d_rays), n, _ptr(d_hits), flags, stream),
                       "rtTraceClosest")

    def trace_host(self, rays: np.ndarray, hits: Optional[np.ndarray] = None) -> np.ndarray:
        """Closest hit for host rays (copies in and out inside the call)."""
        rays = _words(rays, RAY_WORDS, "rays")
        if hits is None:
            hits = np.zeros((len(rays), HIT_WORDS), np.float32)
        self.ctx.check(LIB.rtTraceClosestHost(self.ctx.handle, self.id, _ptr(rays), len(rays), _ptr(hits)),
                       "rtTraceClosestHost")
        return hits


def export_image(ctx: "Context", d_rgba32f, width: int, height: int, d_rgba8, gamma: float = 2.2, stream=None):
    """RGBA32F device image -> gamma-encoded RGBA8 device image (rtExportImage)."""
    ctx.check(LIB.rtExportImage(ctx.handle, _ptr(d_rgba32f), width, height, gamma, _ptr(d_rgba8), stream),
              "rtExportImage")


def autotune_trace(scene: "Scene", d_rays, n: int, d_hits, reps: int = 3):
    """Times the closest-hit launch shapes on these device rays and keeps the
    fastest (rtAutotuneTrace). Returns (Grays/s before, Grays/s after)."""
    a, b = ctypes.c_double(), ctypes.c_double()
    scene.ctx.check(LIB.rtAutotuneTrace(scene.ctx.handle, scene.id, _ptr(d_rays), n, _ptr(d_hits), reps,
                                        ctypes.byref(a), ctypes.byref(b)), "rtAutotuneTrace")
    return a.value, b.value


def autotune_render(scene: "Scene", spp: int = 1, max_bounces: int = 8, max_side: int = 2048) -> int:
    """Chooses the megakernel/wavefront split for this scene (rtAutotuneRender);
    returns the new render.wavefront_pixels."""
    px = ctypes.c_uint64()
    scene.ctx.check(LIB.rtAutotuneRender(scene.ctx.handle, scene.id, spp, max_bounces, max_side, ctypes.byref(px)),
                    "rtAutotuneRender")
    return px.value


def denoise_image(ctx: "Context", d_in, width: int, height: int, d_out, sigma: float = 2.0, ksigma: float = 2.0,
                  threshold: float = 0.05, mix: float = 1.0, stream=None):
    """smartDeNoise of an RGBA32F device image into another (rtDenoiseImage);
    the reference's disabled setting is sigma 2, kSigma 2, threshold 0.05,
    mix 0.5."""
    ctx.check(LIB.rtDenoiseImage(ctx.handle, _ptr(d_in), width, height, sigma, ksigma, threshold, mix, _ptr(d_out),
                                 stream), "rtDenoiseImage")


def write_ppm(path: str, rgba8: np.ndarray) -> None:
    """Writes an (H, W, 4) uint8 image as a binary PPM (alpha dropped)."""
    h, w = rgba8.shape[:2]
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (w, h))
        f.write(np.ascontiguousarray(rgba8[:, :, :3]).tobytes())


def hits_view(hits: np.ndarray):
    """(tri int32, t, u, v) views of an (n, 4) hit array."""
    h = np.ascontiguousarray(hits).reshape(-1, HIT_WORDS)
    return h.view(np.int32)[:, 0], h[:, 1], h[:, 2], h[:, 3]
