"""Python mirror of include/rtgb/rt_serve.h (the render server)."""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import LIB, Camera, Context, RtError, _ptr, _words, TRIANGLE_WORDS, MATERIAL_WORDS, SPHERE_WORDS

QUEUED, RUNNING, DONE, FAILED = 0, 1, 2, 3


class ServerDesc(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("max_active", ctypes.c_uint32),
                ("spp_per_step", ctypes.c_uint32), ("_reserved", ctypes.c_uint32 * 4)]


class Request(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_uint32), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("spp", ctypes.c_uint32), ("max_bounces", ctypes.c_uint32), ("flags", ctypes.c_uint32),
                ("camera", Camera), ("host_out", ctypes.c_void_p)]


class RequestStatus(ctypes.Structure):
    _fields_ = [("state", ctypes.c_uint32), ("error", ctypes.c_int32), ("submit_ms", ctypes.c_double),
                ("start_ms", ctypes.c_double), ("done_ms", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("steps", ctypes.c_uint64), ("scene_uploads", ctypes.c_uint64),
                ("scene_evictions", ctypes.c_uint64), ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double),
                ("mean_ms", ctypes.c_double), ("busy_ms", ctypes.c_double), ("resident_bytes", ctypes.c_uint64)]


_P, _U32, _U64, _I32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
for _name, (_res, _args) in {
    "rtServerCreate": (_I32, [_P, ctypes.POINTER(ServerDesc), ctypes.POINTER(_P)]),
    "rtServerDestroy": (_I32, [_P]),
    "rtServerAddScene": (_I32, [_P, _P, _U32, _P, _U32, _P, _U32, ctypes.POINTER(_U32)]),
    "rtServerSubmit": (_I32, [_P, ctypes.POINTER(Request), ctypes.POINTER(_U64)]),
    "rtServerPoll": (_I32, [_P, _U64, ctypes.POINTER(RequestStatus)]),
    "rtServerWait": (_I32, [_P, _U64, _U32, ctypes.POINTER(RequestStatus)]),
    "rtServerStats": (_I32, [_P, ctypes.POINTER(ServerStats)]),
    "rtServerResetStats": (_I32, [_P]),
}.items():
    _fn = getattr(LIB, _name)
    _fn.restype = _res
    _fn.argtypes = _args


class Server:
    """Continuous-batching render server (rtServerCreate)."""

    def __init__(self, ctx: Context, hbm_budget_bytes: int = 0, max_active: int = 0, spp_per_step: int = 0):
        self.ctx = ctx
        d = ServerDesc(hbm_budget_bytes, max_active, spp_per_step)
        h = ctypes.c_void_p()
        st = LIB.rtServerCreate(ctx.handle, ctypes.byref(d), ctypes.byref(h))
        if st:
            raise RtError(st, "rtServerCreate")
        self.handle = h
        self._outs = {}

    def close(self):
        if self.handle:
            LIB.rtServerDestroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def add_scene(self, tris, mats, spheres=None) -> int:
        tris = _words(tris, TRIANGLE_WORDS, "triangles")
        mats = _words(mats, MATERIAL_WORDS, "materials")
        sph = None if spheres is None or len(spheres) == 0 else _words(spheres, SPHERE_WORDS, "spheres")
        hid = ctypes.c_uint32()
        st = LIB.rtServerAddScene(self.handle, _ptr(tris), len(tris), _ptr(mats), len(mats), _ptr(sph),
                                  0 if sph is None else len(sph), ctypes.byref(hid))
        if st:
            raise RtError(st, "rtServerAddScene")
        return hid.value

    def submit(self, scene: int, cam: Camera, width: int, height: int, spp: int, max_bounces: int = 8,
               flags: int = 0, keep_image: bool = True) -> int:
        out = np.zeros((height, width, 4), np.float32) if keep_image else None
        req = Request(scene, width, height, spp, max_bounces, flags, cam, _ptr(out))
        rid = ctypes.c_uint64()
        st = LIB.rtServerSubmit(self.handle, ctypes.byref(req), ctypes.byref(rid))
        if st:
            raise RtError(st, "rtServerSubmit")
        self._outs[rid.value] = out
        return rid.value

    def wait(self, rid: int, timeout_ms: int = 0) -> RequestStatus:
        s = RequestStatus()
        st = LIB.rtServerWait(self.handle, rid, timeout_ms, ctypes.byref(s))
        if st:
            raise RtError(st, "rtServerWait")
        return s

    def poll(self, rid: int) -> RequestStatus:
        s = RequestStatus()
        st = LIB.rtServerPoll(self.handle, rid, ctypes.byref(s))
        if st:
            raise RtError(st, "rtServerPoll")
        return s

    def image(self, rid: int) -> Optional[np.ndarray]:
        return self._outs.get(rid)

    def stats(self) -> ServerStats:
        s = ServerStats()
        LIB.rtServerStats(self.handle, ctypes.byref(s))
        return s

    def reset_stats(self):
        LIB.rtServerResetStats(self.handle)
