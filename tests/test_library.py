"""CPU tests of the product library that need no GPU: it loads, exports every
function the public headers declare, and its std::sort replay (compiled as
host code) matches libstdc++."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

from conftest import PKG, ROOT


def declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include", "rtgb")
    for fn in os.listdir(inc):
        src = open(os.path.join(inc, fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(rt[A-Za-z0-9_]+)\s*\(", src, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_api():
    names = declared_functions()
    for must in ("rtCreate", "rtDestroy", "rtUploadScene", "rtRender", "rtTraceClosest", "rtTraceClosestHost",
                 "rtSetCamera", "rtCameraFromReference", "rtRenderBatch", "rtGetLastError"):
        assert must in names


def test_library_exports_every_declared_symbol(rt):
    lib = ctypes.CDLL(rt.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_library_is_sm103a_only():
    # The build recipe compiles for exactly one target.
    src = open(os.path.join(PKG, "build.py")).read()
    assert "arch=compute_103a,code=sm_103a" in src


def test_status_strings(rt):
    for code in range(11):
        s = rt.LIB.rtStatusString(code)
        assert s and s.decode()
    assert rt.LIB.rtStatusString(99).decode() == "unknown status"


def test_sort_replay_matches_libstdcxx():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "sort_check")
        subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(PKG, "csrc"),
                        os.path.join(ROOT, "tests", "sort_check.cpp"), "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout + out.stderr
        assert out.stdout.startswith("ok ")


def test_null_arguments_are_rejected(rt):
    # Argument checks happen before any device work.
    assert rt.LIB.rtCreate(None, None) == 1
    assert rt.LIB.rtDestroy(None) == 1
    cam = rt.Camera()
    assert rt.LIB.rtCameraFromReference(None, 8, 8, ctypes.byref(cam)) == 1
    p = (ctypes.c_float * 3)(0, 0, 0)
    assert rt.LIB.rtCameraFromReference(p, 0, 8, ctypes.byref(cam)) == 1
    assert rt.LIB.rtCameraLookAt(p, p, p, 40.0, 8, 8, ctypes.byref(cam)) == 1  # eye == target


def test_autotuner_rejects_missing_context(rt):
    assert rt.LIB.rtAutotuneTrace(None, 1, None, 0, None, 1, None, None) == 1
    assert rt.LIB.rtAutotuneRender(None, 1, 1, 8, 1024, None) == 1
