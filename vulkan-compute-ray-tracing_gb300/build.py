"""Build recipe for librtgb.so (the CUDA kernels and the C-ABI runtime).

Every translation unit under csrc/ is compiled in parallel with nvcc for
sm_103a only and linked into ``librtgb.so`` next to this file. Host code is
built with -ffp-contract=off so the fp32 host helpers (camera, light areas,
scene generators) give the same bits on every machine.

Usage: ``python build.py`` (or ``import build; build.build()``).
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librtgb.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build librtgb.so")


def _sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _compile(src: str, nvcc: str) -> str:
    obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
    cmd = [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-I", os.path.join(ROOT, "include"), "-I", CSRC, "-c", src, "-o", obj]
    if src.endswith(".cu"):
        cmd += ["-Xptxas", "-warn-spills"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{res.stdout}\n{res.stderr}")
    if res.stderr.strip():
        sys.stderr.write(res.stderr)
    return obj


STAMP = os.path.join(HERE, "_build", "librtgb.stamp")


def _toolchain_id(nvcc: str) -> str:
    """Machine architecture and nvcc version: a library built elsewhere (a
    copy from another host, or another toolkit) is stale whatever its mtime."""
    try:
        ver = subprocess.run([nvcc, "--version"], capture_output=True, text=True).stdout.strip().splitlines()[-1]
    except Exception:
        ver = "unknown"
    return f"{platform.machine()} {ver} {ARCH}"


def _stale(srcs: list[str], nvcc: str) -> bool:
    if not os.path.exists(LIB) or not os.path.exists(STAMP):
        return True
    with open(STAMP) as f:
        if f.read().strip() != _toolchain_id(nvcc):
            return True
    t = os.path.getmtime(LIB)
    deps = srcs + [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    inc = os.path.join(ROOT, "include", "rtgb")
    deps += [os.path.join(inc, f) for f in os.listdir(inc)]
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, jobs: int | None = None) -> str:
    """Compile librtgb.so if any source changed; returns its path."""
    srcs = _sources()
    nvcc = _nvcc()
    if not force and not _stale(srcs, nvcc):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    with ThreadPoolExecutor(max_workers=jobs or min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, nvcc), srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc, ARCH, "-shared", "-o", tmp] + objs + ["-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    with open(STAMP, "w") as f:
        f.write(_toolchain_id(nvcc) + "\n")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
