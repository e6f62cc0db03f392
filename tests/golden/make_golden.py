"""Generates the golden fixtures in this directory.

Run once where the reference checkout is present (it needs oracle/_ref, the
reference's own Bvh.h compiled by oracle/Makefile):

    python tests/golden/make_golden.py

Fixtures:
  bvh.json        node-array digests of the REFERENCE's Bvh::createBvh on the
                  synthetic scenes (and the first/last nodes in clear), which pin
                  the oracle's restatement and the GPU builder on machines
                  without the reference checkout;
  scenes.json     digests of the generated scene and ray bytes (cross-machine
                  determinism of the generators);
  rand.json       the first values of glibc rand() for a few seeds;
  trace_*.npy     oracle closest hits for small ray sets;
  render_*.npy    oracle images of small renders;
  ref_shader_*.npy  rgba8 images made by the REFERENCE's own compute shader
                  (ray-trace-compute.comp compiled on the host through
                  oracle/glsl2cpp.py, oracle/_ref/libref_shader.so), driven
                  frame by frame as src/main.cpp drives it (the _simple_ one
                  from ray-trace-compute-simple.comp): the pins for the
                  oracle's shader restatement and the GPU kernels' compat
                  mode on machines without the reference checkout.

`--ref-shader-only` regenerates just the ref_shader_* fixtures.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "vulkan-compute-ray-tracing_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import rtgb  # noqa: E402
import oracle  # noqa: E402

NODE_COLS = [0, 1, 2, 4, 5, 6, 7, 8, 9]


def node_digest(nodes: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(nodes.view(np.uint32)[:, NODE_COLS]).tobytes()).hexdigest()


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


# Scenes used by the BVH fixtures: name -> callable returning triangles.
def bvh_scenes(big: bool):
    s = {
        "cornell_1410": lambda: rtgb.gen_cornell(11, 1410)[0],
        "cornell_12000": lambda: rtgb.gen_cornell(1, 12000)[0],
        "icosphere_l5": lambda: rtgb.gen_icosphere(2, 5),
        "icosphere_l6": lambda: rtgb.gen_icosphere(3, 6),
        "tiny_3": lambda: rtgb.gen_cornell(5, 0)[0][:3],
        "tiny_17": lambda: rtgb.gen_cornell(5, 5)[0],
    }
    if big:
        s["icosphere_l8"] = lambda: rtgb.gen_icosphere(1, 8)
    return s


def node_rows(nodes: np.ndarray, rows):
    return {int(r): nodes.view(np.uint32)[r, NODE_COLS].tolist() for r in rows}


# Reference-shader fixtures: name -> (scene builder, camPos, W, H, frames,
# lights bound, shader). camPos goes through the shader's own camera (vfov
# 30, origin = camPos.zxy * (-1, 1, 1), looking down -z). Shader "full" is
# ray-trace-compute.comp (NUM_BOUNCES 2), "simple" is
# ray-trace-compute-simple.comp (NUM_BOUNCES 4, hemisphere scattering).
def ref_shader_cases():
    def cornell():
        t, m, _ = rtgb.gen_cornell(3, 3000, 0)
        m = m.copy()
        m[:, 1] = 0.0  # metal fuzz is not part of the reference's material
        return t, m, np.zeros((1, 8), np.float32)
    return {
        "ref_shader_cornell_96x64": (cornell, (0.0, 4.5, 0.0), 96, 64, 3, "one", "full"),
        "ref_shader_cornell_96x64_lights": (cornell, (0.0, 4.5, 0.0), 96, 64, 2, "all", "full"),
        "ref_shader_simple_cornell_96x64": (cornell, (0.0, 4.5, 0.0), 96, 64, 4, "one", "simple"),
    }


def ref_shader_fixtures():
    if not oracle.ref_shader_available():
        raise SystemExit("oracle/_ref/libref_shader.so is missing: run `make -C oracle` with the reference present")
    meta = {}
    cases = dict(ref_shader_cases())
    if oracle.ref_scene_available():
        cases["ref_shader_doge_128x96"] = (lambda: rtgb.load_reference_scene(oracle.REF_SCENE_DIR),
                                           rtgb.REFERENCE_CAMERA_POS, 128, 96, 4, "one", "full")
    for name, (build, cam_pos, W, H, frames, lights_mode, shader) in cases.items():
        t, m, sph = build()
        nodes = oracle.ref_build_bvh(t, 1)
        lights = oracle.lights_from_materials(t, m)
        img = oracle.ref_shader_render(t, m, nodes, lights, sph, cam_pos, W, H, frames,
                                       lights_len=1 if lights_mode == "one" else len(lights),
                                       simple=shader == "simple")
        q = np.rint(img * 255.0).astype(np.uint8)
        np.save(os.path.join(HERE, name + ".npy"), q)
        meta[name] = {"cam_pos": list(map(float, cam_pos)), "width": W, "height": H, "frames": frames,
                      "lights": lights_mode, "max_bounces": 4 if shader == "simple" else 2, "shader": shader}
        print(name, W, H, frames, float(img[..., :3].mean()))
    with open(os.path.join(HERE, "ref_shader.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)


def main():
    if "--ref-shader-only" in sys.argv:
        ref_shader_fixtures()
        return
    big = "--no-big" not in sys.argv
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref/libref_bvh.so is missing: run `make -C oracle` with the reference present")
    out = {}
    for name, fn in bvh_scenes(big).items():
        tris = fn()
        ref = oracle.ref_build_bvh(tris, 1)
        n = len(ref)
        out[name] = {"triangles": int(len(tris)), "nodes": int(n), "digest": node_digest(ref),
                     "rows": node_rows(ref, sorted({0, 1, 2, n // 2, n - 2, n - 1}))}
        print(name, len(tris), out[name]["digest"][:16])
    # A second seed on one scene pins the rand() plumbing.
    tris = rtgb.gen_cornell(1, 12000)[0]
    ref = oracle.ref_build_bvh(tris, 7)
    out["cornell_12000_seed7"] = {"triangles": int(len(tris)), "nodes": int(len(ref)), "digest": node_digest(ref),
                                  "seed": 7}
    with open(os.path.join(HERE, "bvh.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)

    scenes = {}
    t, m, s = rtgb.gen_cornell(1, 12000, 16, 0.2, 1.0)
    scenes["cornell_12000_16"] = {"tris": digest(t), "mats": digest(m), "spheres": digest(s)}
    scenes["icosphere_l8"] = {"tris": digest(rtgb.gen_icosphere(1, 8))}
    cam = rtgb.camera_look_at([0, 0, -3], [0, 0, 0], [0, 1, 0], 40.0, 2048, 2048)
    scenes["camera_rays_2048"] = {"rays": digest(rtgb.gen_camera_rays(cam, 2048, 2048)), "camera": cam.as_array().tolist()}
    scenes["random_rays_4m"] = {"rays": digest(rtgb.gen_random_rays(3, 4194304))}
    gt, gm = rtgb.gen_grid(9, 2, 2, 3, 0.35, 0.05, 1000, 1.0)
    scenes["grid_small"] = {"tris": digest(gt), "mats": digest(gm)}
    scenes["uniform"] = [rtgb.LIB.rtgbUniform(s_, i) for s_, i in ((1, 0), (1, 1), (123456789, 987654321))]
    with open(os.path.join(HERE, "scenes.json"), "w") as f:
        json.dump(scenes, f, indent=1, sort_keys=True)

    rand = {str(sd): oracle.glibc_rand(sd, 64).tolist() for sd in (0, 1, 7, 2147483647, 4294967295)}
    with open(os.path.join(HERE, "rand.json"), "w") as f:
        json.dump(rand, f)

    # Closest-hit fixtures on a small icosphere (coherent + random rays).
    tris = rtgb.gen_icosphere(2, 5)
    nodes, _ = oracle.build_bvh(tris, 1)
    cam = rtgb.camera_look_at([0, 0, -3], [0, 0, 0], [0, 1, 0], 40.0, 64, 64)
    rays = np.concatenate([rtgb.gen_camera_rays(cam, 64, 64), rtgb.gen_random_rays(5, 4096)])
    hits = oracle.trace(tris, nodes, rays)
    np.save(os.path.join(HERE, "trace_icosphere_l5.npy"), hits)
    lit = oracle.trace(tris, nodes, rays, mode=1, stack_size=16)
    np.save(os.path.join(HERE, "trace_icosphere_l5_stack16.npy"), lit)

    # Render fixtures: the config-0 scene at 64x64.
    t, m, s = rtgb.gen_cornell(1, 12000, 4, 0.2, 1.0)
    nodes, _ = oracle.build_bvh(t, 1)
    lights = oracle.lights_from_materials(t, m)
    cam = rtgb.camera_look_at([0, 0, -14], [0, 0, 0], [0, 1, 0], 40.0, 64, 64).as_array()
    img, _ = oracle.render(t, m, nodes, lights, s, cam, 64, 64, spp=1, max_bounces=8)
    np.save(os.path.join(HERE, "render_cornell_64.npy"), img)
    img, _ = oracle.render(t, m, nodes, lights, s, cam, 64, 64, spp=4, max_bounces=8,
                           flags=rtgb.COMPAT_STACK16 | rtgb.COMPAT_LEN1 | rtgb.COMPAT_UNORM8)
    np.save(os.path.join(HERE, "render_cornell_64_compat.npy"), img)
    ref_shader_fixtures()
    print("golden fixtures written")


if __name__ == "__main__":
    main()
