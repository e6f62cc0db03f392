"""Host-side pieces of bench.py that its GPU run relies on: the per-kernel
ncu figures parsed from the committed summary, and the algorithmic bytes
per ray, recounted here by the oracle."""
import importlib.util
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_kernel_profiles_parsed_from_summary():
    b = load_bench()
    prof = b.kernel_profiles()
    for name in ("k_trace_packets", "k_trace_wide"):
        p = prof[name]
        assert p["duration_ms"] > 0 and p["inst_issued"] > 0
        # Per batch cast (4,194,304 rays): DRAM bytes well below the algorithmic bytes.
        per_ray = p["dram_bytes"] / b.RAYS_PER_BATCH
        assert 10 < per_ray < min(b.ALG_BYTES_COHERENT, b.ALG_BYTES_INCOHERENT)


def test_algorithmic_bytes_recounted_by_the_oracle(orc):
    """48 B per node or triangle record of the culled near-first traversal of
    the reference tree (the oracle's counts on one ray in 61 of each batch —
    a stride prime to the image width, so every column is sampled), plus a
    32 B ray and a 16 B hit, within 1% of the bench's constants (counted on
    every ray)."""
    b = load_bench()
    tris, coherent, incoherent = orc.closest_hit_workload()
    nodes, _ = orc.build_bvh(tris, 1)
    for rays, quoted in ((coherent, b.ALG_BYTES_COHERENT), (incoherent, b.ALG_BYTES_INCOHERENT)):
        _, st = orc.trace(tris, nodes, rays[::61], slack=0.0, stats=True)
        counted = 48.0 * (st[:, 0].mean() + st[:, 1].mean()) + 48.0
        assert abs(counted - quoted) <= 0.01 * quoted, (counted, quoted)
