"""Host-side pieces of bench.py that its GPU run relies on: the per-launch
DRAM traffic parsed from the committed ncu summary, and the algorithmic
bytes per ray quoted from the oracle's counts."""
import importlib.util
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_traffic_parsed_from_profile():
    b = load_bench()
    t = b.traffic_from_profile()
    assert t is not None and t > 0
    # Per batch cast (4,194,304 rays): well below the algorithmic bytes.
    per_ray = t / b.RAYS_PER_BATCH
    assert 10 < per_ray < min(b.ALG_BYTES_COHERENT, b.ALG_BYTES_INCOHERENT)


def test_algorithmic_bytes_are_the_oracle_counts():
    b = load_bench()
    # 48 B per node or triangle record of the culled near-first traversal
    # of the reference tree, plus a 32 B ray and a 16 B hit.
    assert abs(b.ALG_BYTES_COHERENT - (48.0 * (531.24 + 61.47) + 48.0)) < 1e-6
    assert abs(b.ALG_BYTES_INCOHERENT - (48.0 * (369.86 + 41.28) + 48.0)) < 1e-6
