"""bench.py runs the legs beside its headline (adjoint ratio, batches) in
child processes: a leg's JSON result comes back, and a leg that fails becomes
an {"error": ...} entry instead of ending the benchmark (CPU only)."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_leg_result_comes_back():
    import bench

    assert bench.run_leg("{'a': 1, 'b': [2, 3]}") == {"a": 1, "b": [2, 3]}


def test_failed_leg_is_reported_not_raised():
    import bench

    out = bench.run_leg("1 / 0")
    assert set(out) == {"error"} and "ZeroDivisionError" in out["error"]
