"""CPU tests of the autotuner's search and cache (the GPU timing path runs in bench.py's batched form)."""
import json

from anerend_gb300 import autotune


def test_coordinate_descent_finds_separable_optimum():
    space = {"a": (1, 2, 4, 8), "b": (0, 1), "c": (4, 8, 16)}
    target = {"a": 4, "b": 1, "c": 8}
    calls = []

    def measure(cfg):
        calls.append(dict(cfg))
        return sum((cfg[k] - target[k]) ** 2 for k in target) + 1.0

    best, t, trials = autotune.coordinate_descent(measure, {"a": 1, "b": 0, "c": 16}, space)
    assert best == target and t == 1.0
    # every configuration is timed at most once
    keys = [tuple(sorted(c.items())) for c in calls]
    assert len(keys) == len(set(keys))
    assert len(trials) == len(calls)


def test_invalid_candidates_are_skipped():
    def measure(cfg):
        if cfg["a"] == 2:
            raise ValueError("rejected by the library")
        return float(cfg["a"])

    best, t, _ = autotune.coordinate_descent(measure, {"a": 8}, {"a": (8, 2, 4)})
    assert best == {"a": 4} and t == 4.0


def test_cache_round_trip(tmp_path):
    p = tmp_path / "cache.json"
    autotune._store(p, "k1", {"tuning": {"a": 1}, "ms": 2.0})
    autotune._store(p, "k2", {"tuning": {"a": 2}, "ms": 3.0})
    data = json.loads(p.read_text())
    assert data["k1"]["tuning"] == {"a": 1} and data["k2"]["ms"] == 3.0
    assert autotune._load(tmp_path / "missing.json") == {}


def test_batch_signature_distinguishes_workloads():
    class S:
        def __init__(self, dims, rays):
            self.dims, self.rays = dims, rays

    a = autotune.batch_signature([S((4, 4, 4), 64)], [1000])
    b = autotune.batch_signature([S((4, 4, 4), 128)], [1000])
    c = autotune.batch_signature([S((4, 4, 4), 64)], [2000])
    assert len({a, b, c}) == 3
