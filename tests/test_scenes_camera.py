"""The single-grid workload's camera path: +1 in x every 10 frames over its 60 frames, then back and forth."""
from anerend_gb300 import scenes


def test_first_run_is_the_workload_definition():
    w = scenes.SINGLE_GRID
    assert [scenes.camera(w, f)[0] for f in range(w.frames)] == [float(f // 10) for f in range(w.frames)]


def test_long_runs_stay_bounded_with_unit_moves():
    w = scenes.SINGLE_GRID
    xs = [scenes.camera(w, f)[0] for f in range(2000)]
    assert min(xs) == 0.0 and max(xs) == 5.0
    assert all(abs(b - a) <= 1.0 for a, b in zip(xs, xs[1:]))
    # the path repeats every 120 frames
    assert xs[:120] == xs[120:240]
    assert scenes.camera(scenes.CPU_REFERENCE, 1234) == (0.0, 0.0, 0.0)
