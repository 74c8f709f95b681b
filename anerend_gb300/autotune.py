"""Autotuner for the launch shape of a batch (DdgiBatchTuning) and of a single grid (DdgiTuning).

The knobs change speed only, never results: every combination traces the same closest hits and shadow
bits, so the search is free to pick any of them. It is a coordinate descent from the defaults: for each
knob in turn, every candidate value is timed with the others fixed, and the fastest is kept; two sweeps
over the knobs are usually enough because their interactions are weak. The timing of one candidate is the
median of `reps` timed updates after warm-up updates (the first of which may capture a CUDA graph), with
the device synchronized before and after each timed update.

Results are cached per (device name, workload signature) in a JSON file (default
$XDG_CACHE_HOME/anerend_gb300/autotune.json, else ~/.cache/...); the signature is supplied by the caller
(for a batch: its grids' dims / rays and scene sizes), so a different workload is tuned again.

The convolution mode is not searched: it changes precision (FP32 vs FP16/BF16 tensor cores), so it stays
the caller's choice.
"""
from __future__ import annotations

import json
import os
import statistics
import time
from pathlib import Path
from typing import Callable, Dict, Iterable, List, Optional, Sequence

BATCH_SPACE: Dict[str, Sequence[int]] = {
    "bvh_width": (8, 2),
    "refill_lanes": (4, 8, 16),
    "blocks_per_sm": (8, 6, 4),
    "warp_probes": (1, 2, 4, 8),
    "ray_order": (1, 0),
    "shadow_mode": (1, 0),
}
GRID_SPACE: Dict[str, Sequence[int]] = {
    "bvh_width": (8, 2),
    "refill_lanes": (4, 8, 16),
    "warp_probes": (1, 2, 4, 8),
    "ray_order": (1, 0),
    "shadow_mode": (1, 0),
}


def cache_path() -> Path:
    base = os.environ.get("XDG_CACHE_HOME") or str(Path.home() / ".cache")
    return Path(base) / "anerend_gb300" / "autotune.json"


def _load(path: Path) -> dict:
    try:
        return json.loads(path.read_text())
    except (OSError, ValueError):
        return {}


def _store(path: Path, key: str, entry: dict) -> None:
    try:
        path.parent.mkdir(parents=True, exist_ok=True)
        data = _load(path)
        data[key] = entry
        tmp = path.with_suffix(".tmp")
        tmp.write_text(json.dumps(data, indent=1, sort_keys=True))
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home only loses the cache


def _device_name() -> str:
    try:
        import torch

        if torch.cuda.is_available():
            return torch.cuda.get_device_name(0)
    except Exception:  # noqa: BLE001 - the name is only a cache key
        pass
    return "unknown-device"


def coordinate_descent(measure: Callable[[dict], float], start: dict, space: Dict[str, Sequence[int]],
                       sweeps: int = 2, log: Optional[Callable[[str], None]] = None) -> tuple[dict, float, List[dict]]:
    """Minimises measure(config) one knob at a time. Returns (best config, its time, every trial)."""
    best = dict(start)
    best_t = measure(best)
    trials = [dict(best, ms=best_t)]
    seen = {tuple(sorted(best.items())): best_t}
    for _ in range(sweeps):
        improved = False
        for knob, values in space.items():
            for v in values:
                cand = dict(best, **{knob: v})
                key = tuple(sorted(cand.items()))
                if key in seen:
                    continue
                try:
                    t = measure(cand)
                except Exception as e:  # noqa: BLE001 - an invalid combination is skipped, not fatal
                    if log:
                        log(f"skip {cand}: {e}")
                    seen[key] = float("inf")
                    continue
                seen[key] = t
                trials.append(dict(cand, ms=t))
                if log:
                    log(f"{cand} -> {t:.3f} ms")
                if t < best_t:
                    best, best_t, improved = cand, t, True
        if not improved:
            break
    return best, best_t, trials


def _timer(ctx, stream: int):
    """Returns time_one(fn) -> ms: CUDA events on the stream when torch is present, else wall clock around
    a device synchronization."""
    try:
        import torch

        if torch.cuda.is_available():
            ts = torch.cuda.ExternalStream(stream) if stream else torch.cuda.current_stream()

            def time_one(fn):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                torch.cuda.synchronize()
                e0.record(ts)
                fn()
                e1.record(ts)
                torch.cuda.synchronize()
                return e0.elapsed_time(e1)

            return time_one
    except Exception:  # noqa: BLE001 - fall back to host timing
        pass

    def time_one(fn):
        ctx.sync(stream)
        t0 = time.perf_counter()
        fn()
        ctx.sync(stream)
        return (time.perf_counter() - t0) * 1e3

    return time_one


def tune_batch(batch, frames: Callable[[int], list], signature: str, stream: int = 0, reps: int = 3,
               warmup: int = 2, space: Optional[Dict[str, Sequence[int]]] = None, use_cache: bool = True,
               path: Optional[Path] = None, log: Optional[Callable[[str], None]] = None) -> dict:
    """Tunes `batch` (anerend_gb300.ddgi.Batch) on frames(k) -> per-item FrameParams, applies the best
    tuning and returns {"tuning": {...}, "ms": best, "trials": [...], "cached": bool}."""
    space = BATCH_SPACE if space is None else space
    path = cache_path() if path is None else path
    key = f"batch|{_device_name()}|{signature}|conv{int(batch.tuning.convMode)}"
    if use_cache:
        hit = _load(path).get(key)
        if hit:
            batch.set_tuning(**hit["tuning"])
            return dict(hit, cached=True)
    time_one = _timer(batch.ctx, stream)
    frame_no = [0]

    def measure(cfg: dict) -> float:
        batch.set_tuning(**cfg)
        for _ in range(warmup):
            batch.update(frames(frame_no[0]), stream)
            frame_no[0] += 1
        ts = []
        for _ in range(reps):
            fr = frames(frame_no[0])
            frame_no[0] += 1
            ts.append(time_one(lambda: batch.update(fr, stream)))
        return statistics.median(ts)

    t = batch.tuning
    start = {"bvh_width": t.bvhWidth or 8, "refill_lanes": t.refillLanes, "blocks_per_sm": t.blocksPerSm,
             "warp_probes": t.warpProbes, "ray_order": t.rayOrder, "shadow_mode": t.shadowMode}
    best, best_t, trials = coordinate_descent(measure, start, space, log=log)
    batch.set_tuning(**best)
    entry = {"tuning": best, "ms": best_t, "trials": trials}
    if use_cache:
        _store(path, key, entry)
    return dict(entry, cached=False)


def tune_grid(grid, scene, frames: Callable[[int], object], signature: str, stream: int = 0, reps: int = 3,
              warmup: int = 2, space: Optional[Dict[str, Sequence[int]]] = None, use_cache: bool = True,
              path: Optional[Path] = None, log: Optional[Callable[[str], None]] = None) -> dict:
    """Tunes one grid's DdgiTuning on grid.update(scene, frames(k)); same return value as tune_batch."""
    space = GRID_SPACE if space is None else space
    path = cache_path() if path is None else path
    key = f"grid|{_device_name()}|{signature}|conv{int(grid.tuning.convMode)}"
    if use_cache:
        hit = _load(path).get(key)
        if hit:
            grid.set_tuning(**hit["tuning"])
            return dict(hit, cached=True)
    time_one = _timer(grid.ctx, stream)
    frame_no = [0]

    def measure(cfg: dict) -> float:
        grid.set_tuning(**cfg)
        for _ in range(warmup):
            grid.update(scene, frames(frame_no[0]), stream)
            frame_no[0] += 1
        ts = []
        for _ in range(reps):
            fr = frames(frame_no[0])
            frame_no[0] += 1
            ts.append(time_one(lambda: grid.update(scene, fr, stream)))
        return statistics.median(ts)

    t = grid.tuning
    start = {"bvh_width": t.bvhWidth or 8, "refill_lanes": t.refillLanes or 8, "warp_probes": t.warpProbes,
             "ray_order": t.rayOrder, "shadow_mode": t.shadowMode}
    best, best_t, trials = coordinate_descent(measure, start, space, log=log)
    grid.set_tuning(**best)
    entry = {"tuning": best, "ms": best_t, "trials": trials}
    if use_cache:
        _store(path, key, entry)
    return dict(entry, cached=False)


def batch_signature(specs: Iterable, scene_tris: Iterable[int]) -> str:
    """Workload key of a batch: each grid's dims and rays, and the scenes' triangle counts."""
    g = ";".join(f"{tuple(s.dims)}x{s.rays}" for s in specs)
    return f"{g}|tris={','.join(str(int(t)) for t in scene_tris)}"
