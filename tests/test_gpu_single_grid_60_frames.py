"""The single-grid workload end to end against the FP64 oracle: 32x8x32 probes, 256 rays, 262,144 triangles,
all 60 frames, the camera moving +1 in x every 10 frames (IrradianceProbeTranslationPass.cpp:56-186,
irradiance_probe_update.rgen:35-111, probe_conv.comp:21-90).

Two oracle grids follow the device grid:
  - a lockstep one, which starts every frame from the device's atlas, so each frame is compared on its own;
  - a free-running one, which carries its own FP64 atlas through all 60 multi-bounce frames.

Stated tolerances:
  - translation: the device's atlas after each of the five moves equals the oracle's translation of the
    atlas before it, bit for bit;
  - hit triangle id and shadow bit: bit-exact on every ray the oracle marks certain, every frame;
  - lockstep radiance: relative error <= 1e-4 on 99.99 % of the certain rays and <= 1e-2 on all of them
    (the probe lookup's cell index is a floor of the hit position, so a hit within rounding of a cell
    boundary may pick the neighbouring cell's probes);
  - lockstep atlas: relative error <= 1e-4 (floor 1e-3) on every texel of the probes whose rays are all
    certain, and <= 1e-3 on 99.9 % of all texels;
  - free-running atlas at frames 10, 30 and 60: relative error <= 1e-3 (floor 1e-3) on 99.9 % of texels."""
import numpy as np
import pytest

from anerend_gb300 import _lib as L
from anerend_gb300 import ddgi, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def rel_err(got, want, floor):
    return np.abs(got - want) / np.maximum(np.abs(want), floor)


def probe_taint(uncertain: np.ndarray, dims, n) -> np.ndarray:
    """Atlas-shaped mask of the texels of probes with at least one uncertain ray."""
    X, Y, Z = dims
    g = oracle.GridGeom(X, Y, Z, n)
    bw, bh = g.block
    tainted = uncertain.reshape(Y, Z, bh, X, bw).any(axis=(2, 4))  # (Y, Z, X)
    return np.repeat(np.repeat(tainted.reshape(Y * Z, X), 10, axis=0), 10, axis=1)


def test_single_grid_workload_60_frames(ctx):
    w = scenes.SINGLE_GRID
    arrays = scenes.build_scene(w)
    scene = ddgi.Scene(ctx, arrays)
    grid = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis, options=L.DDGI_GRID_RECORD_HITS)
    grid.set_tuning(warp_probes=2, ray_order=1, shadow_mode=1, conv_mode=0, bvh_width=8)  # the bench's tuning
    osc = oracle.OracleScene(arrays, L.SceneDesc)
    lock = oracle.OracleGrid(grid.desc)
    free = oracle.OracleGrid(grid.desc)
    moves = []
    worst = dict(ray_p9999=0.0, ray_max=0.0, clean_max=0.0, atlas_p999=0.0, free_p999=0.0)
    try:
        for f in range(w.frames):
            fp = ddgi.FrameParams(camera_pos=scenes.camera(w, f), rotation=scenes.rotation(w.seed, f))
            fc = fp.to_c()
            before = grid.download_atlas()
            lock.atlas = before.astype(np.float64)  # the lockstep oracle starts the frame from the device's atlas
            dx = int(np.float32(fp.camera_pos[0]) / np.float32(w.step[0])) - lock.last_probe_idx[0]
            if grid.translate(fp.camera_pos):
                after = grid.download_atlas()
                want = oracle.translate(grid.desc, before, int(np.sign(dx)), 0)
                assert np.array_equal(after.view(np.uint32), want.view(np.uint32)), f
                moves.append(f)
            grid.update(scene, fp)  # the translation state already follows the camera: no second shift
            lock.update(osc, fc)
            free.update(osc, fc)
            ctx.sync()

            rad, hits, _ = grid.download_rays(hits=True)
            certain = lock.uncertain == 0
            assert certain.mean() > 0.99, f
            mism = int(np.count_nonzero((hits != lock.hits) & certain))
            assert mism == 0, (f, mism)
            er = rel_err(rad[..., :3].astype(np.float64), lock.ray_rad[..., :3], 1e-3)[certain]
            worst["ray_p9999"] = max(worst["ray_p9999"], float(np.percentile(er, 99.99)))
            worst["ray_max"] = max(worst["ray_max"], float(er.max()))
            assert np.percentile(er, 99.99) <= 1e-4 and er.max() <= 1e-2, (f, float(np.percentile(er, 99.99)),
                                                                           float(er.max()))

            atlas = grid.download_atlas().astype(np.float64)
            ea = rel_err(atlas, lock.atlas, 1e-3)
            clean = ~probe_taint(lock.uncertain != 0, w.dims, w.rays)
            worst["clean_max"] = max(worst["clean_max"], float(ea[clean].max()))
            worst["atlas_p999"] = max(worst["atlas_p999"], float(np.percentile(ea, 99.9)))
            assert ea[clean].max() <= 1e-4, (f, float(ea[clean].max()))
            assert np.percentile(ea, 99.9) <= 1e-3, (f, float(np.percentile(ea, 99.9)))
            if f + 1 in (10, 30, 60):
                ef = rel_err(atlas, free.atlas, 1e-3)
                worst["free_p999"] = max(worst["free_p999"], float(np.percentile(ef, 99.9)))
                assert np.percentile(ef, 99.9) <= 1e-3, (f, np.percentile(ef, [50, 99, 99.9, 100]))
        assert moves == [10, 20, 30, 40, 50], moves
        print("60-frame single-grid parity:", worst)
    finally:
        osc.close()
        grid.close()
        scene.close()
