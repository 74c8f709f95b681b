"""The specular GI mirror pass (ddgi_mirror_reflections: SpecularGIRTPass.cpp:111-128, mirror_reflections.rgen,
.rchit, .rmiss) against the FP64 oracle.

Tolerances, on every point whose reflected ray and shadow ray the oracle marks certain: sky pixels exactly 0;
misses the linear sky (relative 1e-6) with distance 1e6; hits radiance relative error <= 1e-4 per channel
(floor 1e-3, the probe update's bar) and hit distance within 1e-5 relative + 2e-5 absolute (the FP32 hit
position, interpolated from vertices of magnitude ~10, carries a few 1e-6 of rounding per coordinate)."""
import math

import numpy as np
import pytest

from anerend_gb300 import _lib as L
from anerend_gb300 import ddgi, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _rel(got, want, floor):
    return np.abs(got - want) / np.maximum(np.abs(want), floor)


def _run(ctx, grid, scene, frame, pts):
    dp = torch.from_numpy(pts.view(np.uint8).copy()).cuda()
    out = torch.empty((len(pts), 4), dtype=torch.float32, device="cuda")
    grid.mirror_reflections(scene, frame, dp.data_ptr(), len(pts), out.data_ptr(),
                            torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _points_on_triangles(arrays, n, seed):
    v = arrays.vertices["d0"][:, :3].astype(np.float64)
    tri = arrays.indices.reshape(-1, 3)
    u = [scenes.uniform(seed, 900 + k, n) for k in range(3)]
    k = (u[0] * len(tri)).astype(np.int64) % len(tri)
    a, b = u[1].copy(), u[2].copy()
    flip = a + b > 1
    a[flip], b[flip] = 1 - a[flip], 1 - b[flip]
    p = v[tri[k, 0]] * (1 - a - b)[:, None] + v[tri[k, 1]] * a[:, None] + v[tri[k, 2]] * b[:, None]
    nrm = np.cross(v[tri[k, 1]] - v[tri[k, 0]], v[tri[k, 2]] - v[tri[k, 0]])
    pts = np.zeros(n, L.MIRROR_POINT)
    pts["position"] = p.astype(np.float32)
    pts["normal"] = nrm.astype(np.float32)
    pts["sky"][::23] = 1.0
    return pts


@pytest.mark.parametrize("options", [0, L.DDGI_GRID_EDGE_CLAMP])
@pytest.mark.parametrize("flags", [L.DDGI_UBO_DDGI_FLAG, 0])
@pytest.mark.parametrize("shadow_mode", [1, 0])  # shadow rays in the light-space BVH, or the scene BVH
def test_mirror_matches_oracle(ctx, options, flags, shadow_mode):
    w = scenes.CPU_REFERENCE
    arrays = scenes.build_scene(w)
    scene = ddgi.Scene(ctx, arrays)
    grid = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis, options=options)
    grid.set_tuning(shadow_mode=shadow_mode)
    osc = oracle.OracleScene(arrays, L.SceneDesc)
    try:
        b = grid.buffers
        atlas = (scenes.uniform(3, 950, b.atlasHeight * b.atlasWidth * 4) * 2.0).reshape(b.atlasHeight, b.atlasWidth, 4)
        atlas = atlas.astype(np.float32)
        grid.upload_atlas(atlas)
        frame = ddgi.FrameParams(camera_pos=(0.3, 0.8, -0.4), flags=flags)
        pts = _points_on_triangles(arrays, 6000, 5)
        got = _run(ctx, grid, scene, frame, pts)
        want, unc = oracle.mirror_reflections(osc, grid.desc, frame.to_c(), atlas.astype(np.float64), pts)
        sky = pts["sky"] != 0
        certain = (unc == 0) & ~sky
        assert np.array_equal(got[sky], np.zeros((sky.sum(), 4), np.float32))
        assert certain.sum() > 0.97 * (~sky).sum()
        miss = certain & (want[:, 3] == 1e6)
        hit = certain & (want[:, 3] < 1e6)
        assert hit.mean() > 0.5 and miss.sum() > 0  # the reference scene is dense: most reflections hit
        assert np.array_equal(got[miss, 3], np.full(miss.sum(), 1e6, np.float32))
        assert np.max(_rel(got[miss, :3].astype(np.float64), want[miss, :3], 1e-6)) <= 1e-6
        assert np.all(np.abs(got[hit, 3] - want[hit, 3]) <= 1e-5 * want[hit, 3] + 2e-5)
        err = _rel(got[hit, :3].astype(np.float64), want[hit, :3], 1e-3)
        assert np.max(err) <= 1e-4, np.percentile(err, [50, 99, 100])
    finally:
        osc.close()
        grid.close()
        scene.close()


def test_mirror_known_answer(ctx):
    """A floor point reflecting onto an emissive wall whose hit an occluder shadows: radiance = the emission
    (no DDGI), distance 3 sqrt2; a point reflecting into the sky; a sky pixel."""
    floor = scenes.floor_quad(0.0, 4.0)
    wall = np.array([[[-2, 0, 3], [2, 0, 3], [2, 6, 3]], [[-2, 0, 3], [2, 6, 3], [-2, 6, 3]]], np.float64)
    occ = np.array([[[-1, 5, 2.5], [1, 5, 2.5], [1, 5, 3.5]], [[-1, 5, 2.5], [1, 5, 3.5], [-1, 5, 3.5]]], np.float64)
    mats = scenes.random_materials(0, 3)
    mats["baseColFac"] = [[0.3, 0.3, 0.3, 1.0], [0.5, 0.6, 0.7, 1.0], [0.2, 0.2, 0.2, 1.0]]
    mats["emissive"] = [[0, 0, 0, 0], [1.0, 2.0, 3.0, 1.0], [0, 0, 0, 0]]
    arrays = scenes.assemble(np.concatenate([floor, wall, occ]), np.array([0, 0, 1, 1, 2, 2]), np.arange(3), mats)
    pts = np.zeros(3, L.MIRROR_POINT)
    pts["position"] = [[0.5, 0.0, 0.0], [0.5, 1.0, -6.0], [1.0, 1.0, 1.0]]
    pts["normal"] = [[0.0, 1.0, 0.0], [0.0, 2.0, 0.0], [0.0, 1.0, 0.0]]
    pts["sky"] = [0.0, 0.0, 1.0]
    scene = ddgi.Scene(ctx, arrays)
    grid = ddgi.ProbeGrid(ctx, (4, 2, 4), (1.0, 1.0, 1.0), 64, 0.0, 0.97)
    try:
        frame = ddgi.FrameParams(camera_pos=(0.5, 2.0, -2.0), light_dir=(0.0, -1.0, 0.0), flags=0)
        got = _run(ctx, grid, scene, frame, pts)
        assert np.allclose(got[0], [1.0, 2.0, 3.0, 3.0 * math.sqrt(2.0)], rtol=1e-6)
        c = np.array([0.4, 0.5, 0.7])
        sky = np.where(c < 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4)
        assert np.allclose(got[1], [*sky, 1e6], rtol=1e-6)
        assert np.array_equal(got[2], np.zeros(4, np.float32))
    finally:
        grid.close()
        scene.close()


def test_mirror_argument_errors(ctx):
    w = scenes.CPU_REFERENCE
    scene = ddgi.Scene(ctx, scenes.build_scene(w))
    grid = ddgi.ProbeGrid(ctx, (4, 2, 4), (1.0, 1.0, 1.0), 64, 0.0, 0.97)
    try:
        with pytest.raises(L.DdgiError):
            grid.mirror_reflections(scene, ddgi.FrameParams(), 0, 4, 0)  # NULL buffers
        buf = torch.empty(64, dtype=torch.float32, device="cuda")
        with pytest.raises(L.DdgiError):
            grid.mirror_reflections(scene, ddgi.FrameParams(), buf.data_ptr() + 4, 1, buf.data_ptr())  # misaligned
        grid.mirror_reflections(scene, ddgi.FrameParams(), 0, 0, 0)  # nothing to do
    finally:
        grid.close()
        scene.close()
