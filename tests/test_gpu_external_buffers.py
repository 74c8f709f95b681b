"""Zero-copy interop at the boundary: caller-owned atlas, translation temp and ray images
(ddgi_grid_bind_external), and ray images in the reference's RGBA16F format (DDGI_GRID_RAYS_RGBA16F, the
R16G16B16A16_SFLOAT ProbeRaysIrrTex / ProbeRaysDirTex of IrradianceProbeRayTracingPass.cpp:42-74, next to the
RGBA16F atlas of IrradianceProbeConvolvePass.cpp:88-93).

Stated tolerances:
  - a grid on caller-owned buffers gives the same atlas and ray images, bit for bit, as the same grid on its own
    buffers (the same kernels on the same inputs), through translations;
  - RGBA16F ray images against the FP64 oracle with the same FP16 store: hit ids bit-exact on certain rays, ray
    radiance within one binary16 rounding (4.9e-4 relative) of the oracle's on certain rays, atlas within 1e-3
    relative on 99.9 % of texel channels after eight multi-bounce frames."""
import ctypes as C

import numpy as np
import pytest

from anerend_gb300 import _lib as L
from anerend_gb300 import ddgi, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

OPTS = L.DDGI_GRID_RAYS_RGBA16F | L.DDGI_GRID_WRITE_DIRS


def _workload():
    return scenes.Workload("ext_8x4x8_n64", (8, 4, 8), (1.0, 1.0, 1.0), -1.5, 64, 3000, (-8, -8, -8), (8, 8, 8),
                           1, 0, -2.0, 10.0, 8, 0.97)


# camera positions of the eight frames: moves in +x, +x, -z, -x and +z (five translations)
CAMERAS = [(0.0, 0.0, 0.0), (0.3, 0.0, 0.0), (1.2, 0.0, 0.0), (1.2, 0.0, 0.0), (2.5, 0.0, 0.0), (2.5, 0.0, -1.1),
           (1.4, 0.0, -1.1), (1.4, 0.0, 0.3)]


def _external(grid):
    """Device buffers of the grid's sizes, owned by torch (the caller)."""
    b = grid.buffers
    bufs = {k: torch.empty(n // 2, dtype=torch.float16, device="cuda")
            for k, n in (("atlas", b.atlasBytes), ("atlas_temp", b.atlasBytes), ("ray_radiance", b.rayBytes),
                         ("ray_direction", b.rayBytes))}
    return bufs


def test_external_rgba16f_buffers_equal_grid_owned(ctx):
    w = _workload()
    scene = ddgi.Scene(ctx, scenes.build_scene(w))
    own = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis,
                         atlas_format=L.DDGI_FORMAT_RGBA16F, options=OPTS)
    ext = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis,
                         atlas_format=L.DDGI_FORMAT_RGBA16F, options=OPTS)
    try:
        bufs = _external(ext)
        # the bound atlas is taken as it stands: start it cleared like the grid's own
        ext.bind_external(atlas=bufs["atlas"].data_ptr(), atlas_temp=bufs["atlas_temp"].data_ptr(),
                          ray_radiance=bufs["ray_radiance"].data_ptr(), ray_direction=bufs["ray_direction"].data_ptr())
        ext.reset()
        b = ext.buffers
        assert b.atlas == bufs["atlas"].data_ptr() and b.rayRadiance == bufs["ray_radiance"].data_ptr()
        assert b.rayFormat == L.DDGI_FORMAT_RGBA16F and b.rayBytes == 8 * b.rayWidth * b.rayHeight
        moves = 0
        for f in range(w.frames):
            fp = ddgi.FrameParams(camera_pos=CAMERAS[f], rotation=scenes.rotation(w.seed, f))
            moved = ext.translate(fp.camera_pos)
            assert own.translate(fp.camera_pos) == moved
            moves += moved
            own.update(scene, fp)
            ext.update(scene, fp)
            ctx.sync()
            # the current atlas and the ray images live in the caller's buffers, and equal the grid-owned ones
            assert ext.buffers.atlas == bufs["atlas"].data_ptr()
            a_own = own.download_atlas()
            a_ext = bufs["atlas"].cpu().numpy().reshape(a_own.shape)
            assert np.array_equal(a_own.view(np.uint16), a_ext.view(np.uint16)), f
            r_own, _, _ = own.download_rays()
            r_ext = bufs["ray_radiance"].cpu().numpy().reshape(r_own.shape)
            assert r_own.dtype == np.float16 and np.array_equal(r_own.view(np.uint16), r_ext.view(np.uint16)), f
            assert not np.array_equal(r_ext, np.zeros_like(r_ext))
        assert moves == 5
        # the direction image holds (dir, 1) in FP16: unit directions
        dirs = bufs["ray_direction"].cpu().numpy().reshape(b.rayHeight, b.rayWidth, 4).astype(np.float64)
        assert np.allclose(np.linalg.norm(dirs[..., :3], axis=-1), 1.0, atol=2e-3) and np.all(dirs[..., 3] == 1.0)
    finally:
        own.close()
        ext.close()
        scene.close()


def test_binding_after_a_translation_keeps_the_current_atlas(ctx):
    """A grid that already swapped its atlas and temp on a move, then binds only a caller temp: its current
    atlas stays current, and later updates still equal an unbound grid's."""
    w = _workload()
    scene = ddgi.Scene(ctx, scenes.build_scene(w))
    a = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis)
    b = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis)
    try:
        for g in (a, b):
            g.update(scene, ddgi.FrameParams(camera_pos=(0.0, 0.0, 0.0), rotation=scenes.rotation(1, 0)))
            assert g.translate((1.5, 0.0, 0.0))
        before = a.download_atlas()
        temp = torch.empty(a.buffers.atlasBytes // 4, dtype=torch.float32, device="cuda")
        a.bind_external(atlas_temp=temp.data_ptr())
        assert np.array_equal(a.download_atlas().view(np.uint32), before.view(np.uint32))
        for f, cam in enumerate(((1.5, 0, 0), (2.5, 0, 0), (2.5, 0, -1.2))):
            fp = ddgi.FrameParams(camera_pos=cam, rotation=scenes.rotation(1, f + 1))
            a.update(scene, fp)
            b.update(scene, fp)
        ctx.sync()
        assert np.array_equal(a.download_atlas().view(np.uint32), b.download_atlas().view(np.uint32))
    finally:
        a.close()
        b.close()
        scene.close()


def test_bind_external_validates(ctx):
    g = ddgi.ProbeGrid(ctx, (4, 2, 4), (1.0, 2.0, 1.0), 64, 0.0, 0.97)
    lib = L.load()
    try:
        b = g.buffers
        buf = torch.empty(b.atlasBytes // 4 + 8, dtype=torch.float32, device="cuda")
        for x in (L.GridExternal(buf.data_ptr(), None, None, None, b.atlasBytes + 16, 0),      # wrong size
                  L.GridExternal(buf.data_ptr() + 4, None, None, None, b.atlasBytes, 0),      # misaligned
                  L.GridExternal(None, None, None, buf.data_ptr(), 0, b.rayBytes),            # no WRITE_DIRS
                  L.GridExternal(buf.data_ptr(), buf.data_ptr(), None, None, b.atlasBytes, 0)):  # same buffer
            assert lib.ddgi_grid_bind_external(g.handle, C.byref(x), None) == L.DDGI_EINVAL
        assert g.buffers.atlas == b.atlas  # nothing was bound
    finally:
        g.close()


def test_rgba16f_ray_images_match_oracle(ctx):
    w = scenes.CPU_REFERENCE
    arrays = scenes.build_scene(w)
    scene = ddgi.Scene(ctx, arrays)
    grid = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis,
                          options=L.DDGI_GRID_RAYS_RGBA16F | L.DDGI_GRID_RECORD_HITS)
    osc = oracle.OracleScene(arrays, L.SceneDesc)
    og = oracle.OracleGrid(grid.desc)
    try:
        for f in range(w.frames):
            fp = ddgi.FrameParams(camera_pos=scenes.camera(w, f), rotation=scenes.rotation(w.seed, f))
            og.atlas = grid.download_atlas().astype(np.float64)  # lockstep: the same previous atlas
            grid.update(scene, fp)
            og.update(osc, fp.to_c())
            ctx.sync()
            rad, hits, _ = grid.download_rays(hits=True)
            assert rad.dtype == np.float16
            certain = og.uncertain == 0
            assert np.array_equal(hits[certain], og.hits[certain])
            err = np.abs(rad[..., :3].astype(np.float64) - og.ray_rad[..., :3]) / np.maximum(np.abs(og.ray_rad[..., :3]), 1e-3)
            assert np.percentile(err[certain], 99.9) <= 4.9e-4, np.percentile(err[certain], [99, 99.9, 100])
        atlas = grid.download_atlas().astype(np.float64)
        err = np.abs(atlas - og.atlas) / np.maximum(np.abs(og.atlas), 1e-3)
        assert np.percentile(err, 99.9) <= 1e-3, np.percentile(err, [50, 99, 99.9, 100])
    finally:
        osc.close()
        grid.close()
        scene.close()
