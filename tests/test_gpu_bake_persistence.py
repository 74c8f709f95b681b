"""Baked-atlas persistence in the reference's layout (ddgi_atlas_export_rgba16f / _import_rgba16f): the
exported buffer is the RGBA16F texel data downloadDDGIAtlas returns (8 bytes per texel, 10 X x 10 Z Y), equal
bit for bit to rounding the grid's atlas to FP16 (round to nearest even); importing it restores that atlas
exactly, and baking resumes from it as from the same values uploaded directly."""
import numpy as np
import pytest

from anerend_gb300 import _lib as L
from anerend_gb300 import ddgi, scenes

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

BAKE = L.DDGI_UBO_DDGI_FLAG | L.DDGI_UBO_DDGI_MULTI_FLAG | L.DDGI_UBO_BAKE_MODE_ON_FLAG


def _bake_frame(w, f):
    return ddgi.FrameParams(camera_pos=(0.0, 0.0, 0.0), rotation=scenes.rotation(w.seed, f), flags=BAKE,
                            bake_tile=(0, 0, 8))


@pytest.mark.parametrize("fmt", [L.DDGI_FORMAT_RGBA32F, L.DDGI_FORMAT_RGBA16F])
def test_export_import_round_trip_and_resume(ctx, fmt):
    w = scenes.CPU_REFERENCE
    scene = ddgi.Scene(ctx, scenes.build_scene(w))
    a = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis, atlas_format=fmt)
    b = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis, atlas_format=fmt)
    c = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis, atlas_format=fmt)
    try:
        for f in range(3):
            a.update(scene, _bake_frame(w, f))
        ctx.sync()
        native = a.download_atlas()
        exported = a.export_atlas_rgba16f()
        assert exported.dtype == np.float16 and exported.shape == (10 * w.dims[2] * w.dims[1], 10 * w.dims[0], 4)
        assert exported.nbytes == 8 * exported.shape[0] * exported.shape[1]
        assert np.array_equal(exported.view(np.uint16), native.astype(np.float16).view(np.uint16))
        assert np.count_nonzero(exported[..., 3]) > 0  # baked weights accumulated in .w
        # import into a fresh grid: the FP16 values, exactly
        b.import_atlas_rgba16f(exported)
        restored = b.download_atlas()
        assert np.array_equal(restored.astype(np.float16).view(np.uint16), exported.view(np.uint16))
        assert np.array_equal(restored.astype(np.float64), exported.astype(np.float64))
        # baking resumes from the imported atlas exactly as from the same values uploaded directly
        c.upload_atlas(exported.astype(native.dtype))
        b.update(scene, _bake_frame(w, 3))
        c.update(scene, _bake_frame(w, 3))
        ctx.sync()
        assert np.array_equal(b.download_atlas().view(np.uint8), c.download_atlas().view(np.uint8))
    finally:
        for g in (a, b, c):
            g.close()
        scene.close()


def test_export_import_reject_wrong_size(ctx):
    g = ddgi.ProbeGrid(ctx, (4, 2, 4), (1.0, 1.0, 1.0), 64, 0.0, 0.97)
    try:
        small = np.zeros((10, 10, 4), np.float16)
        with pytest.raises(L.DdgiError):
            g.import_atlas_rgba16f(small)
        import ctypes as C

        assert g.ctx.lib.ddgi_atlas_export_rgba16f(g.handle, small.ctypes.data, small.nbytes, 0) == L.DDGI_EINVAL
    finally:
        g.close()
