"""Asynchronous atlas readback (ddgi_atlas_download_async / ddgi_atlas_download_wait): each readback holds
the atlas as it stood at its place in the stream, although the next update runs while it is copied and
changes the atlas in place; the bytes equal those of the blocking ddgi_atlas_download."""
import numpy as np
import pytest

from anerend_gb300 import _lib as L
from anerend_gb300 import ddgi, scenes

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _frame(w, f):
    return ddgi.FrameParams(camera_pos=scenes.camera(w, f), rotation=scenes.rotation(w.seed, f))


@pytest.mark.parametrize("fmt", [L.DDGI_FORMAT_RGBA32F, L.DDGI_FORMAT_RGBA16F])
def test_async_readback_is_the_stream_ordered_atlas(ctx, fmt):
    w = scenes.CPU_REFERENCE
    scene = ddgi.Scene(ctx, scenes.build_scene(w))
    g = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis, atlas_format=fmt)
    try:
        nb = g.buffers.atlasBytes
        bufs = [torch.zeros(nb, dtype=torch.uint8).pin_memory() for _ in range(3)]
        for f in range(3):
            g.update(scene, _frame(w, f))
        ref = [g.download_atlas().view(np.uint8).reshape(-1).copy()]
        g.download_atlas_async(bufs[0])
        for f in (3, 4):  # two more readbacks in flight behind updates, into their own buffers
            g.update(scene, _frame(w, f))
            g.download_atlas_async(bufs[f - 2])
        g.wait_download()
        got = [b.numpy() for b in bufs]
        ctx.sync()
        final = g.download_atlas().view(np.uint8).reshape(-1)
        assert np.array_equal(got[0], ref[0])
        assert np.array_equal(got[2], final)
        assert not np.array_equal(got[0], got[2])  # the updates in between changed the atlas
        # the middle readback is the atlas after frame 3: redo frames 0-3 on a fresh grid
        h = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis, atlas_format=fmt)
        try:
            for f in range(4):
                h.update(scene, _frame(w, f))
            assert np.array_equal(got[1], h.download_atlas().view(np.uint8).reshape(-1))
        finally:
            h.close()
        g.wait_download()  # nothing pending: returns at once
    finally:
        g.close()
        scene.close()


def test_async_readback_argument_errors_and_close_while_pending(ctx):
    g = ddgi.ProbeGrid(ctx, (4, 2, 4), (1.0, 1.0, 1.0), 64, 0.0, 0.97)
    try:
        small = torch.zeros(16, dtype=torch.uint8).pin_memory()
        with pytest.raises(L.DdgiError):
            g.download_atlas_async(small)
        assert g.ctx.lib.ddgi_atlas_download_async(g.handle, 0, g.buffers.atlasBytes, 0) == L.DDGI_EINVAL
        assert g.ctx.lib.ddgi_atlas_download_wait(None) == L.DDGI_EINVAL
        buf = torch.zeros(g.buffers.atlasBytes, dtype=torch.uint8).pin_memory()
        g.download_atlas_async(buf)
    finally:
        g.close()  # waits for the pending readback before freeing its staging buffer
