"""The batched form (one persistent trace launch over all grids, one convolution launch, CUDA-graph replay)
against the same grids updated one at a time through ddgi_update.

Each ray runs the same per-warp code in both forms and every convolution keeps its summation order, so the
atlases must be bit-identical (FP32 CUDA-core and tensor-core convolutions alike)."""
import numpy as np
import pytest

from anerend_gb300 import _lib as L
from anerend_gb300 import ddgi, scenes

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SPECS = [((4, 2, 4), 64, 0), ((8, 4, 4), 128, 1), ((4, 4, 8), 256, 0), ((16, 2, 8), 64, 1), ((4, 8, 4), 512, 1),
         ((8, 2, 16), 128, 0)]


def _make(ctx, conv_mode):
    arrays = [scenes.build_scene_tris(n, 50 + i, (-10, 0, -10), (10, 8, 10)) for i, n in enumerate((20000, 7000))]
    scs = [ddgi.Scene(ctx, a) for a in arrays]
    grids = []
    for dims, n, si in SPECS:
        g = ddgi.ProbeGrid(ctx, dims, (1.0, 2.0, 1.0), n, 0.0, 0.97)
        g.set_tuning(warp_probes=max(2, 32 // n), ray_order=1, shadow_mode=1, conv_mode=conv_mode)
        grids.append((g, scs[si]))
    return scs, grids


def _frames(f):
    return [ddgi.FrameParams(camera_pos=(0.5 * i + (f // 2), 1.0, -0.3 * i), rotation=scenes.rotation(i, f))
            for i in range(len(SPECS))]


@pytest.mark.parametrize("conv_mode", [0, 1, 2])
def test_batch_equals_individual_updates(ctx, conv_mode):
    scs_a, solo = _make(ctx, conv_mode)
    scs_b, batched = _make(ctx, conv_mode)
    batch = ddgi.Batch(ctx, batched)
    batch.set_tuning(conv_mode=conv_mode, warp_probes=2, ray_order=1, shadow_mode=1, use_graph=1)
    try:
        for f in range(5):  # the shape repeats from the second update on: capture, then replay
            fr = _frames(f)
            for (g, s), fp in zip(solo, fr):
                g.update(s, fp)
            batch.update(fr)
            ctx.sync()
            for i, ((g1, _), (g2, _)) in enumerate(zip(solo, batched)):
                a1, a2 = g1.download_atlas(), g2.download_atlas()
                assert np.array_equal(a1.view(np.uint32), a2.view(np.uint32)), (f, i)
        st = batch.stats
        assert st.graphLaunches >= 2 and st.eagerLaunches >= 1
        assert st.rays == sum(np.prod(d) * n for d, n, _ in SPECS)
    finally:
        batch.close()
        for g, _ in solo + batched:
            g.close()
        for s in scs_a + scs_b:
            s.close()


def test_batch_round_robin_layers_and_tuning_changes(ctx):
    scs_a, solo = _make(ctx, 0)
    scs_b, batched = _make(ctx, 0)
    batch = ddgi.Batch(ctx, batched)
    try:
        for f in range(4):
            fr = _frames(f)
            for fp in fr:
                fp.layer = -2
            for (g, s), fp in zip(solo, fr):
                g.update(s, fp)
            if f == 2:  # a tuning change drops the captured graph; results must not change
                batch.set_tuning(blocks_per_sm=4, refill_lanes=16)
            batch.update(fr)
            ctx.sync()
            for (g1, _), (g2, _) in zip(solo, batched):
                assert np.array_equal(g1.download_atlas().view(np.uint32), g2.download_atlas().view(np.uint32))
    finally:
        batch.close()
        for g, _ in solo + batched:
            g.close()
        for s in scs_a + scs_b:
            s.close()


def test_batch_rejects_bad_items(ctx):
    scs, items = _make(ctx, 0)
    try:
        with pytest.raises(L.DdgiError):
            ddgi.Batch(ctx, [items[0], items[0]])  # a grid twice
        b = ddgi.Batch(ctx, items)
        with pytest.raises(L.DdgiError):
            b.set_tuning(blocks_per_sm=0)
        b.close()
    finally:
        for g, _ in items:
            g.close()
        for s in scs:
            s.close()
