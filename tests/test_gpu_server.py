"""Serving loop: continuous batching with overlapping launches. Each request's atlas must be the same when it
is served alone and when it is served in a mix with others (bit-identical: every ray and every probe runs the
same code in both cases), admission must respect the memory budget, and oversize requests are refused."""
import numpy as np
import pytest

from anerend_gb300 import _lib as L
from anerend_gb300 import ddgi, scenes

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

REQS = [((4, 2, 4), 64, 0), ((8, 4, 8), 128, 1), ((4, 4, 8), 256, 0), ((16, 2, 8), 64, 1), ((8, 8, 4), 512, 0),
        ((8, 2, 16), 128, 1), ((4, 2, 4), 256, 1), ((16, 4, 16), 64, 0)]


def _scenes(ctx):
    arrays = [scenes.build_scene_tris(n, 70 + i, (-12, 0, -12), (12, 8, 12)) for i, n in enumerate((15000, 6000))]
    return [ddgi.Scene(ctx, a) for a in arrays]


def _serve(ctx, scs, max_batch, in_flight, conv_mode, budget=8 << 30, policy=L.DDGI_SERVE_FIFO):
    srv = ddgi.Server(ctx, budget, max_batch=max_batch, in_flight=in_flight, conv_mode=conv_mode, policy=policy,
                      aging_ms=50.0)
    # outputs and descriptions first, so the requests arrive back to back (a pinned allocation between two
    # submissions would let each request finish before the next one arrives)
    outs = [torch.empty(10 * dims[0] * 10 * dims[2] * dims[1] * 4, dtype=torch.float32).pin_memory()
            for dims, _, _ in REQS]
    work = [(ddgi.grid_desc(dims, rays_per_probe=n, hysteresis=0.97),
             ddgi.FrameParams(camera_pos=(0.3 * i, 1.0, -0.2 * i), rotation=scenes.rotation(i, 0)), si)
            for i, (dims, n, si) in enumerate(REQS)]
    ids = []
    try:
        for i, (d, fp, si) in enumerate(work):
            ids.append(srv.submit(scs[si], d, fp, outs[i].data_ptr(), tag=i))
        srv.drain(120.0)
        for rid in ids:
            assert srv.status(rid).state == L.DDGI_REQUEST_DONE
        st = srv.stats
        assert st.completed == len(REQS) and st.failed == 0 and st.rejected == 0
        assert st.peakBytes <= budget
        ctx.sync()
        return [o.numpy().copy() for o in outs], st
    finally:
        srv.close()


# 1 (FP16 tensor cores) with shortest-first admission over four slots is what the serving bench runs
@pytest.mark.parametrize("conv_mode,policy,slots", [(0, L.DDGI_SERVE_FIFO, 2), (1, L.DDGI_SERVE_FIFO, 2),
                                                    (2, L.DDGI_SERVE_FIFO, 2), (1, L.DDGI_SERVE_SHORTEST_FIRST, 4)])
def test_request_alone_equals_in_the_mix(ctx, conv_mode, policy, slots):
    scs = _scenes(ctx)
    try:
        alone, st1 = _serve(ctx, scs, max_batch=1, in_flight=1, conv_mode=conv_mode)
        mixed, st2 = _serve(ctx, scs, max_batch=64, in_flight=slots, conv_mode=conv_mode, policy=policy)
        assert st1.batches == len(REQS)
        assert st2.batches < len(REQS)  # requests shared launches
        for i, (a, b) in enumerate(zip(alone, mixed)):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), i
        # and equal to a grid updated through ddgi_update
        dims, n, si = REQS[3]
        g = ddgi.ProbeGrid(ctx, dims, (1.0, 2.0, 1.0), n, 0.0, 0.97)
        g.set_tuning(warp_probes=2, conv_mode=conv_mode)
        g.update(scs[si], ddgi.FrameParams(camera_pos=(0.9, 1.0, -0.6), rotation=scenes.rotation(3, 0)))
        ctx.sync()
        assert np.array_equal(g.download_atlas().reshape(-1).view(np.uint32), alone[3].view(np.uint32))
        g.close()
    finally:
        for s in scs:
            s.close()


def test_budget_admission_and_rejection(ctx):
    scs = _scenes(ctx)
    try:
        d = ddgi.grid_desc((8, 4, 8), rays_per_probe=128)
        need = L.load().ddgi_grid_footprint(d, 0)
        srv = ddgi.Server(ctx, 2 * need + need // 2, max_batch=64, in_flight=2)  # room for two at a time
        try:
            ids = [srv.submit(scs[0], d, ddgi.FrameParams(rotation=scenes.rotation(k, 1))) for k in range(6)]
            big = ddgi.grid_desc((32, 8, 32), rays_per_probe=512)
            with pytest.raises(L.DdgiError) as e:
                srv.submit(scs[0], big, ddgi.FrameParams())
            assert e.value.code == L.DDGI_EBUSY
            srv.drain(120.0)
            st = srv.stats
            assert st.completed == 6 and st.rejected == 1
            assert st.peakBytes <= 2 * need + need // 2
            assert all(srv.status(i).state == L.DDGI_REQUEST_DONE for i in ids)
        finally:
            srv.close()
    finally:
        for s in scs:
            s.close()


def test_ray_cap_splits_launches(ctx):
    """maxBatchMRays: a launch admits requests while their rays stay within the cap (a larger request runs
    alone); the atlases are the same as without the cap."""
    scs = _scenes(ctx)
    d = ddgi.grid_desc((16, 4, 16), rays_per_probe=512)  # 524,288 rays: two exceed 1 million
    frames = [ddgi.FrameParams(camera_pos=(0.2 * k, 1.0, 0.1), rotation=scenes.rotation(k, 2)) for k in range(6)]

    def run(cap):
        srv = ddgi.Server(ctx, 8 << 30, max_batch=64, in_flight=1, conv_mode=0, max_batch_mrays=cap)
        outs = [torch.empty(10 * 16 * 10 * 16 * 4 * 4, dtype=torch.float32).pin_memory() for _ in frames]
        try:
            for k, fp in enumerate(frames):
                srv.submit(scs[k % 2], d, fp, outs[k].data_ptr(), tag=k)
            srv.drain(120.0)
            st = srv.stats
            assert st.completed == len(frames) and st.failed == 0
            ctx.sync()
            return [o.numpy().copy() for o in outs], st
        finally:
            srv.close()

    try:
        free, _ = run(0)
        capped, st = run(1)
        assert st.batches == len(frames)  # one request per launch
        for k, (a, b) in enumerate(zip(free, capped)):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), k
    finally:
        for s in scs:
            s.close()


@pytest.mark.parametrize("aging_ms,order", [(1e6, ["small", "medium", "large"]), (1e-3, ["large", "small", "medium"])])
def test_shortest_first_admission_and_aging(ctx, aging_ms, order):
    """With one slot and one request per launch, requests queued behind a running one are admitted shortest
    first; with an aging time far below the queueing time every request has aged fully and they go in
    arrival order."""
    scs = _scenes(ctx)
    blocker = ddgi.grid_desc((32, 8, 32), rays_per_probe=512)  # 4.2 M rays: the others queue behind it
    sizes = {"large": ((16, 4, 16), 256), "small": ((4, 2, 4), 64), "medium": ((8, 4, 8), 128)}
    descs = {k: ddgi.grid_desc(dims, rays_per_probe=n) for k, (dims, n) in sizes.items()}
    srv = ddgi.Server(ctx, 8 << 30, max_batch=1, in_flight=1, policy=L.DDGI_SERVE_SHORTEST_FIRST, aging_ms=aging_ms)
    try:
        fp = ddgi.FrameParams(rotation=scenes.rotation(1, 1))
        srv.submit(scs[0], blocker, fp)
        ids = {k: srv.submit(scs[0], descs[k], fp) for k in ("large", "small", "medium")}  # arrival order
        srv.drain(120.0)
        admitted = sorted(ids, key=lambda k: srv.status(ids[k]).admitSeconds)
        assert admitted == order, [(k, srv.status(ids[k]).admitSeconds) for k in ids]
        assert srv.stats.completed == 4
    finally:
        srv.close()
        for s in scs:
            s.close()


def test_server_config_is_validated(ctx):
    for kw in (dict(policy=7), dict(in_flight=9), dict(aging_ms=-1.0)):
        with pytest.raises(L.DdgiError) as e:
            ddgi.Server(ctx, 1 << 30, **kw)
        assert e.value.code == L.DDGI_EINVAL
    ddgi.Server(ctx, 1 << 30, in_flight=8, policy=L.DDGI_SERVE_SHORTEST_FIRST).close()
