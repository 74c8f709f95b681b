"""Failure detection without a GPU fault.

  - Bounded device waits: the tensor-core convolution's test hook makes each CTA's first accumulator wait wait
    for an mbarrier phase that no arrival completes. The wait gives up after the context's spin limit; the kernel
    raises the sticky timeout, waits for its own copies and tensor-core work in flight, releases its tensor
    memory and returns. ddgi_sync reports DDGI_ETIMEDOUT, and the same context then convolves correctly.
  - Allocation failures: an allocation hook that refuses device memory makes grid and scene creation fail with
    DDGI_ENOMEM, leaving nothing half-built; without the hook the same calls succeed.
Nothing here traps, faults or hangs the GPU: every wait is bounded, and refusals happen on the host."""
import ctypes as C

import numpy as np
import pytest

from anerend_gb300 import _lib as L
from anerend_gb300 import ddgi, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _conv_inputs(dims, n, seed):
    P = dims[0] * dims[1] * dims[2]
    rng = np.random.default_rng(seed)
    R = np.exp(rng.uniform(np.log(1e-3), np.log(1e2), size=(3, P, n)))
    return R


def test_tensor_core_wait_timeout_reports_etimedout_and_context_recovers():
    lib = L.load()
    dims, n = (16, 2, 8), 512  # 256 probes: four 64-probe units, four CTAs
    d = ddgi.grid_desc(dims, rays_per_probe=n, hysteresis=0.0)
    R = _conv_inputs(dims, n, 3)
    r16 = torch.from_numpy(R.astype(np.float16).view(np.int16)).cuda()
    g = oracle.GridGeom(*dims, n)
    ah, aw = g.atlas_hw
    with ddgi.Context(0) as ctx:
        stream = torch.cuda.current_stream().cuda_stream
        dirs = torch.empty(n * 4, dtype=torch.float32, device="cuda")
        assert lib.ddgi_fibonacci_lattice(n, (C.c_float * 9)(*scenes.rotation(2, 0).tolist()), dirs.data_ptr(),
                                          stream) == L.DDGI_OK
        atlas = torch.zeros((ah, aw, 4), dtype=torch.float32, device="cuda")
        # a wait that nothing ends, bounded to 2^14 attempts (about a millisecond)
        ctx.check(lib.ddgi_context_set_waits(ctx.handle, C.byref(L.WaitConfig(1 << 14, 1))))
        rc = lib.ddgi_convolve_tc_raw(ctx.handle, C.byref(d), r16.data_ptr(), L.DDGI_ELEM_F16, dirs.data_ptr(),
                                      atlas.data_ptr(), 0, dims[1], 0, stream)
        assert rc == L.DDGI_OK  # the launch itself succeeds
        assert lib.ddgi_sync(ctx.handle, stream) == L.DDGI_ETIMEDOUT
        assert lib.ddgi_sync(ctx.handle, stream) == L.DDGI_OK  # the word was cleared
        # default waits again: the same context convolves, and the result is the oracle's
        ctx.check(lib.ddgi_context_set_waits(ctx.handle, C.byref(L.WaitConfig(0, 0))))
        atlas.zero_()
        ctx.check(lib.ddgi_convolve_tc_raw(ctx.handle, C.byref(d), r16.data_ptr(), L.DDGI_ELEM_F16, dirs.data_ptr(),
                                           atlas.data_ptr(), 0, dims[1], 0, stream))
        ctx.sync(stream)
        got = atlas.cpu().numpy().astype(np.float64)
    want = np.zeros((ah, aw, 4))
    bw, bh = g.block
    img = np.zeros((bh * dims[2] * dims[1], bw * dims[0], 4))
    p = np.arange(dims[0] * dims[1] * dims[2])
    for j in range(n):
        img[(p // dims[0]) * bh + j // bw, (p % dims[0]) * bw + j % bw, :3] = R[:, :, j].T
    oracle.convolve(d, img, dirs.cpu().numpy().reshape(n, 4)[:, :3].astype(np.float64), want, 0, dims[1], 0,
                    hysteresis=0.0)
    inner = want[..., 3] > 0  # interior texels (the border holds no result)
    err = np.abs(got[..., :3] - want[..., :3]) / np.maximum(np.abs(want[..., :3]), 1e-6)
    assert err[inner].max() <= 1e-3


def test_refused_allocations_give_enomem_and_leave_nothing_behind():
    lib = L.load()
    w = scenes.CPU_REFERENCE
    arrays = scenes.build_scene(w)
    seen = []
    budget = {"allow": 0}

    @L.ALLOC_HOOK
    def hook(user, nbytes):
        seen.append(int(nbytes))
        if budget["allow"] > 0:
            budget["allow"] -= 1
            return 0
        return 1  # refuse

    with ddgi.Context(0) as ctx:
        ctx.check(lib.ddgi_context_set_alloc_hook(ctx.handle, hook, None))
        d = ddgi.grid_desc(w.dims, rays_per_probe=w.rays, hysteresis=0.97)
        h = C.c_void_p()
        for allow in (0, 3):  # the first allocation refused, then the fourth
            budget["allow"] = allow
            seen.clear()
            rc = lib.ddgi_grid_create(ctx.handle, C.byref(d), C.byref(h))
            assert rc == L.DDGI_ENOMEM and not h.value
            assert len(seen) == allow + 1
            assert b"grid allocation" in lib.ddgi_last_error(ctx.handle)
        budget["allow"] = 0
        with pytest.raises(L.DdgiError) as e:
            ddgi.Scene(ctx, arrays)
        assert e.value.code == L.DDGI_ENOMEM
        # without the hook the same calls succeed, and the grid works
        ctx.check(lib.ddgi_context_set_alloc_hook(ctx.handle, L.ALLOC_HOOK(), None))
        scene = ddgi.Scene(ctx, arrays)
        grid = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis)
        grid.update(scene, ddgi.FrameParams(rotation=scenes.rotation(0, 0)))
        ctx.sync()
        assert np.isfinite(grid.download_atlas()).all()
        grid.close()
        scene.close()
