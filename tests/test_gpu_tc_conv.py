"""Tensor-core (tcgen05) probe convolution against the FP64 oracle.

The inputs are the FP64 radiance R (log-uniform per channel in [1e-3, 1e2], the precision workload's
distribution); the device sees R rounded to FP16 or BF16 and weights rounded likewise, accumulates in FP32
and blends in FP32. Stated tolerances, per texel channel relative to the FP64 oracle on the unrounded R:
FP16 <= 1e-3 (max), the bound the engine's batched and served updates are held to; BF16 <= 8e-3 (max). Each
rounding (of a radiance and of a weight; unit roundoff 2^-11 for FP16, 2^-9 for BF16) moves a weighted mean by
an amount that grows with the spread of the radiance it averages, here five decades: BF16 measured up to 4.1e-3
on these inputs and 5.7e-3 on traced radiance, so BF16 does not meet 1e-3 and is offered only as an extra mode.
Against the oracle fed the same rounded R: FP16 <= 2e-3, BF16 <= 8e-3 (the weights are still rounded to 16 bits
and the bake sums are not renormalised)."""
import ctypes as C

import numpy as np
import pytest

from anerend_gb300 import _lib as L
from anerend_gb300 import ddgi, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def desc(dims, n, h=0.97):
    d = L.GridDesc()
    d.dims[:] = list(dims)
    d.step[:] = [1.0, 2.0, 1.0]
    d.originY = 0.0
    d.raysPerProbe = n
    d.atlasFormat = L.DDGI_FORMAT_RGBA32F
    d.hysteresis = h
    d.options = 0
    return d


def round16(x: np.ndarray, fmt: int) -> np.ndarray:
    if fmt == L.DDGI_ELEM_F16:
        return x.astype(np.float16)
    t = torch.from_numpy(x.astype(np.float32)).to(torch.bfloat16)
    return t


def planar16(R: np.ndarray, fmt: int):
    """R: (3, P, N) float64 -> device tensor of 16-bit values, and its rounded float64 copy."""
    if fmt == L.DDGI_ELEM_F16:
        h = R.astype(np.float16)
        return torch.from_numpy(h.view(np.int16)).cuda(), h.astype(np.float64)
    t = torch.from_numpy(R.astype(np.float32)).to(torch.bfloat16)
    return t.view(torch.int16).cuda(), t.to(torch.float64).numpy()


def ray_image(g: oracle.GridGeom, R: np.ndarray) -> np.ndarray:
    """(3, P, N) -> RGBA ray image (rh, rw, 4) in the reference layout."""
    bw, bh = g.block
    rh, rw = g.ray_hw
    img = np.zeros((rh, rw, 4))
    img[..., 3] = 1.0
    P = g.X * g.Y * g.Z
    p = np.arange(P)
    px, pz = p % g.X, p // g.X
    for j in range(g.N):
        img[pz * bh + j // bw, px * bw + j % bw, :3] = R[:, :, j].T
    return img


@pytest.mark.parametrize("fmt", [L.DDGI_ELEM_F16, L.DDGI_ELEM_BF16])
@pytest.mark.parametrize("n,dims,layers", [
    (64, (5, 3, 3), None), (256, (8, 2, 9), None), (512, (16, 2, 8), None),
    # more 64-probe units than SMs, so CTAs take two-unit tiles; a layer range starting mid-unit and a
    # last unit cut short by the grid's end
    (64, (61, 9, 37), (2, 9)),
])
@pytest.mark.parametrize("bake", [False, True])
def test_tc_convolve_matches_fp64(ctx, fmt, n, dims, layers, bake):
    lib = L.load()
    d = desc(dims, n)
    g = oracle.GridGeom(*dims, n)
    P = dims[0] * dims[1] * dims[2]
    rng = np.random.default_rng(n + 7 * fmt)
    R = np.exp(rng.uniform(np.log(1e-3), np.log(1e2), size=(3, P, n)))
    ah, aw = g.atlas_hw
    atlas = rng.uniform(0.0, 3.0, size=(ah, aw, 4)).astype(np.float32)
    if bake:
        atlas[..., 3] = rng.uniform(0.0, 20.0, size=(ah, aw))
    rot = scenes.rotation(5, n)
    stream = torch.cuda.current_stream().cuda_stream
    dirs = torch.empty(n * 4, dtype=torch.float32, device="cuda")
    assert lib.ddgi_fibonacci_lattice(n, (C.c_float * 9)(*rot.tolist()), dirs.data_ptr(), stream) == 0
    r16, r16d = planar16(R, fmt)
    a_dev = torch.from_numpy(atlas).cuda()
    flags = L.DDGI_UBO_BAKE_MODE_ON_FLAG if bake else 0
    b, e = layers or (0, dims[1])
    ctx.check(lib.ddgi_convolve_tc_raw(ctx.handle, C.byref(d), r16.data_ptr(), fmt, dirs.data_ptr(),
                                       a_dev.data_ptr(), b, e, flags, stream))
    ctx.sync(stream)
    got = a_dev.cpu().numpy().astype(np.float64)
    dirs64 = dirs.cpu().numpy().reshape(n, 4)[:, :3].astype(np.float64)
    want_exact = atlas.astype(np.float64)
    oracle.convolve(d, ray_image(g, R), dirs64, want_exact, b, e, flags)
    want_rounded = atlas.astype(np.float64)
    oracle.convolve(d, ray_image(g, r16d), dirs64, want_rounded, b, e, flags)
    err_exact = np.abs(got - want_exact) / np.maximum(np.abs(want_exact), 1e-6)
    err_round = np.abs(got - want_rounded) / np.maximum(np.abs(want_rounded), 1e-6)
    bound = 1e-3 if fmt == L.DDGI_ELEM_F16 else 8e-3
    assert err_exact[..., :3].max() <= bound, (float(err_exact[..., :3].max()), float(np.percentile(err_exact, 99)))
    # weights rounded to 16 bits: FP16 unit roundoff 2^-11, BF16 2^-8 (bake sums are not renormalised)
    assert err_round[..., :3].max() <= (2e-3 if fmt == L.DDGI_ELEM_F16 else 8e-3), float(err_round[..., :3].max())
    assert err_round[..., 3].max() <= 1e-5  # .w: FP32 weight sums


def test_tc_rejects_bad_arguments(ctx):
    lib = L.load()
    d = desc((2, 1, 2), 32)  # N not a multiple of 64
    x = torch.zeros(1024, dtype=torch.int16, device="cuda")
    rc = lib.ddgi_convolve_tc_raw(ctx.handle, C.byref(d), x.data_ptr(), 0, x.data_ptr(), x.data_ptr(), 0, 1, 0, None)
    assert rc == L.DDGI_EINVAL
    d = desc((2, 1, 2), 64)
    rc = lib.ddgi_convolve_tc_raw(ctx.handle, C.byref(d), x.data_ptr(), 7, x.data_ptr(), x.data_ptr(), 0, 1, 0, None)
    assert rc == L.DDGI_EINVAL
    ctx.sync()


@pytest.mark.parametrize("conv_mode", [1, 2])
def test_grid_update_with_tensor_core_convolution(ctx, conv_mode):
    """Full probe updates of the 8x4x8 / 64-ray workload with the tensor-core convolution against the FP64
    oracle: hits bit-exact on certain rays, atlas within the 16-bit tolerance (FP16 2e-3, BF16 8e-3 at the
    99.9th percentile: eight hysteresis-blended frames, each feeding the next frame's probe lookup)."""
    w = scenes.CPU_REFERENCE
    arrays = scenes.build_scene(w)
    scene = ddgi.Scene(ctx, arrays)
    grid = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis, options=L.DDGI_GRID_RECORD_HITS)
    grid.set_tuning(conv_mode=conv_mode)
    osc = oracle.OracleScene(arrays, L.SceneDesc)
    og = oracle.OracleGrid(grid.desc)
    try:
        for f in range(w.frames):
            fp = ddgi.FrameParams(camera_pos=scenes.camera(w, f), rotation=scenes.rotation(w.seed, f))
            grid.update(scene, fp)
            og.update(osc, fp.to_c())
            ctx.sync()
            _, hits, _ = grid.download_rays(hits=True)
            certain = og.uncertain == 0
            assert np.array_equal(hits[certain], og.hits[certain])
        atlas = grid.download_atlas().astype(np.float64)
        err = np.abs(atlas - og.atlas) / np.maximum(np.abs(og.atlas), 1e-3)
        bound = 2e-3 if conv_mode == 1 else 8e-3
        assert np.percentile(err, 99.9) <= bound, np.percentile(err, [50, 99, 99.9, 100])
    finally:
        osc.close()
        grid.close()
        scene.close()
