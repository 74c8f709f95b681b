"""GPU parity of every kernel on the path against the FP64 oracle, through the C ABI.

Tolerances (stated here, used below):
  - translation: bit-exact (integer gather of texel bits), RGBA32F and RGBA16F;
  - lattice: within one FP32 rounding of the FP64 oracle (the device computes it in FP64);
  - convolution, FP32 on CUDA cores: relative error <= 2e-5 per channel (abs floor 1e-6);
  - traced rays: hit triangle id and shadow bit bit-exact on every ray the oracle marks certain;
    radiance relative error <= 1e-4 on those rays when the previous atlas is identical;
  - atlas after several multi-bounce frames: relative error <= 1e-3 per texel channel for 99.9% of texels
    (the remaining rays near edges may legitimately pick the other triangle in FP32).
"""
import ctypes as C

import numpy as np
import pytest

from anerend_gb300 import _lib as L
from anerend_gb300 import ddgi, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def desc(dims, n, h=0.97, step=(1.0, 2.0, 1.0), origin_y=0.0, fmt=L.DDGI_FORMAT_RGBA32F, options=0):
    d = L.GridDesc()
    d.dims[:] = list(dims)
    d.step[:] = list(step)
    d.originY = origin_y
    d.raysPerProbe = n
    d.atlasFormat = fmt
    d.hysteresis = h
    d.options = options
    return d


def stream_ptr():
    return torch.cuda.current_stream().cuda_stream


def rel_err(got, want, floor=1e-6):
    return np.abs(got - want) / np.maximum(np.abs(want), floor)


# ---- lattice ------------------------------------------------------------------------------------

@pytest.mark.parametrize("n", [16, 64, 128, 256, 512, 1024])
def test_lattice_fp64_on_device(ctx, n):
    lib = L.load()
    rot = scenes.rotation(0, n)
    dev = torch.empty(n * 4, dtype=torch.float32, device="cuda")
    r = (C.c_float * 9)(*rot.tolist())
    assert lib.ddgi_fibonacci_lattice(n, r, dev.data_ptr(), stream_ptr()) == L.DDGI_OK
    torch.cuda.synchronize()
    got = dev.cpu().numpy().reshape(n, 4)
    want = oracle.lattice(n, rot)
    assert np.all(got[:, 3] == 0)
    assert np.max(np.abs(got[:, :3] - want)) <= 6e-8


# ---- translation ----------------------------------------------------------------------------------

@pytest.mark.parametrize("fmt", [L.DDGI_FORMAT_RGBA32F, L.DDGI_FORMAT_RGBA16F])
@pytest.mark.parametrize("dims", [(4, 3, 4), (32, 8, 32), (5, 2, 3)])
def test_translate_bit_exact(ctx, fmt, dims):
    lib = L.load()
    d = desc(dims, 64, fmt=fmt)
    X, Y, Z = dims
    texel = 16 if fmt == L.DDGI_FORMAT_RGBA32F else 8
    rng = np.random.default_rng(7)
    a = rng.integers(0, 2**32, size=(10 * Z * Y * 10 * X * texel // 4,), dtype=np.uint32)
    src = torch.from_numpy(a.view(np.int32)).cuda()
    dst = torch.empty_like(src)
    for dx, dz in [(1, 0), (-1, 0), (0, 1), (0, -1), (1, -1), (-1, 1), (0, 0), (4, -3)]:
        assert lib.ddgi_translate_raw(C.byref(d), src.data_ptr(), dst.data_ptr(), dx, dz, stream_ptr()) == L.DDGI_OK
        torch.cuda.synchronize()
        got = dst.cpu().numpy().view(np.uint32)
        want = oracle.translate(d, a.view(np.uint8).reshape(10 * Z * Y, 10 * X, texel), dx, dz)
        assert np.array_equal(got.view(np.uint8), want.reshape(-1)), (dx, dz)


# ---- convolution ---------------------------------------------------------------------------------

@pytest.mark.parametrize("n", [16, 64, 128, 256, 512, 1024])
@pytest.mark.parametrize("bake", [False, True])
def test_convolve_fp32(ctx, n, bake):
    lib = L.load()
    dims = (5, 3, 3)
    d = desc(dims, n, h=0.97)
    g = oracle.GridGeom(*dims, n)
    rh, rw = g.ray_hw
    ah, aw = g.atlas_hw
    rng = np.random.default_rng(n)
    rays = np.exp(rng.uniform(np.log(1e-3), np.log(1e2), size=(rh, rw, 4))).astype(np.float32)
    atlas = rng.uniform(0.0, 3.0, size=(ah, aw, 4)).astype(np.float32)
    rot = scenes.rotation(1, n)
    dirs = torch.empty(n * 4, dtype=torch.float32, device="cuda")
    assert lib.ddgi_fibonacci_lattice(n, (C.c_float * 9)(*rot.tolist()), dirs.data_ptr(), stream_ptr()) == 0
    r_dev = torch.from_numpy(rays).cuda()
    a_dev = torch.from_numpy(atlas).cuda()
    flags = L.DDGI_UBO_BAKE_MODE_ON_FLAG if bake else 0
    assert lib.ddgi_convolve_raw(C.byref(d), r_dev.data_ptr(), dirs.data_ptr(), a_dev.data_ptr(), 1, 3, flags,
                                 stream_ptr()) == L.DDGI_OK
    torch.cuda.synchronize()
    got = a_dev.cpu().numpy().astype(np.float64)
    want = atlas.astype(np.float64)
    dirs64 = dirs.cpu().numpy().reshape(n, 4)[:, :3].astype(np.float64)
    oracle.convolve(d, rays.astype(np.float64), dirs64, want, 1, 3, flags)
    # layer 0 untouched, every other texel within the stated tolerance
    assert np.array_equal(got[: 10 * dims[2]], atlas[: 10 * dims[2]].astype(np.float64))
    assert np.max(rel_err(got, want)) <= 2e-5


# ---- full update: trace + shade + convolve against the oracle ---------------------------------------

def _run_lockstep(ctx, w, frames, options=0, layer=-1, fmt=L.DDGI_FORMAT_RGBA32F, check_rays=True, tuning=None,
                  arrays=None):
    arrays = arrays if arrays is not None else scenes.build_scene(w)
    scene = ddgi.Scene(ctx, arrays)
    grid = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis, atlas_format=fmt,
                          options=options | L.DDGI_GRID_RECORD_HITS)
    if tuning:
        grid.set_tuning(**tuning)
    osc = oracle.OracleScene(arrays, L.SceneDesc)
    og = oracle.OracleGrid(grid.desc)
    stats = []
    try:
        for f in range(frames):
            fp = ddgi.FrameParams(camera_pos=scenes.camera(w, f), rotation=scenes.rotation(w.seed, f), layer=layer)
            prev_equal = f == 0
            grid.update(scene, fp)
            og.update(osc, fp.to_c())
            ctx.sync()
            if check_rays:
                rad, hits, _ = grid.download_rays(hits=True)
                b, e = og.traced
                rows = slice(b * g_rows(og), e * g_rows(og))
                certain = og.uncertain[rows] == 0
                hit_mismatch = int(np.count_nonzero((hits[rows] != og.hits[rows]) & certain))
                err = rel_err(rad[rows, :, :3].astype(np.float64), og.ray_rad[rows, :, :3], 1e-3)
                stats.append(dict(frame=f, certain=float(certain.mean()), hit_mismatch=hit_mismatch,
                                  ray_err_max=float(err[certain].max()), prev_equal=prev_equal))
        atlas = grid.download_atlas().astype(np.float64)
        return atlas, og.atlas.copy(), stats
    finally:
        osc.close()
        grid.close()
        scene.close()


def g_rows(og):
    return og.geom.ray_hw[0] // og.geom.Y


@pytest.mark.parametrize("tuning", [
    dict(shadow_mode=1, ray_order=1, warp_probes=2),   # light-space shadow BVH, Morton direction order
    dict(shadow_mode=0, ray_order=0, warp_probes=32),  # scene-BVH shadow rays, 32 parallel rays per warp
    dict(shadow_mode=1, ray_order=0, warp_probes=1),
    dict(shadow_mode=1, ray_order=1, warp_probes=2, bvh_width=2),  # the binary LBVH instead of the 8-wide tree
])
def test_cpu_reference_workload_8_frames(ctx, tuning):
    w = scenes.CPU_REFERENCE
    atlas, want, stats = _run_lockstep(ctx, w, w.frames, tuning=tuning)
    for s in stats:
        assert s["hit_mismatch"] == 0, s
        assert s["certain"] > 0.99, s
        if s["prev_equal"]:
            assert s["ray_err_max"] <= 1e-4, s
        else:
            assert s["ray_err_max"] <= 1e-2, s
    err = rel_err(atlas, want, 1e-3)
    assert np.percentile(err, 99.9) <= 1e-3, np.percentile(err, [50, 99, 99.9, 100])


def test_cpu_reference_workload_lockstep_clean_texels(ctx):
    """The 8x4x8 / 64-ray workload with the oracle started every frame from the device's atlas: every texel of a
    probe whose 64 rays the oracle marks certain within 1e-4 (floor 1e-3), frame after frame, beside the 99.9th
    percentile over all texels (1e-3). The free-running comparison above excuses 0.1 % of texels; this one
    bounds the maximum wherever no uncertain ray reached."""
    w = scenes.CPU_REFERENCE
    arrays = scenes.build_scene(w)
    scene = ddgi.Scene(ctx, arrays)
    grid = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis, options=L.DDGI_GRID_RECORD_HITS)
    osc = oracle.OracleScene(arrays, L.SceneDesc)
    og = oracle.OracleGrid(grid.desc)
    X, Y, Z = w.dims
    bw, bh = og.geom.block
    try:
        for f in range(w.frames):
            fp = ddgi.FrameParams(camera_pos=scenes.camera(w, f), rotation=scenes.rotation(w.seed, f))
            og.atlas = grid.download_atlas().astype(np.float64)
            grid.update(scene, fp)
            og.update(osc, fp.to_c())
            ctx.sync()
            atlas = grid.download_atlas().astype(np.float64)
            err = rel_err(atlas, og.atlas, 1e-3)
            tainted = (og.uncertain != 0).reshape(Y, Z, bh, X, bw).any(axis=(2, 4)).reshape(Y * Z, X)
            clean = ~np.repeat(np.repeat(tainted, 10, axis=0), 10, axis=1)
            assert clean.mean() > 0.5, f
            assert err[clean].max() <= 1e-4, (f, float(err[clean].max()))
            assert np.percentile(err, 99.9) <= 1e-3, (f, float(np.percentile(err, 99.9)))
    finally:
        osc.close()
        grid.close()
        scene.close()


def test_round_robin_layers_and_edge_clamp(ctx):
    w = scenes.Workload("rr_6x3x5_n128", (6, 3, 5), (1.0, 1.5, 1.0), -1.0, 128, 2000, (-6, -4, -6), (6, 4, 6),
                        4, 0, -3.0, 8.0, 6, 0.96)
    atlas, want, stats = _run_lockstep(ctx, w, 6, options=L.DDGI_GRID_EDGE_CLAMP, layer=-2)
    for s in stats:
        assert s["hit_mismatch"] == 0, s
    err = rel_err(atlas, want, 1e-3)
    assert np.percentile(err, 99.9) <= 1e-3


def test_fp16_atlas(ctx):
    w = scenes.Workload("fp16_4x2x4_n64", (4, 2, 4), (1.0, 1.0, 1.0), -0.5, 64, 1000, (-5, -5, -5), (5, 5, 5),
                        1, 0, -2.0, 6.0, 4, 0.97)
    atlas, want, stats = _run_lockstep(ctx, w, 4, fmt=L.DDGI_FORMAT_RGBA16F)
    err = rel_err(atlas, want, 1e-2)
    assert np.percentile(err, 99) <= 5e-3


def test_bake_mode_matches_oracle(ctx):
    """Bake mode (rgen:61-73 tile origin, pbr_light.glsl:276-293 tile lookup, probe_conv.comp:307-319
    accumulation, translation skipped): four accumulated frames against the oracle."""
    w = scenes.Workload("bake_8x2x8_n64", (8, 2, 8), (1.0, 1.0, 1.0), 0.0, 64, 1500, (0, -1, 0), (16, 3, 16), 1, 0,
                        -1.5, 20.0, 4, 0.96)
    arrays = scenes.build_scene(w)
    scene = ddgi.Scene(ctx, arrays)
    grid = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis, options=L.DDGI_GRID_RECORD_HITS)
    osc = oracle.OracleScene(arrays, L.SceneDesc)
    og = oracle.OracleGrid(grid.desc)
    try:
        zero = np.zeros(grid.atlas_shape(), np.float32)  # bake starts from an empty accumulation
        grid.upload_atlas(zero)
        og.atlas[...] = 0.0
        for f in range(w.frames):
            fp = ddgi.FrameParams(camera_pos=(3.7, 0.0, -2.2), rotation=scenes.rotation(9, f),
                                  flags=L.DDGI_UBO_DDGI_FLAG | L.DDGI_UBO_DDGI_MULTI_FLAG | L.DDGI_UBO_BAKE_MODE_ON_FLAG,
                                  bake_tile=(0, 0, 16))
            grid.update(scene, fp)  # ddgi_update skips the translation while baking (TranslationPass.cpp:59)
            og.trace(osc, fp.to_c())
            og.convolve(fp.to_c())
            ctx.sync()
            _, hits, _ = grid.download_rays(hits=True)
            certain = og.uncertain == 0
            assert np.array_equal(hits[certain], og.hits[certain])
        atlas = grid.download_atlas().astype(np.float64)
        err = np.abs(atlas - og.atlas) / np.maximum(np.abs(og.atlas), 1e-3)
        assert np.percentile(err, 99.9) <= 1e-3, np.percentile(err, [50, 99, 99.9, 100])
        assert atlas[1:9, 1:9, 3].min() > 0  # accumulated weight
    finally:
        osc.close()
        grid.close()
        scene.close()


def test_closed_octahedron_is_watertight(ctx):
    # one probe inside a closed octahedron: every ray of every rotation must hit (no leak at edges/vertices)
    X, Y, Z = 1, 1, 1
    probe = np.array([-0.5, 0.0, -0.5])  # (0,0,0) * step + camOffset with camera at the origin
    v = np.array([[3, 0, 0], [-3, 0, 0], [0, 3, 0], [0, -3, 0], [0, 0, 3], [0, 0, -3]], np.float64) + probe
    faces = [(0, 2, 4), (2, 1, 4), (1, 3, 4), (3, 0, 4), (2, 0, 5), (1, 2, 5), (3, 1, 5), (0, 3, 5)]
    tris = np.array([[v[a], v[b], v[c]] for a, b, c in faces])
    arrays = scenes.assemble(tris, np.arange(8), np.arange(8), scenes.random_materials(3, 8))
    scene = ddgi.Scene(ctx, arrays)
    grid = ddgi.ProbeGrid(ctx, (X, Y, Z), (1.0, 1.0, 1.0), 1024, 0.0, 0.97, options=L.DDGI_GRID_RECORD_HITS)
    try:
        for f in range(8):
            rot = scenes.rotation(11, f) if f else np.eye(3, dtype=np.float32).reshape(-1)
            grid.trace(scene, ddgi.FrameParams(rotation=rot))
            ctx.sync()
            _, hits, _ = grid.download_rays(hits=True)
            assert np.all(hits >= 0), int(np.count_nonzero(hits < 0))
    finally:
        grid.close()
        scene.close()


def test_empty_scene_is_all_sky(ctx):
    from anerend_gb300.scenes import Scene as Arrays

    arrays = Arrays(np.zeros(0, L.PACKED_VERTEX), np.zeros(0, np.uint32), np.zeros(0, L.MESH_INFO),
                    np.zeros(0, L.INSTANCE), np.zeros(0, L.MATERIAL_INFO))
    scene = ddgi.Scene(ctx, arrays)
    grid = ddgi.ProbeGrid(ctx, (3, 2, 5), (1.0, 1.0, 1.0), 16, 0.0, 0.96, options=L.DDGI_GRID_RECORD_HITS)
    try:
        fp = ddgi.FrameParams(sky_color=(0.4, 0.5, 0.7), sky_intensity=1.0)
        grid.update(scene, fp)
        ctx.sync()
        rad, hits, _ = grid.download_rays(hits=True)
        assert np.all(hits == -1)
        lin = lambda c: c / 12.92 if c < 0.04045 else ((c + 0.055) / 1.055) ** 2.4  # noqa: E731
        sky = np.array([lin(0.4), lin(0.5), lin(0.7)])
        assert np.allclose(rad[..., :3], sky, rtol=1e-6)
        # every texel converges towards the sky radiance: one frame = 0.04 * sky
        atlas = grid.download_atlas()
        assert np.allclose(atlas[1:9, 1:9, :3], (1 - np.float32(0.96)) * sky, rtol=1e-5)
    finally:
        grid.close()
        scene.close()


def test_single_triangle_scene(ctx):
    tris = np.array([[[-20, -1, -20], [20, -1, -20], [0, -1, 30]]], np.float64)
    arrays = scenes.assemble(tris, np.array([0]), np.array([0]), scenes.random_materials(5, 1))
    scene = ddgi.Scene(ctx, arrays)
    grid = ddgi.ProbeGrid(ctx, (2, 1, 2), (1.0, 1.0, 1.0), 64, 0.0, 0.96, options=L.DDGI_GRID_RECORD_HITS)
    osc = oracle.OracleScene(arrays, L.SceneDesc)
    og = oracle.OracleGrid(grid.desc)
    try:
        fp = ddgi.FrameParams(rotation=scenes.rotation(2, 0))
        grid.update(scene, fp)
        og.update(osc, fp.to_c())
        ctx.sync()
        rad, hits, _ = grid.download_rays(hits=True)
        certain = og.uncertain == 0
        assert np.array_equal(hits[certain], og.hits[certain])
        assert np.any(hits >= 0) and np.any(hits < 0)
        assert np.max(rel_err(rad[..., :3].astype(np.float64), og.ray_rad[..., :3], 1e-3)[certain]) <= 1e-4
    finally:
        osc.close()
        grid.close()
        scene.close()


def test_errors_are_status_codes(ctx):
    lib = L.load()
    # bad grid descriptions
    for kw in [dict(dims=(0, 1, 1)), dict(rays_per_probe=100), dict(rays_per_probe=2048), dict(step=(0, 1, 1))]:
        args = dict(dims=(2, 2, 2), step=(1, 1, 1), rays_per_probe=64)
        args.update(kw)
        with pytest.raises(L.DdgiError) as e:
            ddgi.ProbeGrid(ctx, args["dims"], args["step"], args["rays_per_probe"])
        assert e.value.code == L.DDGI_EINVAL
    # textured material
    arrays = scenes.build_scene(scenes.Workload("err", (2, 1, 2), (1, 1, 1), 0, 16, 8, (-1, -1, -1), (1, 1, 1), 1, 0,
                                                None, 0, 1, 0.96))
    arrays.materials["bindlessIndices"][0, 1] = 3
    with pytest.raises(L.DdgiError) as e:
        ddgi.Scene(ctx, arrays)
    assert e.value.code == L.DDGI_EUNSUPPORTED
    # index out of its mesh
    arrays.materials["bindlessIndices"] = -1
    arrays.indices[2] = 999
    with pytest.raises(L.DdgiError) as e:
        ddgi.Scene(ctx, arrays)
    assert e.value.code == L.DDGI_EINVAL
    arrays.indices[2] = 2
    scene = ddgi.Scene(ctx, arrays)
    grid = ddgi.ProbeGrid(ctx, (2, 2, 2), (1, 1, 1), 16)
    try:
        with pytest.raises(L.DdgiError):  # convolve before any trace
            grid.convolve(ddgi.FrameParams())
        with pytest.raises(L.DdgiError):  # layer out of range
            grid.trace(scene, ddgi.FrameParams(layer=5))
        with pytest.raises(L.DdgiError):  # wrong atlas size
            grid.upload_atlas(np.zeros(7, np.float32))
        with pytest.raises(L.DdgiError):  # bake mode without a tile size
            grid.trace(scene, ddgi.FrameParams(flags=L.DDGI_UBO_BAKE_MODE_ON_FLAG))
        assert lib.ddgi_translate_raw(C.byref(grid.desc), 0, 0, 1, 0, None) == L.DDGI_EINVAL
        ctx.sync()
    finally:
        grid.close()
        scene.close()


def test_single_grid_workload_translation_and_rays(ctx):
    """The 32x8x32 / 256-ray / 262,144-triangle workload: translation indices bit-exact when the camera
    moves, and one layer of the first frame against the oracle."""
    w = scenes.SINGLE_GRID
    arrays = scenes.build_scene(w)
    scene = ddgi.Scene(ctx, arrays)
    assert scene.info.numTriangles == 262144
    grid = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis, options=L.DDGI_GRID_RECORD_HITS)
    osc = oracle.OracleScene(arrays, L.SceneDesc)
    try:
        og = oracle.OracleGrid(grid.desc)
        fp = ddgi.FrameParams(camera_pos=scenes.camera(w, 0), rotation=scenes.rotation(w.seed, 0), layer=3)
        grid.trace(scene, fp)
        og.trace(osc, fp.to_c())
        ctx.sync()
        rad, hits, _ = grid.download_rays(hits=True)
        rows = slice(3 * g_rows(og), 4 * g_rows(og))
        certain = og.uncertain[rows] == 0
        assert certain.mean() > 0.99
        assert np.array_equal(hits[rows][certain], og.hits[rows][certain])
        assert np.max(rel_err(rad[rows, :, :3].astype(np.float64), og.ray_rad[rows, :, :3], 1e-3)[certain]) <= 1e-4
        # frames 0..10 through ddgi_update; the camera steps +1 in x at frame 10
        for f in range(w.move_every + 1):
            fp = ddgi.FrameParams(camera_pos=scenes.camera(w, f), rotation=scenes.rotation(w.seed, f))
            if f == w.move_every:
                before = grid.download_atlas()
                assert grid.translate(fp.camera_pos)
                after = grid.download_atlas()
                want = oracle.translate(grid.desc, before, 1, 0)
                assert np.array_equal(after.view(np.uint32), want.view(np.uint32))
            grid.update(scene, fp)
        ctx.sync()
    finally:
        osc.close()
        grid.close()
        scene.close()


@pytest.mark.parametrize("shadow_mode", [0, 1])
def test_bvh_widths_give_identical_rays(ctx, shadow_mode):
    """The 8-wide BVH and the binary LBVH it is collapsed from return the same closest hit and shadow bit
    for every ray, so the traced radiance is bit-identical (one layer of the 262,144-triangle workload)."""
    w = scenes.SINGLE_GRID
    scene = ddgi.Scene(ctx, scenes.build_scene(w))
    grid = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis, options=L.DDGI_GRID_RECORD_HITS)
    try:
        out = {}
        for width in (8, 2):
            grid.set_tuning(shadow_mode=shadow_mode, bvh_width=width)
            assert grid.tuning.bvhWidth == width
            fp = ddgi.FrameParams(camera_pos=scenes.camera(w, 0), rotation=scenes.rotation(w.seed, 0), layer=5)
            grid.trace(scene, fp)
            ctx.sync()
            rad, hits, _ = grid.download_rays(hits=True)
            out[width] = (rad.copy(), hits.copy())
        rows = slice(5 * w.dims[2] * 16, 6 * w.dims[2] * 16)
        assert np.array_equal(out[8][1][rows], out[2][1][rows])
        assert np.array_equal(out[8][0][rows].view(np.uint32), out[2][0][rows].view(np.uint32))
        assert (out[8][1][rows] >= 0).mean() > 0.5
    finally:
        grid.close()
        scene.close()


def test_bvh_width_is_validated(ctx):
    grid = ddgi.ProbeGrid(ctx, (4, 2, 4), (1.0, 1.0, 1.0), 64, 0.0, 0.97)
    try:
        assert grid.tuning.bvhWidth == 8
        with pytest.raises(L.DdgiError):
            grid.set_tuning(bvh_width=4)
    finally:
        grid.close()


@pytest.mark.parametrize("shadow_mode", [0, 1])
def test_skipped_shadow_rays_leave_radiance_unchanged(ctx, shadow_mode):
    """A trace without per-ray hit codes casts no shadow ray for a hit whose lit and shadowed radiance have
    the same bits (calcLight is exactly 0 on a surface facing away from the sun); a recorded trace casts all
    of them. Ray radiance and atlas must stay bit-identical between the two over several multi-bounce frames
    of the 4096-triangle workload."""
    w = scenes.CPU_REFERENCE
    scene = ddgi.Scene(ctx, scenes.build_scene(w))
    grids = [ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis, options=o)
             for o in (0, L.DDGI_GRID_RECORD_HITS)]
    try:
        for g in grids:
            g.set_tuning(shadow_mode=shadow_mode)
        for f in range(4):
            fp = ddgi.FrameParams(camera_pos=scenes.camera(w, f), rotation=scenes.rotation(w.seed, f))
            for g in grids:
                g.update(scene, fp)
            ctx.sync()
            (rad0, _, _), (rad1, hits, _) = grids[0].download_rays(), grids[1].download_rays(hits=True)
            assert np.array_equal(rad0.view(np.uint32), rad1.view(np.uint32)), f
            assert np.array_equal(grids[0].download_atlas().view(np.uint32), grids[1].download_atlas().view(np.uint32))
        assert (hits >= 0).mean() > 0.3  # the frames hit geometry (about half of it facing away from the sun)
    finally:
        for g in grids:
            g.close()
        scene.close()


@pytest.mark.parametrize("bvh_width", [8, 2])
def test_seeded_closest_hits_equal_unseeded(ctx, bvh_width):
    """A grid traced frame after frame first tests, for each ray, the closest hit its probe's ray in the
    nearest direction of the previous lattice had, and for each shadow ray that ray's occluder; a fresh grid
    has no such candidates. Hit ids and shadow bits of every ray must be the same either way, across frames
    8-11 of the 262,144-triangle workload (the camera moves between frames 9 and 10)."""
    w = scenes.SINGLE_GRID
    scene = ddgi.Scene(ctx, scenes.build_scene(w))
    opts = L.DDGI_GRID_RECORD_HITS
    seeded = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis, options=opts)
    try:
        seeded.set_tuning(bvh_width=bvh_width)
        for f in range(8, 12):
            fp = ddgi.FrameParams(camera_pos=scenes.camera(w, f), rotation=scenes.rotation(w.seed, f), layer=3)
            seeded.update(scene, fp)
            fresh = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis, options=opts)
            try:
                fresh.set_tuning(bvh_width=bvh_width)
                fresh.update(scene, fp)
                ctx.sync()
                _, want, _ = fresh.download_rays(hits=True)
                _, got, _ = seeded.download_rays(hits=True)
            finally:
                fresh.close()
            rows = slice(3 * w.dims[2] * 16, 4 * w.dims[2] * 16)
            assert np.array_equal(got[rows], want[rows]), f
            assert (got[rows] >= 0).mean() > 0.5
    finally:
        seeded.close()
        scene.close()


def test_dark_materials_take_the_vertex_colour(ctx):
    """Materials whose base colour factor sums to <= 0.1 are shaded with the interpolated vertex colour in
    linear space (getSurfaceDataFromMat, bindless.glsl:199-203): half the materials of the 4096-triangle
    workload set to a black base colour, the traced rays and the atlas against the oracle."""
    w = scenes.CPU_REFERENCE
    arrays = scenes.build_scene(w)
    arrays.materials["baseColFac"][::2, :3] = 0.0
    atlas, want, stats = _run_lockstep(ctx, w, 3, arrays=arrays)
    for s in stats:
        assert s["hit_mismatch"] == 0, s
        assert s["ray_err_max"] <= (1e-4 if s["prev_equal"] else 1e-2), s
    err = rel_err(atlas, want, 1e-3)
    assert np.percentile(err, 99.9) <= 1e-3, np.percentile(err, [50, 99, 99.9, 100])
