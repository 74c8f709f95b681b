"""Known-answer tests of the FP64 oracle (CPU only). The reference ships no tests or golden data for this
path, so these pin the restatement's arithmetic to closed forms: the lattice, the translation map, the
convolution of constant radiance, the hysteresis recurrence and the watertight edge rule."""
import math

import numpy as np
import pytest

from anerend_gb300 import _lib as L
from anerend_gb300 import scenes
from oracle import oracle


def grid_desc(dims=(4, 2, 4), n=64, h=0.96, step=(1.0, 2.0, 1.0), origin_y=0.0, options=0):
    d = L.GridDesc()
    d.dims[:] = list(dims)
    d.step[:] = list(step)
    d.originY = origin_y
    d.raysPerProbe = n
    d.atlasFormat = L.DDGI_FORMAT_RGBA32F
    d.hysteresis = h
    d.options = options
    return d


@pytest.mark.parametrize("n", [16, 64, 128, 256, 512])
def test_lattice_unit_and_z_spacing(n):
    # worldDirFromFibonacciIndex (rgen:35-46): |d| = 1, z_i = cos(phi_i) = 1 - 2 (i + 0.5) / N
    d = oracle.lattice(n, np.eye(3, dtype=np.float32).reshape(-1))
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-14)
    z = 1.0 - 2.0 * (np.arange(n) + 0.5) / n
    assert np.allclose(d[:, 2], z, atol=1e-14)
    theta = 2.0 * 3.14159265359 * np.arange(n) / 1.6180339887
    assert np.allclose(np.arctan2(d[:, 1], d[:, 0]), np.angle(np.exp(1j * theta)), atol=1e-9)


def test_lattice_rotation_applied_column_major():
    rot = scenes.rotation(0, 3)
    R = rot.reshape(3, 3).T.astype(np.float64)  # column-major storage
    d0 = oracle.lattice(64, np.eye(3, dtype=np.float32).reshape(-1))
    d1 = oracle.lattice(64, rot)
    assert np.allclose(d1, d0 @ R.T, atol=1e-12)


def _region_translate(a, X, Z, Y, dx, dz):
    """Independent restatement of the vkCmdCopyImage regions (TranslationPass.cpp:122-168)."""
    out = a.copy()
    W, Hp = 10 * X, 10 * Z
    sx, sz = int(np.sign(dx)), int(np.sign(dz))
    for layer in range(Y):
        y0 = layer * Hp
        plane = a[y0:y0 + Hp].copy()
        if sx > 0:
            xs, xd = slice(10, W), slice(0, W - 10)
        elif sx < 0:
            xs, xd = slice(0, W - 10), slice(10, W)
        else:
            xs = xd = slice(0, W)
        if sz > 0:
            ys, yd = slice(10, Hp), slice(0, Hp - 10)
        elif sz < 0:
            ys, yd = slice(0, Hp - 10), slice(10, Hp)
        else:
            ys = yd = slice(0, Hp)
        out[y0:y0 + Hp][yd, xd] = plane[ys, xs]
    return out


@pytest.mark.parametrize("dx,dz", [(1, 0), (-1, 0), (0, 1), (0, -1), (1, 1), (-1, 1), (1, -1), (-1, -1), (3, 0), (0, -5), (2, 7)])
def test_translation_map(dx, dz):
    X, Y, Z = 4, 3, 4
    d = grid_desc((X, Y, Z))
    rng = np.random.default_rng(1)
    a = rng.standard_normal((10 * Z * Y, 10 * X, 4))
    got = oracle.translate(d, a, dx, dz)
    assert np.array_equal(got, _region_translate(a, X, Z, Y, dx, dz))
    # the shift is by the sign only (teleports lose alignment, TranslationPass.cpp:69-77)
    assert np.array_equal(got, oracle.translate(d, a, int(np.sign(dx)), int(np.sign(dz))))


def test_translation_identity_and_stale_edge():
    X, Y, Z = 3, 2, 3
    d = grid_desc((X, Y, Z))
    a = np.arange(10 * Z * Y * 10 * X * 4, dtype=np.float64).reshape(10 * Z * Y, 10 * X, 4)
    assert np.array_equal(oracle.translate(d, a, 0, 0), a)
    out = oracle.translate(d, a, 1, 0)
    # dx > 0: src x + 10 -> dst x; the last probe column keeps its stale texels
    assert np.array_equal(out[:, :10 * X - 10], a[:, 10:])
    assert np.array_equal(out[:, 10 * X - 10:], a[:, 10 * X - 10:])


def _conv_setup(n, L0):
    X, Y, Z = 2, 1, 2
    d = grid_desc((X, Y, Z), n=n, h=0.97)
    g = oracle.GridGeom(X, Y, Z, n)
    rh, rw = g.ray_hw
    rays = np.zeros((rh, rw, 4))
    rays[..., :3] = L0
    rays[..., 3] = 1.0
    ah, aw = g.atlas_hw
    atlas = np.zeros((ah, aw, 4))
    atlas[..., 3] = 1.0
    dirs = oracle.lattice(n, np.eye(3, dtype=np.float32).reshape(-1))
    return d, g, rays, atlas, dirs


@pytest.mark.parametrize("n", [64, 256])
def test_conv_constant_radiance_and_hysteresis(n):
    # constant radiance L: the normalised cosine sum is L for every texel; after k frames starting from
    # 0, the blend gives L * (1 - h^k)
    Lc = np.array([0.25, 1.5, 4.0])
    d, g, rays, atlas, dirs = _conv_setup(n, Lc)
    h = float(np.float32(0.97))  # the grid stores the hysteresis as a 32-bit float
    for k in range(1, 6):
        oracle.convolve(d, rays, dirs, atlas, 0, 1, 0)
        interior = atlas[1:9, 1:9, :3]
        assert np.allclose(interior, Lc * (1 - h ** k), rtol=1e-12)
    # borders are never written by the convolution
    assert np.all(atlas[0, :, :3] == 0.0) and np.all(atlas[0, :, 3] == 1.0)


def test_conv_weight_sum_in_alpha():
    # probe_conv.comp blends result.w = sum of cosine weights into .w: after one frame w = (1-h) s + h
    n = 256
    d, g, rays, atlas, dirs = _conv_setup(n, np.ones(3))
    oracle.convolve(d, rays, dirs, atlas, 0, 1, 0)
    t = 0
    for ty in range(8):
        for tx in range(8):
            u, v = (2 * tx + 1) / 16 * 2 - 1, (2 * ty + 1) / 16 * 2 - 1
            vz = 1 - abs(u) - abs(v)
            if vz < 0:
                u, v = (1 - abs(v)) * (1 if u >= 0 else -1), (1 - abs(u)) * (1 if v >= 0 else -1)
            om = np.array([u, vz, v]) / np.linalg.norm([u, vz, v])
            w = np.maximum(0.0, dirs @ om)
            s = w[w > 1e-6].sum()
            h = float(np.float32(0.97))
            assert math.isclose(atlas[1 + ty, 1 + tx, 3], (1 - h) * s + h, rel_tol=1e-12)
            t += 1
    assert t == 64


def test_bake_accumulation():
    # bake mode (probe_conv.comp:307-319): running weighted mean, weight accumulates in .w
    n = 64
    d, g, rays, atlas, dirs = _conv_setup(n, np.array([2.0, 2.0, 2.0]))
    atlas[..., 3] = 0.0
    oracle.convolve(d, rays, dirs, atlas, 0, 1, L.DDGI_UBO_BAKE_MODE_ON_FLAG)
    w1 = atlas[1:9, 1:9, 3].copy()
    assert np.all(w1 > 0)
    oracle.convolve(d, rays, dirs, atlas, 0, 1, L.DDGI_UBO_BAKE_MODE_ON_FLAG)
    assert np.allclose(atlas[1:9, 1:9, 3], 2 * w1)
    # the rgb is the raw weighted sum divided by the total weight: sum_j w_j L / sum_j w_j ... = L
    assert np.allclose(atlas[1:9, 1:9, :3], 2.0)


def _two_triangle_scene():
    # a quad at z = 5 split along its diagonal: triangles 0 and 1 share the edge (-1,-1,5)-(1,1,5)
    tris = np.array([[[-1, -1, 5], [1, -1, 5], [1, 1, 5]], [[-1, -1, 5], [1, 1, 5], [-1, 1, 5]]], np.float64)
    mats = scenes.random_materials(0, 2)
    return scenes.assemble(tris, np.array([0, 1]), np.array([0, 1]), mats)


def test_watertight_shared_edge_and_vertices():
    arrays = _two_triangle_scene()
    s = oracle.OracleScene(arrays, L.SceneDesc)
    try:
        # a ray through the shared edge hits both at the same t: the lower id wins, and it is uncertain
        gid, t, b, unc = s.closest_hit((0, 0, 0), (0.2, 0.2, 5.0) / np.linalg.norm((0.2, 0.2, 5.0)))
        assert gid == 0 and unc
        assert math.isclose(t, np.linalg.norm((0.2, 0.2, 5.0)), rel_tol=1e-12)
        # through the shared vertex (1,1,5): still a hit
        d = np.array([1.0, 1.0, 5.0])
        gid, t, b, unc = s.closest_hit((0, 0, 0), d / np.linalg.norm(d))
        assert gid in (0, 1) and unc
        # interior points: certain hits on the right triangle
        for p, want in [((0.5, -0.5, 5.0), 0), ((-0.5, 0.5, 5.0), 1)]:
            d = np.asarray(p) / np.linalg.norm(p)
            gid, t, b, unc = s.closest_hit((0, 0, 0), d)
            assert gid == want and not unc
        # outside the quad, and beyond tMax / inside tMin
        gid, *_ = s.closest_hit((0, 0, 0), (0.0, 0.6, 0.8))
        assert gid == -1
        gid, *_ = s.closest_hit((0, 0, -60), (0, 0, 1))
        assert gid == -1
        gid, *_ = s.closest_hit((0, 0, 4.95), (0, 0, 1))
        assert gid == -1
        # double-sided: from behind
        gid, t, b, unc = s.closest_hit((0.5, -0.5, 10.0), (0, 0, -1))
        assert gid == 0 and math.isclose(t, 5.0)
    finally:
        s.close()


def test_octant_fan_closed():
    # a closed octahedron around the origin: every lattice ray hits (no leaks through edges or vertices)
    v = np.array([[10, 0, 0], [-10, 0, 0], [0, 10, 0], [0, -10, 0], [0, 0, 10], [0, 0, -10]], np.float64)
    faces = [(0, 2, 4), (2, 1, 4), (1, 3, 4), (3, 0, 4), (2, 0, 5), (1, 2, 5), (3, 1, 5), (0, 3, 5)]
    tris = np.array([[v[a], v[b], v[c]] for a, b, c in faces])
    arrays = scenes.assemble(tris, np.arange(8), np.arange(8), scenes.random_materials(0, 8))
    s = oracle.OracleScene(arrays, L.SceneDesc)
    try:
        for n in (16, 64, 256):
            for d in oracle.lattice(n, np.eye(3, dtype=np.float32).reshape(-1)):
                gid, *_ = s.closest_hit((0, 0, 0), d)
                assert gid >= 0
    finally:
        s.close()


# ---- atlas consumer (deferred_tiled.comp:263-299) --------------------------------------------------

def _consumer_desc(dims=(8, 4, 8)):
    d = L.GridDesc()
    d.dims[:] = list(dims)
    d.step[:] = [1.0, 2.0, 1.0]
    d.raysPerProbe = 64
    d.hysteresis = 0.97
    return d


def _points(pos, normal, albedo=(0.5, 0.6, 0.7), metallic=0.0, roughness=0.5, shadow=1.0):
    p = np.zeros(len(pos), L.SURFACE_POINT)
    p["position"] = pos
    p["normal"] = normal
    p["albedo"] = albedo
    p["metallic"] = metallic
    p["roughness"] = roughness
    p["shadow"] = shadow
    return p


def _frame(flags, cam=(0.0, 0.0, 0.0), sky=1.0):
    f = L.Frame()
    f.cameraPos[:] = list(cam)
    f.flags = flags
    f.skyIntensity = sky
    return f


def test_consumer_constant_atlas_closed_form():
    """A constant atlas c: every probe sample is c, so sampleProbe = c * 0.5 * 3.1415926 and the ambient term is
    kD * (that * albedo) with kS = fresnelSchlickRoughness(max(n.V, 0), F0, roughness^2) (pbr_light.glsl)."""
    d = _consumer_desc()
    atlas = np.zeros((10 * 8 * 4, 10 * 8, 4))
    atlas[..., :3] = [0.2, 0.4, 0.8]
    cam = np.array([0.3, 1.0, -0.4])
    pos = np.array([[0.5, 1.7, 0.25], [-2.2, 3.1, 1.9]])
    nrm = np.array([[0.0, 1.0, 0.0], [1.0, 1.0, 0.0]])
    out = oracle.query_irradiance(d, _frame(L.DDGI_UBO_DDGI_FLAG, cam), atlas, _points(pos, nrm))
    albedo = np.array([0.5, 0.6, 0.7])
    for k in range(2):
        n = nrm[k] / np.linalg.norm(nrm[k])
        v = cam - pos[k]
        v /= np.linalg.norm(v)
        ndv = max(float(n @ v), 0.0)
        f0 = np.full(3, 0.04)
        ks = f0 + (np.maximum(1.0 - 0.25, f0) - f0) * (1.0 - ndv) ** 5
        want = (1.0 - ks) * (np.array([0.2, 0.4, 0.8]) * 0.5 * 3.1415926 * albedo)
        assert np.allclose(out[k], want, rtol=1e-6, atol=0)  # float32 inputs


def test_consumer_far_points_and_no_ddgi():
    d = _consumer_desc()
    atlas = np.ones((320, 80, 4))
    pts = _points(np.array([[10.0, 1.0, 0.0], [0.0, 1.0, 0.0]]), np.array([[0, 1, 0], [0, 1, 0]]), shadow=0.1)
    # beyond X * step.x / 2 = 4 from the camera: skyIntensity * 0.3 * albedo * clamp(shadow, 0.3, 1)
    far = oracle.query_irradiance(d, _frame(L.DDGI_UBO_DDGI_FLAG, sky=2.0), atlas, pts[:1])
    assert np.allclose(far[0], 2.0 * 0.3 * np.array([0.5, 0.6, 0.7]) * 0.3)
    off = oracle.query_irradiance(d, _frame(0), atlas, pts)
    assert np.allclose(off, 0.3 * np.array([0.5, 0.6, 0.7]) * 0.3)


def test_consumer_clamps_to_edge():
    """At the +x edge of the grid the +1 neighbour's texels lie past the atlas: the deferred pass's
    CLAMP_TO_EDGE sampler reads the last column (the trace pass would wrap to column 0)."""
    d = _consumer_desc()
    atlas = np.zeros((320, 80, 4))
    atlas[:, :40, :3] = 1.0   # left half bright: reached only by wrapping
    atlas[:, 40:, :3] = 0.25
    # a point in the last probe cell along x (camera at the origin: probes x = -4..3), normal +x
    pts = _points(np.array([[3.6, 1.0, 0.5]]), np.array([[1.0, 0.0, 0.0]]))
    out = oracle.query_irradiance(d, _frame(L.DDGI_UBO_DDGI_FLAG), atlas, pts)
    n = np.array([1.0, 0.0, 0.0])
    v = -np.array([3.6, 1.0, 0.5])
    v /= np.linalg.norm(v)
    ks = 0.04 + (np.maximum(0.75, 0.04) - 0.04) * (1.0 - max(float(n @ v), 0.0)) ** 5
    want = (1.0 - ks) * (0.25 * 0.5 * 3.1415926 * np.array([0.5, 0.6, 0.7]))
    assert np.allclose(out[0], want, rtol=1e-6)  # every sample from the dim right half


# ---- specular GI mirror pass (mirror_reflections.rgen/.rchit/.rmiss) ---------------------------------------

def _mirror_world():
    """A floor (y = 0), an emissive wall at z = 3 facing +z and a small occluder above the wall at y = 5."""
    floor = scenes.floor_quad(0.0, 4.0)
    wall = np.array([[[-2, 0, 3], [2, 0, 3], [2, 6, 3]], [[-2, 0, 3], [2, 6, 3], [-2, 6, 3]]], np.float64)
    occ = np.array([[[-1, 5, 2.5], [1, 5, 2.5], [1, 5, 3.5]], [[-1, 5, 2.5], [1, 5, 3.5], [-1, 5, 3.5]]], np.float64)
    tris = np.concatenate([floor, wall, occ])
    mats = scenes.random_materials(0, 3)
    mats["baseColFac"] = [[0.3, 0.3, 0.3, 1.0], [0.5, 0.6, 0.7, 1.0], [0.2, 0.2, 0.2, 1.0]]
    mats["metRough"][:, :2] = [[0.0, 0.5], [0.0, 0.5], [0.0, 0.5]]
    mats["emissive"] = [[0, 0, 0, 0], [1.0, 2.0, 3.0, 1.0], [0, 0, 0, 0]]
    return scenes.assemble(tris, np.array([0, 0, 1, 1, 2, 2]), np.arange(3), mats)


def _mirror_points():
    p = np.zeros(3, L.MIRROR_POINT)
    p["position"] = [[0.5, 0.0, 0.0], [0.5, 1.0, -6.0], [1.0, 1.0, 1.0]]
    p["normal"] = [[0.0, 1.0, 0.0], [0.0, 1.0, 0.0], [0.0, 1.0, 0.0]]
    p["sky"] = [0.0, 0.0, 1.0]
    return p


def _mirror_frame(flags, sun=3.0):
    f = L.Frame()
    f.cameraPos[:] = [0.5, 2.0, -2.0]
    f.lightDir[:] = [0.0, -1.0, 0.0]
    f.sunIntensity = sun
    f.skyColor[:] = [0.4, 0.5, 0.7]
    f.skyIntensity = 1.0
    f.flags = flags
    return f


def test_mirror_shadowed_emitter_miss_and_sky():
    """From (0.5,0,0) with normal +y and the camera at (0.5,2,-2) the reflected ray runs along (0,1,1)/sqrt2 to
    the wall at (0.5,3,3), distance 3 sqrt2, away from the edges of both walls' triangles; the occluder shadows
    that point and without DDGI the radiance is the
    wall's emission. The second point reflects into the empty sky: linear sky, 1e6; the sky pixel gets 0."""
    arrays = _mirror_world()
    s = oracle.OracleScene(arrays, L.SceneDesc)
    try:
        out, unc = oracle.mirror_reflections(s, grid_desc(), _mirror_frame(0), np.zeros((80, 40, 4)), _mirror_points())
    finally:
        s.close()
    assert np.all(unc == 0)
    assert np.allclose(out[0], [1.0, 2.0, 3.0, 3.0 * math.sqrt(2.0)], rtol=1e-12)
    c = np.array([0.4, 0.5, 0.7])
    sky = np.where(c < 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4)  # toLinear (bindless.glsl:240-247)
    assert np.allclose(out[1], [*sky, 1e6], rtol=1e-7)
    assert np.array_equal(out[2], np.zeros(4))


@pytest.mark.parametrize("flags,indirect", [(L.DDGI_UBO_DDGI_FLAG, True), (L.DDGI_UBO_DDGI_MULTI_FLAG, False)])
def test_mirror_indirect_term_gated_by_ddgi_flag(flags, indirect):
    """With the sun off, a constant atlas c gives the wall hit L = kD (c 0.5 3.1415926 albedo) + emission, kD =
    1 - kS with kS = F0 + (max(1 - r^2, F0) - F0) (1 - max(n.v, 0))^5 = 0.75 (the wall's normal +z points away
    from the viewer, n.v < 0); the mirror pass gates it on UBO_DDGI_FLAG (rchit:106), not the multi flag."""
    arrays = _mirror_world()
    atlas = np.zeros((80, 40, 4))
    atlas[..., :3] = [0.2, 0.4, 0.8]
    s = oracle.OracleScene(arrays, L.SceneDesc)
    try:
        out, unc = oracle.mirror_reflections(s, grid_desc(), _mirror_frame(flags, sun=0.0), atlas, _mirror_points()[:1])
    finally:
        s.close()
    assert unc[0] == 0
    want = np.array([1.0, 2.0, 3.0])
    if indirect:
        want = want + 0.25 * (np.array([0.2, 0.4, 0.8]) * 0.5 * 3.1415926 * np.array([0.5, 0.6, 0.7]))
    assert np.allclose(out[0, :3], want, rtol=1e-6)  # float32 material inputs


def test_rgba16f_ray_image_store_rounds_to_half():
    # DDGI_GRID_RAYS_RGBA16F: every stored ray radiance is the binary16 value nearest to the FP32 value (the
    # store into the reference's R16G16B16A16_SFLOAT ray image, rgen:108-109); everything else is unchanged
    w = scenes.CPU_REFERENCE
    arrays = scenes.build_scene(w)
    s = oracle.OracleScene(arrays, L.SceneDesc)
    try:
        outs = []
        for opts in (0, L.DDGI_GRID_RAYS_RGBA16F):
            d = grid_desc(w.dims, w.rays, 0.97, w.step, w.origin_y, options=opts)
            g = oracle.OracleGrid(d)
            fp = L.Frame()
            fp.lightDir[:] = list(np.array(w.light_dir) / np.linalg.norm(w.light_dir))
            fp.sunIntensity, fp.skyIntensity = w.sun, w.sky_intensity
            fp.skyColor[:] = list(w.sky)
            fp.flags = L.DDGI_UBO_DDGI_FLAG | L.DDGI_UBO_DDGI_MULTI_FLAG
            fp.rotation[:] = scenes.rotation(w.seed, 0).tolist()
            fp.layer = -1
            g.trace(s, fp)
            outs.append((g.ray_rad.copy(), g.hits.copy()))
        (full, hits0), (half, hits1) = outs
        assert np.array_equal(hits0, hits1)
        want = full[..., :3].astype(np.float32).astype(np.float16).astype(np.float64)
        assert np.array_equal(half[..., :3], want)
        assert np.array_equal(half[..., 3], full[..., 3])
        assert not np.array_equal(half, full)
    finally:
        s.close()
