"""ORACLE — test infrastructure only. The seeded inputs on which the oracle restatement is compared with the
reference's shader code compiled as FP64 C++: the reference's own grid constants (64 x 8 x 64 probes,
256 rays, step (1, 2, 1), hysteresis 0.96), a 3,000-triangle scene with a floor in 24 meshes and 25
materials (the reference packs material and mesh into 10 + 14 bits of the instance custom index), a
previous atlas of seeded values, two frames (camera-relative, and bake mode on a tile), and the pixel and
invocation rectangles compared. Every value comes from the counter-based generator of
anerend_gb300.scenes, so the fixtures regenerate bit for bit."""
from __future__ import annotations

import numpy as np

from anerend_gb300 import _lib as L
from anerend_gb300 import scenes
from anerend_gb300.ddgi import FrameParams

DIMS = (64, 8, 64)
STEP = (1.0, 2.0, 1.0)
RAYS = 256
HYSTERESIS = 0.96
SEED = 7

# ray-image pixels [x0, x1) x [y0, y1) of the traced layer: 3 x 2 interior probes, and the 2 x 2 probes at
# the +x / +z corner of the grid (their probe lookups reach the wrapped +1 neighbours); 16 x 16 rays each
TRACE_RECTS = [(16 * 20, 16 * 30, 16 * 23, 16 * 32), (16 * 62, 16 * 62, 16 * 64, 16 * 64)]
# convolution invocations of the same probes (8 x 8 texels each)
CONV_RECTS = [(8 * 20, 8 * 30, 8 * 23, 8 * 32), (8 * 62, 8 * 62, 8 * 64, 8 * 64)]


def scene_arrays() -> scenes.Scene:
    n = 3000
    tris = scenes.random_triangles(SEED, n, (-30.0, 0.0, -30.0), (30.0, 15.0, 30.0))
    tris = np.concatenate([tris, scenes.floor_quad(-0.5, 40.0)])
    tri_mesh = np.concatenate([np.arange(n) // 125, [24, 24]])
    mesh_material = np.arange(25) % 25
    return scenes.assemble(tris, tri_mesh, mesh_material, scenes.random_materials(SEED, 25))


def scene_desc(arrays) -> L.SceneDesc:
    a = arrays
    return L.SceneDesc(a.vertices.ctypes.data, len(a.vertices), a.indices.ctypes.data, len(a.indices),
                       a.meshes.ctypes.data, len(a.meshes), a.instances.ctypes.data, len(a.instances),
                       a.materials.ctypes.data, len(a.materials))


def grid_desc() -> L.GridDesc:
    d = L.GridDesc()
    d.dims[:] = list(DIMS)
    d.step[:] = list(STEP)
    d.originY = 0.0
    d.raysPerProbe = RAYS
    d.atlasFormat = L.DDGI_FORMAT_RGBA32F
    d.hysteresis = HYSTERESIS
    return d


def atlas_prev() -> np.ndarray:
    """Previous atlas (5120 x 640 RGBA, FP64): seeded values in [0, 2), .w in [0, 1)."""
    h, w = 10 * DIMS[2] * DIMS[1], 10 * DIMS[0]
    v = np.stack([scenes.uniform(SEED, 300 + c, h * w) for c in range(4)], 1).reshape(h, w, 4)
    v[..., :3] *= 2.0
    return np.ascontiguousarray(v, np.float64)


def frames():
    """(name, FrameParams, layer) of the compared frames."""
    base = dict(camera_pos=(3.7, 1.3, -2.6), light_dir=(-0.3, -1.0, -0.2), sun_intensity=3.0,
                sky_color=(0.4, 0.5, 0.7), sky_intensity=1.0, rotation=scenes.rotation(SEED, 3))
    normal = FrameParams(flags=L.DDGI_UBO_DDGI_FLAG | L.DDGI_UBO_DDGI_MULTI_FLAG, layer=3, **base)
    bake = FrameParams(flags=L.DDGI_UBO_DDGI_FLAG | L.DDGI_UBO_DDGI_MULTI_FLAG | L.DDGI_UBO_BAKE_MODE_ON_FLAG,
                       layer=2, bake_tile=(0, -1, 32), **base)
    return [("camera_relative", normal, 3), ("bake_tile", bake, 2)]


def conv_inputs(rotation):
    """One layer's ray images for the convolution: radiance seeded in [0, 4), directions = the rotated
    lattice repeated in every probe's 16 x 16 block (what the ray-generation stage stores)."""
    from oracle import oracle

    dirs = oracle.lattice(RAYS, np.asarray(rotation, np.float32))
    irr = np.stack([4.0 * scenes.uniform(SEED, 400 + c, 1024 * 1024) for c in range(3)], 1)
    irr = np.concatenate([irr, np.ones((1024 * 1024, 1))], 1).reshape(1024, 1024, 4)
    block = np.concatenate([dirs, np.ones((RAYS, 1))], 1).reshape(16, 16, 4)
    dir_img = np.tile(block, (64, 64, 1))
    return np.ascontiguousarray(irr), np.ascontiguousarray(dir_img), dirs


def _points_on_triangles(arrays, n: int, stream: int) -> np.ndarray:
    """n seeded points on the scene's triangles (FP64)."""
    v = arrays.vertices["d0"][:, :3].astype(np.float64)
    tri = arrays.indices.reshape(-1, 3)
    u = [scenes.uniform(SEED, stream + k, n) for k in range(3)]
    k = (u[0] * len(tri)).astype(np.int64) % len(tri)
    a, b = u[1].copy(), u[2].copy()
    flip = a + b > 1
    a[flip], b[flip] = 1 - a[flip], 1 - b[flip]
    return v[tri[k, 0]] * (1 - a - b)[:, None] + v[tri[k, 1]] * a[:, None] + v[tri[k, 2]] * b[:, None]


def _unit(n: int, stream: int) -> np.ndarray:
    z = 2.0 * scenes.uniform(SEED, stream, n) - 1.0
    phi = 2.0 * np.pi * scenes.uniform(SEED, stream + 1, n)
    r = np.sqrt(1.0 - z * z)
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], 1)


def mirror_points(arrays, n: int = 400) -> np.ndarray:
    """MIRROR_POINT records for the specular GI pass: points on the scene's triangles with seeded normals
    (not unit length), every 13th a sky pixel."""
    pts = np.zeros(n, dtype=L.MIRROR_POINT)
    pts["position"] = _points_on_triangles(arrays, n, 500)
    pts["normal"] = _unit(n, 510) * (0.5 + scenes.uniform(SEED, 512, n))[:, None]
    pts["sky"][::13] = 1.0
    return pts


def shadow_points(arrays, n: int = 400) -> np.ndarray:
    """float32 (x, y, z, sky) points for the RT shadow pass: on the scene's triangles, every 11th a sky pixel."""
    pts = np.zeros((n, 4), np.float32)
    pts[:, :3] = _points_on_triangles(arrays, n, 520)
    pts[::11, 3] = 1.0
    return pts


def surface_points(n: int = 400) -> np.ndarray:
    """SURFACE_POINT records for the deferred pass's DDGI block: positions in the scene's box (some beyond
    NUM_PROBES_PER_PLANE * PROBE_STEP.x / 2 = 32 of the camera), seeded normals, materials and shadows."""
    pts = np.zeros(n, dtype=L.SURFACE_POINT)
    lo, hi = np.array([-30.0, 0.0, -30.0]), np.array([30.0, 15.0, 30.0])
    pts["position"] = lo + (hi - lo) * np.stack([scenes.uniform(SEED, 530 + k, n) for k in range(3)], 1)
    pts["normal"] = _unit(n, 540) * (0.5 + scenes.uniform(SEED, 542, n))[:, None]
    pts["albedo"] = np.stack([scenes.uniform(SEED, 550 + k, n) for k in range(3)], 1)
    pts["metallic"] = (scenes.uniform(SEED, 553, n) < 0.3).astype(np.float32)
    pts["roughness"] = 0.1 + 0.9 * scenes.uniform(SEED, 554, n)
    pts["shadow"] = np.floor(3.0 * scenes.uniform(SEED, 555, n)) / 2.0  # 0, 0.5 or 1
    return pts


def pass_frames():
    """(name, FrameParams) of the G-buffer passes: the DDGI flag on and off."""
    base = dict(camera_pos=(3.7, 1.3, -2.6), light_dir=(-0.3, -1.0, -0.2), sun_intensity=3.0,
                sky_color=(0.4, 0.5, 0.7), sky_intensity=1.0)
    return [("ddgi_on", FrameParams(flags=L.DDGI_UBO_DDGI_FLAG, **base)), ("ddgi_off", FrameParams(flags=0, **base))]
