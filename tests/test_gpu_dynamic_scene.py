"""Dynamic scenes (ddgi_scene_update_transforms / _update_vertices): after moving instances or vertices, with
the BVHs refitted or rebuilt, a trace gives the same rays bit for bit as a scene created from scratch with the
new data (closest hits do not depend on the tree, and the triangle records are transformed by the same
arithmetic), including the light-space shadow BVH built before the update; and the hits agree with the FP64
oracle on the moved scene (every certain ray)."""
import math

import numpy as np
import pytest

from anerend_gb300 import _lib as L
from anerend_gb300 import ddgi, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

DIMS, STEP, RAYS = (8, 3, 8), (1.5, 2.0, 1.5), 128


def _arrays(seed=4):
    n = 3000
    tris = scenes.random_triangles(seed, n, (-9.0, -2.0, -9.0), (9.0, 5.0, 9.0))
    tris = np.concatenate([tris, scenes.floor_quad(-2.5, 12.0)])
    tri_mesh = np.concatenate([np.arange(n) // 250, [12, 12]])
    return scenes.assemble(tris, tri_mesh, np.arange(13), scenes.random_materials(seed, 13))


def _motion(count, frame):
    """Rigid motions: a rotation about y and a translation, different per instance and frame."""
    out = np.zeros((count, 3, 4), np.float32)
    for i in range(count):
        a = 0.07 * (i + 1) * (frame + 1)
        c, s = math.cos(a), math.sin(a)
        out[i, :, :3] = [[c, 0, s], [0, 1, 0], [-s, 0, c]]
        out[i, :, 3] = [0.3 * math.sin(i + frame), 0.1 * frame, 0.25 * math.cos(i - frame)]
    out[-1] = np.eye(3, 4)  # the floor stays
    return out


def _trace(ctx, scene, frame, shadow_mode):
    g = ddgi.ProbeGrid(ctx, DIMS, STEP, RAYS, -1.0, 0.97, options=L.DDGI_GRID_RECORD_HITS)
    try:
        g.set_tuning(shadow_mode=shadow_mode)
        g.trace(scene, frame)
        ctx.sync()
        rad, hits, _ = g.download_rays(hits=True)
        return rad, hits, g.desc
    finally:
        g.close()


def _frame(k):
    return ddgi.FrameParams(camera_pos=(0.4, 1.0, -0.3), rotation=scenes.rotation(11, k), layer=-1)


@pytest.mark.parametrize("rebuild", [False, True])
@pytest.mark.parametrize("shadow_mode", [1, 0])
def test_moved_instances_equal_fresh_scene(ctx, rebuild, shadow_mode):
    arrays = _arrays()
    scene = ddgi.Scene(ctx, arrays)
    try:
        _trace(ctx, scene, _frame(0), shadow_mode)  # builds the light-space shadow BVH before the update
        for step in range(3):  # several updates in a row, as frames of an animation
            T = _motion(len(arrays.instances), step)
            scene.update_transforms(T, rebuild=rebuild)
        moved = scenes.Scene(arrays.vertices, arrays.indices, arrays.meshes, arrays.instances.copy(), arrays.materials)
        moved.instances["transform"] = T.reshape(-1, 12)
        fresh = ddgi.Scene(ctx, moved)
        try:
            ra, ha, desc = _trace(ctx, scene, _frame(1), shadow_mode)
            rb, hb, _ = _trace(ctx, fresh, _frame(1), shadow_mode)
            assert np.array_equal(ha, hb)
            assert np.array_equal(ra.view(np.uint32), rb.view(np.uint32))
            assert 0.2 < (ha >= 0).mean() < 0.98
            # against the oracle on the moved scene
            osc = oracle.OracleScene(moved, L.SceneDesc)
            try:
                og = oracle.OracleGrid(desc)
                og.trace(osc, _frame(1).to_c())
                certain = og.uncertain == 0
                assert certain.mean() > 0.99
                assert np.array_equal(ha[certain], og.hits[certain])
            finally:
                osc.close()
        finally:
            fresh.close()
    finally:
        scene.close()


def test_moved_vertices_equal_fresh_scene(ctx):
    arrays = _arrays(5)
    scene = ddgi.Scene(ctx, arrays)
    try:
        _trace(ctx, scene, _frame(0), 1)
        verts = arrays.vertices.copy()
        # a skinning-like displacement of the first 1,500 vertices (a mesh range), normals unchanged
        k = np.arange(1500)
        verts["d0"][k, 0] += 0.2 * np.sin(0.05 * k)
        verts["d0"][k, 1] += 0.1 * np.cos(0.03 * k)
        scene.update_vertices(verts[:1500], first=0)
        moved = scenes.Scene(verts, arrays.indices, arrays.meshes, arrays.instances, arrays.materials)
        fresh = ddgi.Scene(ctx, moved)
        try:
            ra, ha, _ = _trace(ctx, scene, _frame(2), 1)
            rb, hb, _ = _trace(ctx, fresh, _frame(2), 1)
            assert np.array_equal(ha, hb)
            assert np.array_equal(ra.view(np.uint32), rb.view(np.uint32))
        finally:
            fresh.close()
    finally:
        scene.close()


def test_update_argument_errors(ctx):
    arrays = _arrays(6)
    scene = ddgi.Scene(ctx, arrays)
    try:
        with pytest.raises(L.DdgiError):
            scene.update_transforms(np.zeros((3, 3, 4), np.float32))  # wrong instance count
        T = _motion(len(arrays.instances), 0)
        T[2, :, :3] = 0.0  # singular
        with pytest.raises(L.DdgiError):
            scene.update_transforms(T)
        with pytest.raises(L.DdgiError):
            scene.update_vertices(arrays.vertices[:10], first=len(arrays.vertices) - 5)
    finally:
        scene.close()
