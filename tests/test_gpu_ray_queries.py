"""Ray queries on a scene (ddgi_trace_rays) and the RT shadow pass (ddgi_shadow_mask, shadow.rgen:29-82)
against the FP64 oracle's closest hit.

Tolerances: the hit triangle (global id) and the hit / miss decision bit-exact on every ray the oracle marks
certain; t within 1e-5 relative; barycentrics within 1e-4 absolute."""
import numpy as np
import pytest

from anerend_gb300 import _lib as L
from anerend_gb300 import ddgi, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _oracle_hits(osc, origins, dirs):
    out = []
    for o, d in zip(origins, dirs):
        out.append(osc.closest_hit(o.astype(np.float64), d.astype(np.float64)))
    return out


@pytest.fixture(scope="module")
def world(ctx):
    w = scenes.CPU_REFERENCE
    arrays = scenes.build_scene(w)
    scene = ddgi.Scene(ctx, arrays)
    osc = oracle.OracleScene(arrays, L.SceneDesc)
    yield w, arrays, scene, osc
    osc.close()
    scene.close()


@pytest.mark.parametrize("any_hit", [False, True])
def test_trace_rays_match_oracle(world, any_hit):
    w, arrays, scene, osc = world
    n = 6000
    u = [scenes.uniform(5, 700 + k, n) for k in range(5)]
    origins = np.stack([u[0] * 16 - 8, u[1] * 16 - 8, u[2] * 16 - 8], 1).astype(np.float32)
    z = u[3] * 2 - 1
    ph = u[4] * 2 * np.pi
    s = np.sqrt(1 - z * z)
    dirs = np.stack([s * np.cos(ph), s * np.sin(ph), z], 1).astype(np.float32)
    rays = np.zeros(n, L.RAY)
    rays["origin"], rays["direction"], rays["tmin"], rays["tmax"] = origins, dirs, 0.1, 50.0
    dr = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    dh = torch.empty(n * 16, dtype=torch.uint8, device="cuda")
    scene.trace_rays(dr.data_ptr(), n, dh.data_ptr(), any_hit=any_hit, stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    hits = dh.cpu().numpy().view(L.HIT)
    want = _oracle_hits(osc, origins, dirs)
    certain = np.array([not u_ for (_, _, _, u_) in want])
    gid = np.array([g for (g, _, _, _) in want])
    assert certain.mean() > 0.99
    assert np.array_equal(hits["triangle"][certain] >= 0, gid[certain] >= 0)
    assert 0.2 < (gid >= 0).mean() < 0.95
    if not any_hit:
        assert np.array_equal(hits["triangle"][certain], gid[certain])
        sel = certain & (gid >= 0)
        t = np.array([t_ for (_, t_, _, _) in want])
        b = np.array([b_ for (_, _, b_, _) in want])
        assert np.max(np.abs(hits["t"][sel] - t[sel]) / t[sel]) <= 1e-5
        assert np.max(np.abs(hits["b1"][sel] - b[sel, 0])) <= 1e-4
        assert np.max(np.abs(hits["b2"][sel] - b[sel, 1])) <= 1e-4
    else:
        sel = certain & (gid >= 0)
        assert np.all((hits["t"][sel] >= 0.1) & (hits["t"][sel] <= 50.0))


def test_shadow_mask_matches_oracle(world):
    w, arrays, scene, osc = world
    # points on the scene's triangles (what a G-buffer holds), plus sky pixels
    v = arrays.vertices["d0"][:, :3]
    tri = arrays.indices.reshape(-1, 3)
    n = 5000
    u = [scenes.uniform(9, 800 + k, n) for k in range(3)]
    k = (u[0] * len(tri)).astype(np.int64) % len(tri)
    a, b = u[1], u[2]
    flip = a + b > 1
    a[flip], b[flip] = 1 - a[flip], 1 - b[flip]
    p = v[tri[k, 0]] * (1 - a - b)[:, None] + v[tri[k, 1]] * a[:, None] + v[tri[k, 2]] * b[:, None]
    pts = np.zeros((n, 4), np.float32)
    pts[:, :3] = p
    pts[::17, 3] = 1.0  # sky pixels
    fp = ddgi.FrameParams(light_dir=(-0.3, -1.0, -0.2))
    f = fp.to_c()
    dp = torch.from_numpy(pts).cuda()
    vis = torch.empty(n, dtype=torch.float32, device="cuda")
    scene.shadow_mask(fp, dp.data_ptr(), n, vis.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = vis.cpu().numpy()
    d = -np.array(f.lightDir[:], np.float32)
    want = _oracle_hits(osc, pts[:, :3], np.repeat(d[None], n, 0))
    certain = np.array([not u_ for (_, _, _, u_) in want])
    lit = np.array([g < 0 for (g, _, _, _) in want]).astype(np.float32)
    sky = pts[:, 3] != 0
    assert np.all(got[sky] == 1.0)
    sel = certain & ~sky
    assert sel.mean() > 0.9
    assert np.array_equal(got[sel], lit[sel])
    assert 0.1 < got[sel].mean() < 0.9
