"""Atlas consumer on the GPU (ddgi_query_irradiance: the DDGI block of deferred_tiled.comp:263-299 with the
CLAMP_TO_EDGE sampler) against the FP64 oracle on the same atlas.

Tolerance: ambient term within 1e-4 relative per channel (absolute floor 1e-6); the kernel is FP32 and the
oracle FP64 on identical inputs."""
import numpy as np
import pytest

from anerend_gb300 import _lib as L
from anerend_gb300 import ddgi, scenes
from oracle import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _random_points(n, seed):
    u = [scenes.uniform(seed, 900 + k, n) for k in range(14)]
    p = np.zeros(n, L.SURFACE_POINT)
    # most points inside the grid's reach, some beyond X * step.x / 2 (sky term), some at its edges
    p["position"] = np.stack([u[0] * 14 - 7, u[1] * 9 - 1, u[2] * 14 - 7], 1)
    nrm = np.stack([u[3] * 2 - 1, u[4] * 2 - 1, u[5] * 2 - 1], 1)
    p["normal"] = nrm * (0.5 + u[6][:, None])  # not unit length: the kernel normalises, as the shader does
    p["albedo"] = np.stack([u[7], u[8], u[9]], 1)
    p["metallic"] = (u[10] < 0.2).astype(np.float32)
    p["roughness"] = 0.1 + 0.9 * u[11]
    p["shadow"] = u[12]
    return p


@pytest.mark.parametrize("flags", [L.DDGI_UBO_DDGI_FLAG | L.DDGI_UBO_DDGI_MULTI_FLAG, L.DDGI_UBO_DDGI_MULTI_FLAG])
def test_query_irradiance_matches_oracle(ctx, flags):
    w = scenes.CPU_REFERENCE
    scene = ddgi.Scene(ctx, scenes.build_scene(w))
    grid = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis)
    try:
        for f in range(3):  # a non-trivial atlas
            grid.update(scene, ddgi.FrameParams(camera_pos=scenes.camera(w, f), rotation=scenes.rotation(w.seed, f)))
        cam = (0.7, 1.2, -0.3)
        fp = ddgi.FrameParams(camera_pos=cam, flags=flags)
        pts = _random_points(20000, 3)
        dp = torch.from_numpy(pts.view(np.uint8).copy()).cuda()
        out = torch.empty((len(pts), 4), dtype=torch.float32, device="cuda")
        grid.query_irradiance(fp, dp.data_ptr(), len(pts), out.data_ptr(), torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        atlas = grid.download_atlas().astype(np.float64)
        want = oracle.query_irradiance(grid.desc, fp.to_c(), atlas, pts)
        err = np.abs(got[:, :3] - want) / np.maximum(np.abs(want), 1e-6)
        assert err.max() <= 1e-4, (err.max(), np.argmax(err.max(1)))
        assert np.all(got[:, 3] == 0.0)
        # the workload reaches both branches of the block
        d = np.linalg.norm(pts["position"] - np.array(cam, np.float32), axis=1)
        far = d > w.dims[0] * w.step[0] / 2
        assert 0.05 < far.mean() < 0.95
    finally:
        grid.close()
        scene.close()


def test_query_irradiance_argument_errors(ctx):
    grid = ddgi.ProbeGrid(ctx, (4, 2, 4), (1.0, 1.0, 1.0), 64, 0.0, 0.97)
    try:
        assert grid.ctx.lib.ddgi_query_irradiance(grid.handle, None, 0, 1, 0, 0) == L.DDGI_EINVAL
        f = ddgi.FrameParams().to_c()
        import ctypes as C

        assert grid.ctx.lib.ddgi_query_irradiance(grid.handle, C.byref(f), 0, 1, 0, 0) == L.DDGI_EINVAL
        assert grid.ctx.lib.ddgi_query_irradiance(grid.handle, C.byref(f), 0, 0, 0, 0) == L.DDGI_OK
    finally:
        grid.close()
