"""ddgi_convolve_raw_noalloc: the probe convolution for callers that cannot allocate device memory during
a frame (renderers that reserve all device memory before the frame loop, processes whose device memory is
committed to a budget). It keeps its weight scratch in a static device array instead of allocating, so its
output must equal the allocating ddgi_convolve_raw on the same inputs, call after call, even though every
call reuses the array the previous call left behind. This file runs last (its name sorts last) and also
passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from anerend_gb300 import _lib as L
from anerend_gb300 import scenes

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

# Both entry points run the same weights and convolution kernels in the same order on the same inputs, so
# their atlases must agree bit for bit; only where the weight scratch lives differs.


def _desc(dims, n, h):
    d = L.GridDesc()
    d.dims[:] = list(dims)
    d.step[:] = [1.0, 2.0, 1.0]
    d.originY = 0.0
    d.raysPerProbe = n
    d.atlasFormat = L.DDGI_FORMAT_RGBA32F
    d.hysteresis = h
    d.options = 0
    return d


def _inputs(dims, n, seed):
    X, Y, Z = dims
    lg = (n - 1).bit_length()
    bw = 1 << ((lg + 1) // 2)
    bh = n // bw
    rng = np.random.default_rng(seed)
    rays = np.exp(rng.uniform(np.log(1e-3), np.log(1e2), size=(bh * Z * Y, bw * X, 4))).astype(np.float32)
    atlas = rng.uniform(0.0, 3.0, size=(10 * Z * Y, 10 * X, 4)).astype(np.float32)
    return rays, atlas


def _lattice(lib, n, seed, stream):
    rot = scenes.rotation(seed, n)
    dirs = torch.empty(n * 4, dtype=torch.float32, device="cuda")
    assert lib.ddgi_fibonacci_lattice(n, (C.c_float * 9)(*rot.tolist()), dirs.data_ptr(), stream) == L.DDGI_OK
    return dirs


def test_noalloc_convolve_matches_allocating_entry_point_twice():
    lib = L.load()
    stream = torch.cuda.current_stream().cuda_stream
    # calls in a row with different sizes, layers and modes, each reusing the static scratch the previous one
    # left behind: the largest size the scratch holds (its weight table full, the sums right after it), then
    # smaller ones
    cases = [((3, 2, 2), L.DDGI_NOALLOC_MAX_RAYS, 0.97, 0, 2, 0),
             ((5, 3, 3), 256, 0.97, 0, 3, 0),
             ((4, 2, 6), 64, 0.96, 1, 2, L.DDGI_UBO_BAKE_MODE_ON_FLAG)]
    for i, (dims, n, h, b, e, flags) in enumerate(cases):
        d = _desc(dims, n, h)
        rays, atlas = _inputs(dims, n, 100 + i)
        dirs = _lattice(lib, n, i, stream)
        r_dev = torch.from_numpy(rays).cuda()
        ref = torch.from_numpy(atlas).cuda()
        got = ref.clone()
        assert lib.ddgi_convolve_raw(C.byref(d), r_dev.data_ptr(), dirs.data_ptr(), ref.data_ptr(), b, e, flags,
                                     stream) == L.DDGI_OK
        assert lib.ddgi_convolve_raw_noalloc(C.byref(d), r_dev.data_ptr(), dirs.data_ptr(), got.data_ptr(), b, e,
                                             flags, stream) == L.DDGI_OK
        torch.cuda.synchronize()
        want = ref.cpu().numpy()
        have = got.cpu().numpy()
        assert np.array_equal(have.view(np.uint32), want.view(np.uint32)), (i, n)
        assert not np.array_equal(have, atlas)  # the call did update the atlas


def test_noalloc_rejects_what_the_allocating_entry_point_rejects():
    lib = L.load()
    stream = torch.cuda.current_stream().cuda_stream
    dims, n = (2, 1, 2), 64
    rays, atlas = _inputs(dims, n, 9)
    dirs = _lattice(lib, n, 4, stream)
    r_dev = torch.from_numpy(rays).cuda()
    a_dev = torch.from_numpy(atlas).cuda()
    bad = []
    d = _desc(dims, n, 0.97)
    d.step[1] = float("inf")
    bad.append(d)
    d = _desc(dims, n, 0.97)
    d.options = 1 << 7  # not a DDGI_GRID_* bit
    bad.append(d)
    d = _desc(dims, 48, 0.97)  # not a power of two
    bad.append(d)
    for d in bad:
        for fn in (lib.ddgi_convolve_raw, lib.ddgi_convolve_raw_noalloc):
            assert fn(C.byref(d), r_dev.data_ptr(), dirs.data_ptr(), a_dev.data_ptr(), 0, 1, 0, stream) == L.DDGI_EINVAL
    torch.cuda.synchronize()
    assert np.array_equal(a_dev.cpu().numpy(), atlas)


def test_noalloc_rejects_more_rays_than_its_scratch_holds():
    lib = L.load()
    stream = torch.cuda.current_stream().cuda_stream
    n = 2 * L.DDGI_NOALLOC_MAX_RAYS
    dims = (2, 1, 2)
    d = _desc(dims, n, 0.97)
    rays, atlas = _inputs(dims, n, 7)
    dirs = _lattice(lib, n, 3, stream)
    r_dev = torch.from_numpy(rays).cuda()
    a_dev = torch.from_numpy(atlas).cuda()
    rc = lib.ddgi_convolve_raw_noalloc(C.byref(d), r_dev.data_ptr(), dirs.data_ptr(), a_dev.data_ptr(), 0, 1, 0,
                                       stream)
    assert rc == L.DDGI_EINVAL
    torch.cuda.synchronize()
    assert np.array_equal(a_dev.cpu().numpy(), atlas)
