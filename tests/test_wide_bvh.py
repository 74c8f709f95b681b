"""CPU checks of the 8-wide BVH collapse (FP32 and quantized node layouts) and of the binary and wide
traversals (host build of the same header the trace kernel uses): closest hits equal a brute-force loop over all triangles bit for bit,
including exact-duplicate triangles (t ties broken by the lowest global id), zero-area triangles,
axis-aligned rays with signed zero components and rays aimed at vertices and edges."""
import ctypes
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "native" / "wbvh_check.cpp"


def _cuda_include():
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "include" / "cuda_runtime.h").exists():
            return str(Path(cand) / "include")
    nvcc = shutil.which("nvcc")
    if nvcc:
        inc = Path(nvcc).resolve().parent.parent / "include"
        if (inc / "cuda_runtime.h").exists():
            return str(inc)
    return None


@pytest.fixture(scope="module", params=[0, 1], ids=["fp32-nodes", "quantized-nodes"])
def lib(request, tmp_path_factory):
    inc = _cuda_include()
    if inc is None or shutil.which("g++") is None:
        pytest.skip("g++ or the CUDA headers are missing")
    out = tmp_path_factory.mktemp("wbvh") / "libwbvh_check.so"
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-shared", "-fPIC", f"-DDDGI_WIDE_QUANT={request.param}",
           f"-I{inc}", f"-I{ROOT / 'anerend_gb300' / 'csrc'}", str(SRC), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(str(out))
    lib.wbvh_check.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.c_int,
                               ctypes.POINTER(ctypes.c_longlong)]
    lib.wbvh_check.restype = ctypes.c_int
    lib.divfast_check.argtypes = [ctypes.c_int, ctypes.c_uint64]
    lib.divfast_check.restype = ctypes.c_longlong
    lib.raydir_check.argtypes = [ctypes.c_int, ctypes.c_uint64]
    lib.raydir_check.restype = ctypes.c_longlong
    return lib


def run(lib, n, rays, seed, dup=0):
    st = (ctypes.c_longlong * 8)()
    bad = lib.wbvh_check(n, rays, seed, dup, st)
    return bad, list(st)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 8, 9, 17, 64, 333])
def test_small_trees(lib, n):
    bad, st = run(lib, n, 3000, 1000 + n)
    assert bad == 0, st


@pytest.mark.parametrize("n,dup", [(4000, 0), (20000, 0), (6000, 3)])
def test_larger_trees(lib, n, dup):
    bad, st = run(lib, n, 4000, 7 + n, dup)
    assert bad == 0, st
    assert st[6] > 1000  # enough rays hit something for the comparison to mean something
    # an 8-wide tree has far fewer nodes than the binary tree (n - 1)
    assert st[0] < n // 3


def test_invariant_divisor_division_is_exact(lib):
    """divFast, the ray-slot mapping's division by a per-grid reciprocal, equals integer division for every
    dividend below 2^31 tried, including the divisor's multiples and the values one below them."""
    assert lib.divfast_check(300000, 99) == 0


def test_direction_records_build_the_same_ray(lib):
    """A ray built from its direction's record (packRayDir, written once per lattice direction) equals the ray
    built from the direction itself, every field bit for bit."""
    assert lib.raydir_check(200000, 5) == 0
