"""The C-ABI library builds, loads and exports every function include/ddgi.h declares (CPU only: no
compute call is made)."""
import ctypes
import re
from pathlib import Path

import pytest

from anerend_gb300 import _lib as L
from anerend_gb300 import build

HEADER = Path(__file__).resolve().parent.parent / "include" / "ddgi.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ddgi_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return ctypes.CDLL(str(build.LIB))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_header():
    assert set(declared_functions()) == set(L.SIGNATURES)


def test_abi_version_callable_without_gpu(lib):
    lib.ddgi_abi_version.restype = ctypes.c_int
    assert lib.ddgi_abi_version() == 2


def test_struct_sizes_match_header():
    # sizes of the records shared with the reference layouts
    assert L.PACKED_VERTEX.itemsize == 96     # PackedVertex, bindless.glsl:60-68
    assert L.MESH_INFO.itemsize == 48         # MeshInfo, bindless.glsl:51-58
    assert L.MATERIAL_INFO.itemsize == 64     # MaterialInfo, bindless.glsl:43-49
    assert ctypes.sizeof(L.Frame) == 4 * (3 + 3 + 1 + 3 + 1 + 1 + 9 + 1 + 3)
    assert ctypes.sizeof(L.GridDesc) == 4 * 11


def test_context_create_without_device_fails_cleanly(lib):
    # no GPU in the CPU suite: the call must return an error code, not crash
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L.load()
    h = ctypes.c_void_p()
    rc = L.load().ddgi_context_create(0, ctypes.byref(h))
    assert rc == L.DDGI_EDEVICE and not h.value
