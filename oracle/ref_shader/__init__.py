"""ORACLE — test infrastructure only. The reference's DDGI shader stages compiled as FP64 C++ (build_ref.py,
ref_harness.cpp): ray generation + closest-hit + miss on chosen pixels of one layer's ray image, and the
convolution on chosen invocations, at the reference's compile-time grid (64 x 8 x 64 probes, 256 rays,
hysteresis 0.96); and, per G-buffer point, the specular GI mirror pass, the RT shadow pass and the deferred
pass's DDGI block. Used to pin the oracle restatement (tests/test_oracle_vs_reference_shaders.py) and to
make the golden fixtures in tests/golden/. Available only where the reference sources are present."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build_ref import LIB, build_if_available

# the reference's compile-time grid (probe_helpers.glsl) and convolution hysteresis (probe_conv.comp)
DIMS = (64, 8, 64)
STEP = (1.0, 2.0, 1.0)
RAYS = 256
HYSTERESIS = 0.96
RAY_IMAGE = (1024, 1024)    # per layer: 16 x 64 texels each way
ATLAS = (5120, 640)         # (10 * Z * Y, 10 * X)


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


class RefShaders:
    def __init__(self):
        path = build_if_available()
        if path is None or not Path(path).exists():
            raise FileNotFoundError("reference shader sources not available")
        self.lib = C.CDLL(str(path))
        self.lib.ref_scene_set.argtypes = [C.c_void_p]
        self.lib.ref_scene_set.restype = C.c_int
        self.lib.ref_trace.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                       C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        self.lib.ref_trace.restype = C.c_int
        self.lib.ref_convolve.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                          C.c_int, C.c_int]
        self.lib.ref_convolve.restype = C.c_int
        for name in ("ref_mirror", "ref_query_irradiance"):
            fn = getattr(self.lib, name)
            fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int64, C.c_void_p]
            fn.restype = C.c_int
        self.lib.ref_shadow_mask.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
        self.lib.ref_shadow_mask.restype = C.c_int
        self._keep = None

    def set_scene(self, scene_desc) -> None:
        """scene_desc: an anerend_gb300._lib.SceneDesc whose arrays stay alive while this object is used."""
        self._keep = scene_desc
        assert self.lib.ref_scene_set(C.addressof(scene_desc)) == 0

    def trace(self, frame, rotation, layer: int, atlas_prev: np.ndarray, x0: int, y0: int, x1: int, y1: int):
        """Ray-image texels [x0, x1) x [y0, y1) of `layer`: (radiance RGBA, direction RGBA), FP64."""
        atlas = np.ascontiguousarray(atlas_prev, np.float64)
        assert atlas.shape == ATLAS + (4,)
        rot = np.ascontiguousarray(rotation, np.float32).reshape(9)
        irr = np.zeros((y1 - y0, x1 - x0, 4), np.float64)
        dirs = np.zeros_like(irr)
        assert self.lib.ref_trace(C.addressof(frame), _p(rot), layer, _p(atlas), ATLAS[1], ATLAS[0], x0, y0, x1, y1,
                                  _p(irr), _p(dirs)) == 0
        return irr, dirs

    def convolve(self, frame, layer: int, irr_image: np.ndarray, dir_image: np.ndarray, atlas: np.ndarray,
                 x0: int, y0: int, x1: int, y1: int) -> None:
        """Convolution invocations [x0, x1) x [y0, y1) of `layer` into `atlas` (FP64, in place)."""
        irr = np.ascontiguousarray(irr_image, np.float64)
        dirs = np.ascontiguousarray(dir_image, np.float64)
        assert irr.shape == RAY_IMAGE + (4,) and dirs.shape == RAY_IMAGE + (4,)
        assert atlas.dtype == np.float64 and atlas.flags.c_contiguous and atlas.shape == ATLAS + (4,)
        assert self.lib.ref_convolve(C.addressof(frame), layer, _p(irr), _p(dirs), _p(atlas), x0, y0, x1, y1) == 0


    def mirror(self, frame, atlas: np.ndarray, points: np.ndarray) -> np.ndarray:
        """mirror_reflections.rgen on MIRROR_POINT records with `atlas` (FP64, the reference's atlas size) as
        probeTex: (count, 4) (radiance, hit distance)."""
        a = np.ascontiguousarray(atlas, np.float64)
        assert a.shape == ATLAS + (4,)
        pts = np.ascontiguousarray(points)
        out = np.zeros((len(pts), 4))
        assert self.lib.ref_mirror(C.addressof(frame), _p(a), ATLAS[1], ATLAS[0], _p(pts), len(pts), _p(out)) == 0
        return out

    def shadow_mask(self, frame, points: np.ndarray) -> np.ndarray:
        """shadow.rgen on float32 (x, y, z, sky) points: the stored visibility per point."""
        pts = np.ascontiguousarray(points, np.float32)
        out = np.zeros(len(pts))
        assert self.lib.ref_shadow_mask(C.addressof(frame), _p(pts), len(pts), _p(out)) == 0
        return out

    def query_irradiance(self, frame, atlas: np.ndarray, points: np.ndarray) -> np.ndarray:
        """The deferred pass's DDGI block (doLight with the direct light off) on SURFACE_POINT records with
        `atlas` as probeTex (CLAMP_TO_EDGE): (count, 3) ambient terms."""
        a = np.ascontiguousarray(atlas, np.float64)
        assert a.shape == ATLAS + (4,)
        pts = np.ascontiguousarray(points)
        out = np.zeros((len(pts), 3))
        assert self.lib.ref_query_irradiance(C.addressof(frame), _p(a), ATLAS[1], ATLAS[0], _p(pts), len(pts),
                                             _p(out)) == 0
        return out


__all__ = ["RefShaders", "build_if_available", "LIB", "DIMS", "STEP", "RAYS", "HYSTERESIS", "RAY_IMAGE", "ATLAS"]
