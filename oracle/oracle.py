"""ORACLE — test infrastructure only. Python driver of the FP64 CPU restatement in ddgi_oracle.cpp.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module, and only as the
checker or the timed CPU baseline. It restates the per-frame pass sequence of the reference
(VulkanRenderer.cpp:4473-4475: translation, ray tracing, convolution) and the translation pass's host logic
(IrradianceProbeTranslationPass.cpp:61-80) in FP64."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "ddgi_oracle.cpp"
LIB = HERE / "liboracle.so"
ROOT = HERE.parent


def build(force: bool = False) -> Path:
    """Compiles ddgi_oracle.cpp with g++ into oracle/liboracle.so (portable flags: x86 and Arm)."""
    deps = [SRC, ROOT / "include" / "ddgi.h"]
    if not force and LIB.exists() and all(p.stat().st_mtime <= LIB.stat().st_mtime for p in deps):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", str(SRC), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        vp, ip, dp = C.c_void_p, C.c_int, C.POINTER(C.c_double)
        lib.oracle_scene_create.restype = vp
        lib.oracle_scene_create.argtypes = [vp]
        lib.oracle_scene_destroy.argtypes = [vp]
        lib.oracle_lattice.argtypes = [ip, vp, vp]
        lib.oracle_trace.restype = ip
        lib.oracle_trace.argtypes = [vp, vp, vp, vp, ip, ip, vp, vp, vp, ip]
        lib.oracle_convolve.restype = ip
        lib.oracle_convolve.argtypes = [vp, vp, vp, vp, ip, ip, C.c_uint32, C.c_double, ip]
        lib.oracle_translate.restype = ip
        lib.oracle_translate.argtypes = [vp, vp, vp, ip, ip, ip]
        lib.oracle_num_triangles.restype = ip
        lib.oracle_num_triangles.argtypes = [vp]
        lib.oracle_closest_hit.restype = ip
        lib.oracle_closest_hit.argtypes = [vp, vp, vp, vp, vp, vp]
        lib.oracle_query_irradiance.restype = ip
        lib.oracle_query_irradiance.argtypes = [vp, vp, vp, vp, C.c_int64, vp]
        lib.oracle_mirror_reflections.restype = ip
        lib.oracle_mirror_reflections.argtypes = [vp, vp, vp, vp, vp, C.c_int64, vp, vp, ip]
        _lib = lib
    return _lib


def _p(a: np.ndarray) -> int:
    return a.ctypes.data if a is not None else 0


class OracleScene:
    def __init__(self, arrays, scene_desc_cls):
        self.lib = load()
        self.arrays = arrays
        d = scene_desc_cls(_p(arrays.vertices), len(arrays.vertices), _p(arrays.indices), len(arrays.indices),
                           _p(arrays.meshes), len(arrays.meshes), _p(arrays.instances), len(arrays.instances),
                           _p(arrays.materials), len(arrays.materials))
        self.handle = self.lib.oracle_scene_create(C.addressof(d))

    def closest_hit(self, origin, direction):
        """(global id or -1, t, (b1, b2), uncertain) of one ray in [0.1, 50]."""
        o = np.asarray(origin, np.float64)
        d = np.asarray(direction, np.float64)
        t = np.zeros(1)
        b = np.zeros(2)
        u = np.zeros(1, np.int32)
        gid = self.lib.oracle_closest_hit(self.handle, _p(o), _p(d), _p(t), _p(b), _p(u))
        return gid, float(t[0]), (float(b[0]), float(b[1])), bool(u[0])

    def close(self):
        if self.handle:
            self.lib.oracle_scene_destroy(self.handle)
            self.handle = None


@dataclass
class GridGeom:
    X: int
    Y: int
    Z: int
    N: int

    @property
    def block(self):
        lg = (self.N - 1).bit_length()
        bw = 1 << ((lg + 1) // 2)
        return bw, self.N // bw

    @property
    def atlas_hw(self):
        return 10 * self.Z * self.Y, 10 * self.X

    @property
    def ray_hw(self):
        bw, bh = self.block
        return bh * self.Z * self.Y, bw * self.X


class OracleGrid:
    """FP64 probe grid: atlas RGBA doubles cleared to (0,0,0,1), translation state (0,0), round-robin layer."""

    def __init__(self, desc, threads: int = 0):
        self.lib = load()
        self.desc = desc
        self.threads = threads
        self.geom = GridGeom(desc.dims[0], desc.dims[1], desc.dims[2], desc.raysPerProbe)
        h, w = self.geom.atlas_hw
        self.atlas = np.zeros((h, w, 4), np.float64)
        self.atlas[..., 3] = 1.0
        rh, rw = self.geom.ray_hw
        self.ray_rad = np.zeros((rh, rw, 4), np.float64)
        self.hits = np.full((rh, rw), -1, np.int32)
        self.uncertain = np.zeros((rh, rw), np.uint8)
        self.last_probe_idx = (0, 0)
        self.current_layer = 0
        self.traced = (0, 0)
        self.dirs = None

    def translate(self, camera_pos) -> bool:
        step = np.float32(self.desc.step[0]), np.float32(self.desc.step[2])
        ix = int(np.float32(camera_pos[0]) / step[0])
        iz = int(np.float32(camera_pos[2]) / step[1])
        dx, dz = ix - self.last_probe_idx[0], iz - self.last_probe_idx[1]
        if dx == 0 and dz == 0:
            return False
        self.last_probe_idx = (ix, iz)
        out = np.empty_like(self.atlas)
        self.lib.oracle_translate(C.addressof(self.desc), _p(self.atlas), _p(out), dx, dz, 32)
        self.atlas = out
        return True

    def layer_range(self, layer: int, advance: bool):
        if layer == -1:
            return 0, self.geom.Y
        if layer == -2:
            b = self.current_layer
            if advance:
                self.current_layer = (self.current_layer + 1) % self.geom.Y
            return b, b + 1
        return layer, layer + 1

    def trace(self, scene: OracleScene, frame) -> None:
        b, e = self.layer_range(frame.layer, True)
        atlas_prev = np.ascontiguousarray(self.atlas)
        self.lib.oracle_trace(scene.handle, C.addressof(self.desc), C.addressof(frame), _p(atlas_prev), b, e,
                              _p(self.ray_rad), _p(self.hits), _p(self.uncertain), self.threads)
        self.dirs = lattice(self.desc.raysPerProbe, np.array(frame.rotation[:], np.float32))
        self.traced = (b, e)

    def convolve(self, frame) -> None:
        b, e = self.traced if frame.layer == -2 else self.layer_range(frame.layer, False)
        self.lib.oracle_convolve(C.addressof(self.desc), _p(self.ray_rad), _p(self.dirs), _p(self.atlas), b, e,
                                 frame.flags, float(self.desc.hysteresis), self.threads)

    def update(self, scene: OracleScene, frame, bake_flag: int = 1 << 11) -> None:
        if not (frame.flags & bake_flag):
            self.translate(frame.cameraPos[:])
        self.trace(scene, frame)
        self.convolve(frame)


def lattice(n: int, rot: np.ndarray) -> np.ndarray:
    out = np.empty((n, 3), np.float64)
    r = np.ascontiguousarray(rot, np.float32)
    load().oracle_lattice(n, _p(r), _p(out))
    return out


def convolve(desc, ray_rad: np.ndarray, dirs: np.ndarray, atlas: np.ndarray, layer_begin: int, layer_end: int,
             flags: int, threads: int = 0, hysteresis: float | None = None) -> None:
    """probe_conv.comp on FP64 arrays; `atlas` is updated in place. hysteresis defaults to the grid
    description's (a float32 value)."""
    ray_rad = np.ascontiguousarray(ray_rad, np.float64)
    dirs = np.ascontiguousarray(dirs, np.float64)
    assert atlas.dtype == np.float64 and atlas.flags.c_contiguous
    h = float(desc.hysteresis) if hysteresis is None else float(hysteresis)
    load().oracle_convolve(C.addressof(desc), _p(ray_rad), _p(dirs), _p(atlas), layer_begin, layer_end, flags, h,
                           threads)


def translate(desc, atlas: np.ndarray, dx: int, dz: int) -> np.ndarray:
    a = np.ascontiguousarray(atlas)
    assert a.ndim == 3, "atlas must be (height, width, texel components or bytes)"
    out = np.empty_like(a)
    load().oracle_translate(C.addressof(desc), _p(a), _p(out), dx, dz, a.itemsize * a.shape[-1])
    return out


def query_irradiance(desc, frame, atlas: np.ndarray, points: np.ndarray) -> np.ndarray:
    """deferred_tiled.comp:263-299 on FP64: ambient term (count x 3) of SURFACE_POINT records from `atlas`."""
    a = np.ascontiguousarray(atlas, np.float64)
    pts = np.ascontiguousarray(points)
    out = np.empty((len(pts), 3), np.float64)
    load().oracle_query_irradiance(C.addressof(desc), C.addressof(frame), _p(a), _p(pts), len(pts), _p(out))
    return out


def mirror_reflections(scene: OracleScene, desc, frame, atlas: np.ndarray, points: np.ndarray, threads: int = 0):
    """mirror_reflections.rgen/.rchit/.rmiss on FP64: (radiance, hit distance) per MIRROR_POINT record (count x 4)
    and the uncertainty bits per point (1: the reflected ray near a tie or an edge, 2: its shadow ray)."""
    a = np.ascontiguousarray(atlas, np.float64)
    pts = np.ascontiguousarray(points)
    out = np.empty((len(pts), 4), np.float64)
    unc = np.zeros(len(pts), np.uint8)
    scene.lib.oracle_mirror_reflections(scene.handle, C.addressof(desc), C.addressof(frame), _p(a), _p(pts), len(pts),
                                        _p(out), _p(unc), threads)
    return out, unc
