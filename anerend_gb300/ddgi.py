"""Python host mirror of the reference's probe-update passes over the C ABI (include/ddgi.h).

The reference drives the path with three RenderPass objects
(src/anerend/render/passes/IrradianceProbe{Translation,RayTracing,Convolve}Pass.cpp); the classes of the same
names below keep their execution order and state (translation's last probe index, the round-robin layer,
the "ProbeLayer" hand-off) but run on a ProbeGrid + Scene owned by a Context. Errors raise DdgiError with the
library's status code and message; nothing here computes on the CPU."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from .scenes import Scene as SceneArrays


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data if a is not None and a.size else 0


class Context:
    """DdgiContext on one CUDA device."""

    def __init__(self, device: int = 0):
        self.lib = L.load()
        h = C.c_void_p()
        rc = self.lib.ddgi_context_create(device, C.byref(h))
        if rc != L.DDGI_OK:
            raise L.DdgiError(rc, f"ddgi_context_create(device={device}) failed")
        self.handle = h

    def check(self, rc: int) -> None:
        if rc != L.DDGI_OK:
            msg = self.lib.ddgi_last_error(self.handle)
            raise L.DdgiError(rc, msg.decode() if msg else "")

    def sync(self, stream: int = 0) -> None:
        self.check(self.lib.ddgi_sync(self.handle, stream))

    def close(self) -> None:
        if self.handle:
            self.lib.ddgi_context_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Scene:
    """Resident scene + LBVH (DdgiScene)."""

    def __init__(self, ctx: Context, arrays: SceneArrays, stream: int = 0):
        self.ctx = ctx
        self.arrays = arrays
        d = L.SceneDesc(_ptr(arrays.vertices), len(arrays.vertices), _ptr(arrays.indices), len(arrays.indices),
                        _ptr(arrays.meshes), len(arrays.meshes), _ptr(arrays.instances), len(arrays.instances),
                        _ptr(arrays.materials), len(arrays.materials))
        h = C.c_void_p()
        ctx.check(ctx.lib.ddgi_scene_create(ctx.handle, C.byref(d), stream, C.byref(h)))
        self.handle = h

    @property
    def info(self) -> L.SceneInfo:
        i = L.SceneInfo()
        self.ctx.check(self.ctx.lib.ddgi_scene_info(self.handle, C.byref(i)))
        return i

    def update_transforms(self, transforms: np.ndarray, rebuild: bool = False, stream: int = 0) -> None:
        """New (numInstances, 3, 4) object-to-world transforms; the BVHs are refitted (or rebuilt)."""
        t = np.ascontiguousarray(transforms, np.float32).reshape(-1, 12)
        self.ctx.check(self.ctx.lib.ddgi_scene_update_transforms(self.handle, _ptr(t), len(t),
                                                                 L.DDGI_SCENE_REBUILD if rebuild else L.DDGI_SCENE_REFIT,
                                                                 stream))

    def update_vertices(self, vertices: np.ndarray, first: int = 0, rebuild: bool = False, stream: int = 0) -> None:
        """New PACKED_VERTEX records starting at `first`; the BVHs are refitted (or rebuilt)."""
        v = np.ascontiguousarray(vertices)
        self.ctx.check(self.ctx.lib.ddgi_scene_update_vertices(self.handle, _ptr(v), first, len(v),
                                                               L.DDGI_SCENE_REBUILD if rebuild else L.DDGI_SCENE_REFIT,
                                                               stream))

    def trace_rays(self, rays_ptr: int, count: int, hits_ptr: int, any_hit: bool = False, stream: int = 0) -> None:
        """Closest (or any) hit of `count` device DdgiRay records into device DdgiHit records."""
        self.ctx.check(self.ctx.lib.ddgi_trace_rays(self.handle, rays_ptr, count, L.DDGI_RAY_ANY_HIT if any_hit else 0,
                                                    hits_ptr, stream))

    def shadow_mask(self, frame: "FrameParams", points_ptr: int, count: int, vis_ptr: int, stream: int = 0) -> None:
        """The RT shadow pass (shadow.rgen): visibility of device float4 points (w != 0: sky) along -lightDir."""
        f = frame.to_c()
        self.ctx.check(self.ctx.lib.ddgi_shadow_mask(self.handle, C.byref(f), points_ptr, count, vis_ptr, stream))

    def close(self) -> None:
        if self.handle:
            self.ctx.lib.ddgi_scene_destroy(self.handle)
            self.handle = None


@dataclass
class FrameParams:
    """Per-frame UBO fields and push constants of the path (scene_ubo.glsl:14-37, rgen:26-29)."""
    camera_pos: tuple = (0.0, 0.0, 0.0)
    light_dir: tuple = (-0.3, -1.0, -0.2)
    sun_intensity: float = 3.0
    sky_color: tuple = (0.4, 0.5, 0.7)
    sky_intensity: float = 1.0
    flags: int = L.DDGI_UBO_DDGI_FLAG | L.DDGI_UBO_DDGI_MULTI_FLAG
    rotation: np.ndarray = field(default_factory=lambda: np.eye(3, dtype=np.float32).reshape(-1))
    layer: int = -1
    bake_tile: tuple = (0, 0, 0)

    def to_c(self) -> L.Frame:
        f = L.Frame()
        f.cameraPos[:] = [float(v) for v in self.camera_pos]
        ld = np.asarray(self.light_dir, np.float64)
        ld = ld / np.linalg.norm(ld)
        f.lightDir[:] = [float(v) for v in ld.astype(np.float32)]
        f.sunIntensity = self.sun_intensity
        f.skyColor[:] = [float(v) for v in self.sky_color]
        f.skyIntensity = self.sky_intensity
        f.flags = self.flags
        f.rotation[:] = [float(v) for v in np.asarray(self.rotation, np.float32).reshape(-1)]
        f.layer = self.layer
        f.bakeTileInfo[:] = list(self.bake_tile)
        return f


class ProbeGrid:
    """Probe grid with its atlas, translation temp and ray images (DdgiGrid)."""

    def __init__(self, ctx: Context, dims, step=(1.0, 2.0, 1.0), rays_per_probe: int = 256, origin_y: float = 0.0,
                 hysteresis: float = 0.96, atlas_format: int = L.DDGI_FORMAT_RGBA32F, options: int = 0):
        self.ctx = ctx
        self.desc = L.GridDesc()
        self.desc.dims[:] = list(dims)
        self.desc.step[:] = list(step)
        self.desc.originY = origin_y
        self.desc.raysPerProbe = rays_per_probe
        self.desc.atlasFormat = atlas_format
        self.desc.hysteresis = hysteresis
        self.desc.options = options
        h = C.c_void_p()
        ctx.check(ctx.lib.ddgi_grid_create(ctx.handle, C.byref(self.desc), C.byref(h)))
        self.handle = h

    @property
    def buffers(self) -> L.GridBuffers:
        b = L.GridBuffers()
        self.ctx.check(self.ctx.lib.ddgi_grid_buffers(self.handle, C.byref(b)))
        return b

    @property
    def tuning(self) -> L.Tuning:
        t = L.Tuning()
        self.ctx.check(self.ctx.lib.ddgi_grid_get_tuning(self.handle, C.byref(t)))
        return t

    def set_tuning(self, warp_probes: int | None = None, ray_order: int | None = None,
                   shadow_mode: int | None = None, conv_mode: int | None = None,
                   bvh_width: int | None = None, refill_lanes: int | None = None) -> None:
        t = self.tuning
        if warp_probes is not None:
            t.warpProbes = warp_probes
        if ray_order is not None:
            t.rayOrder = ray_order
        if shadow_mode is not None:
            t.shadowMode = shadow_mode
        if conv_mode is not None:
            t.convMode = conv_mode
        if bvh_width is not None:
            t.bvhWidth = bvh_width
        if refill_lanes is not None:
            t.refillLanes = refill_lanes
        self.ctx.check(self.ctx.lib.ddgi_grid_set_tuning(self.handle, C.byref(t)))

    def reset(self, stream: int = 0) -> None:
        self.ctx.check(self.ctx.lib.ddgi_grid_reset(self.handle, stream))

    def translate(self, camera_pos, stream: int = 0) -> bool:
        cp = (C.c_float * 3)(*camera_pos)
        moved = C.c_int(0)
        self.ctx.check(self.ctx.lib.ddgi_translate(self.handle, cp, C.byref(moved), stream))
        return bool(moved.value)

    def trace(self, scene: Scene, frame: FrameParams, stream: int = 0) -> None:
        f = frame.to_c()
        self.ctx.check(self.ctx.lib.ddgi_trace(self.handle, scene.handle, C.byref(f), stream))

    def convolve(self, frame: FrameParams, stream: int = 0) -> None:
        f = frame.to_c()
        self.ctx.check(self.ctx.lib.ddgi_convolve(self.handle, C.byref(f), stream))

    def update(self, scene: Scene, frame: FrameParams, stream: int = 0) -> None:
        f = frame.to_c()
        self.ctx.check(self.ctx.lib.ddgi_update(self.handle, scene.handle, C.byref(f), stream))

    def atlas_shape(self) -> tuple:
        b = self.buffers
        return (b.atlasHeight, b.atlasWidth, 4)

    def download_atlas(self, stream: int = 0) -> np.ndarray:
        b = self.buffers
        dt = np.float32 if self.desc.atlasFormat == L.DDGI_FORMAT_RGBA32F else np.float16
        out = np.empty((b.atlasHeight, b.atlasWidth, 4), dt)
        self.ctx.check(self.ctx.lib.ddgi_atlas_download(self.handle, _ptr(out), out.nbytes, stream))
        return out

    def download_atlas_async(self, out, stream: int = 0) -> None:
        """Start a readback of the atlas into `out` (a contiguous host array or pinned torch tensor of
        atlasBytes, kept alive by the caller); it is complete once wait_download() returns."""
        ptr = out.data_ptr() if hasattr(out, "data_ptr") else _ptr(out)
        nbytes = out.numel() * out.element_size() if hasattr(out, "element_size") else out.nbytes
        self.ctx.check(self.ctx.lib.ddgi_atlas_download_async(self.handle, ptr, nbytes, stream))

    def wait_download(self) -> None:
        """Block until every readback started with download_atlas_async has reached the host."""
        self.ctx.check(self.ctx.lib.ddgi_atlas_download_wait(self.handle))

    def upload_atlas(self, arr: np.ndarray, stream: int = 0) -> None:
        arr = np.ascontiguousarray(arr)
        self.ctx.check(self.ctx.lib.ddgi_atlas_upload(self.handle, _ptr(arr), arr.nbytes, stream))

    def bind_external(self, atlas: int = 0, atlas_temp: int = 0, ray_radiance: int = 0, ray_direction: int = 0,
                      stream: int = 0) -> None:
        """Use caller-owned device buffers (pointers; 0 keeps the current binding) in place of the grid's own
        (ddgi_grid_bind_external): zero-copy interop with a renderer that owns the atlas and ray images."""
        b = self.buffers
        x = L.GridExternal(atlas or None, atlas_temp or None, ray_radiance or None, ray_direction or None,
                           b.atlasBytes, b.rayBytes)
        self.ctx.check(self.ctx.lib.ddgi_grid_bind_external(self.handle, C.byref(x), stream))

    def download_rays(self, hits: bool = False, stream: int = 0):
        """(radiance, hits, lattice): radiance in the grid's ray format (float32, or float16 with
        DDGI_GRID_RAYS_RGBA16F), shape (rayHeight, rayWidth, 4)."""
        b = self.buffers
        rad = np.empty((b.rayHeight, b.rayWidth, 4), np.float32 if b.rayFormat == L.DDGI_FORMAT_RGBA32F else np.float16)
        hit = np.empty((b.rayHeight, b.rayWidth), np.int32) if hits else None
        lat = np.empty((self.desc.raysPerProbe, 4), np.float32)
        self.ctx.check(self.ctx.lib.ddgi_rays_download(self.handle, _ptr(rad), _ptr(hit) if hits else None,
                                                       _ptr(lat), stream))
        return rad, hit, lat

    def export_atlas_rgba16f(self, stream: int = 0) -> np.ndarray:
        """The atlas in the reference's persisted layout: (10 Z Y, 10 X, 4) float16 (downloadDDGIAtlas)."""
        b = self.buffers
        out = np.empty((b.atlasHeight, b.atlasWidth, 4), np.float16)
        self.ctx.check(self.ctx.lib.ddgi_atlas_export_rgba16f(self.handle, _ptr(out), out.nbytes, stream))
        return out

    def import_atlas_rgba16f(self, arr: np.ndarray, stream: int = 0) -> None:
        arr = np.ascontiguousarray(arr, np.float16)
        self.ctx.check(self.ctx.lib.ddgi_atlas_import_rgba16f(self.handle, _ptr(arr), arr.nbytes, stream))

    def query_irradiance(self, frame: "FrameParams", points_ptr: int, count: int, ambient_ptr: int,
                         stream: int = 0) -> None:
        """Ambient term of `count` device DdgiSurfacePoint records into device float4 (deferred_tiled.comp's
        DDGI block, CLAMP_TO_EDGE sampling), stream-ordered."""
        f = frame.to_c()
        self.ctx.check(self.ctx.lib.ddgi_query_irradiance(self.handle, C.byref(f), points_ptr, count, ambient_ptr,
                                                          stream))

    def mirror_reflections(self, scene: "Scene", frame: "FrameParams", points_ptr: int, count: int, out_ptr: int,
                           stream: int = 0) -> None:
        """The specular GI mirror pass for `count` device DdgiMirrorPoint records into device float4
        (radiance, hit distance), with this grid's current atlas (mirror_reflections.rgen/.rchit/.rmiss),
        stream-ordered."""
        f = frame.to_c()
        self.ctx.check(self.ctx.lib.ddgi_mirror_reflections(self.handle, scene.handle, C.byref(f), points_ptr, count,
                                                            out_ptr, stream))

    def close(self) -> None:
        if self.handle:
            self.ctx.lib.ddgi_grid_destroy(self.handle)
            self.handle = None


# ---- the reference's three passes -----------------------------------------------------------------

class IrradianceProbeTranslationPass:
    """IrradianceProbeTranslationPass.cpp:56-186: shift the atlas when the camera's probe index changes.
    Skipped while baking (:59)."""

    def execute(self, grid: ProbeGrid, frame: FrameParams, stream: int = 0) -> bool:
        if frame.flags & L.DDGI_UBO_BAKE_MODE_ON_FLAG:
            return False
        return grid.translate(frame.camera_pos, stream)


class IrradianceProbeRayTracingPass:
    """IrradianceProbeRayTracingPass.cpp:95-165: trace one layer (round robin, frame.layer == -2) or all."""

    def execute(self, grid: ProbeGrid, scene: Scene, frame: FrameParams, stream: int = 0) -> None:
        grid.trace(scene, frame, stream)


class IrradianceProbeConvolvePass:
    """IrradianceProbeConvolvePass.cpp:109-143: convolve the layer(s) the ray-tracing pass wrote."""

    def execute(self, grid: ProbeGrid, frame: FrameParams, stream: int = 0) -> None:
        grid.convolve(frame, stream)


class Batch:
    """Many (grid, scene) items updated with one persistent trace launch and one convolution launch
    (DdgiBatch), replayed from a CUDA graph once the batch's shape repeats."""

    def __init__(self, ctx: Context, items):
        self.ctx = ctx
        self.items = list(items)
        arr = (L.BatchItem * len(self.items))(*[L.BatchItem(g.handle.value, s.handle.value) for g, s in self.items])
        h = C.c_void_p()
        ctx.check(ctx.lib.ddgi_batch_create(ctx.handle, arr, len(self.items), C.byref(h)))
        self.handle = h
        self._frames = (L.Frame * len(self.items))()

    @property
    def tuning(self) -> L.BatchTuning:
        t = L.BatchTuning()
        self.ctx.check(self.ctx.lib.ddgi_batch_get_tuning(self.handle, C.byref(t)))
        return t

    def set_tuning(self, **kw) -> None:
        t = self.tuning
        names = {"warp_probes": "warpProbes", "ray_order": "rayOrder", "shadow_mode": "shadowMode",
                 "conv_mode": "convMode", "blocks_per_sm": "blocksPerSm", "refill_lanes": "refillLanes",
                 "use_graph": "useGraph", "bvh_width": "bvhWidth"}
        for k, v in kw.items():
            setattr(t, names.get(k, k), int(v))
        self.ctx.check(self.ctx.lib.ddgi_batch_set_tuning(self.handle, C.byref(t)))

    @property
    def stats(self) -> L.BatchStats:
        s = L.BatchStats()
        self.ctx.check(self.ctx.lib.ddgi_batch_stats(self.handle, C.byref(s)))
        return s

    def update(self, frames, stream: int = 0) -> None:
        for i, fp in enumerate(frames):
            self._frames[i] = fp.to_c()
        self.ctx.check(self.ctx.lib.ddgi_batch_update(self.handle, self._frames, stream))

    def close(self) -> None:
        if self.handle:
            self.ctx.lib.ddgi_batch_destroy(self.handle)
            self.handle = None


def grid_desc(dims, step=(1.0, 2.0, 1.0), rays_per_probe: int = 256, origin_y: float = 0.0,
              hysteresis: float = 0.96, atlas_format: int = L.DDGI_FORMAT_RGBA32F, options: int = 0) -> L.GridDesc:
    d = L.GridDesc()
    d.dims[:] = list(dims)
    d.step[:] = list(step)
    d.originY = origin_y
    d.raysPerProbe = rays_per_probe
    d.atlasFormat = atlas_format
    d.hysteresis = hysteresis
    d.options = options
    return d


class Server:
    """Serving loop (DdgiServer): requests are admitted under a device-memory budget and launched in
    batches, up to `in_flight` launches overlapping on the device."""

    def __init__(self, ctx: Context, memory_budget: int, max_batch: int = 64, in_flight: int = 2,
                 conv_mode: int = 0, max_batch_mrays: int = 0, policy: int = L.DDGI_SERVE_FIFO,
                 aging_ms: float = 0.0):
        self.ctx = ctx
        cfg = L.ServerConfig()
        cfg.memoryBudget = int(memory_budget)
        cfg.maxBatch = max_batch
        cfg.inFlight = in_flight
        cfg.convMode = conv_mode
        cfg.maxBatchMRays = max_batch_mrays
        cfg.policy = policy
        cfg.agingMs = aging_ms
        h = C.c_void_p()
        ctx.check(ctx.lib.ddgi_server_create(ctx.handle, C.byref(cfg), C.byref(h)))
        self.handle = h

    def submit(self, scene: Scene, desc: L.GridDesc, frame: FrameParams, atlas_out: int = 0, tag: int = 0) -> int:
        r = L.Request()
        r.scene = scene.handle.value
        r.grid = desc
        r.frame = frame.to_c()
        r.atlasOut = atlas_out
        r.tag = tag
        rid = C.c_uint64(0)
        self.ctx.check(self.ctx.lib.ddgi_server_submit(self.handle, C.byref(r), C.byref(rid)))
        return rid.value

    def status(self, rid: int) -> L.RequestStatus:
        s = L.RequestStatus()
        self.ctx.check(self.ctx.lib.ddgi_server_status(self.handle, rid, C.byref(s)))
        return s

    def drain(self, timeout: float = 60.0) -> None:
        self.ctx.check(self.ctx.lib.ddgi_server_drain(self.handle, timeout))

    @property
    def stats(self) -> L.ServerStats:
        s = L.ServerStats()
        self.ctx.check(self.ctx.lib.ddgi_server_stats(self.handle, C.byref(s)))
        return s

    def close(self) -> None:
        if self.handle:
            self.ctx.lib.ddgi_server_destroy(self.handle)
            self.handle = None
