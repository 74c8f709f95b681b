"""ctypes view of include/ddgi.h. Loading fails loudly when libddgi.so has not been built: there is no
CPU or PyTorch fallback for any entry point."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

import os

LIB_PATH = Path(os.environ.get("DDGI_LIB", Path(__file__).resolve().parent / "libddgi.so"))

DDGI_OK = 0
DDGI_EINVAL = -1
DDGI_ENOMEM = -2
DDGI_ETIMEDOUT = -3
DDGI_EDEVICE = -4
DDGI_EUNSUPPORTED = -5
DDGI_EOVERFLOW = -6
DDGI_EBUSY = -7

DDGI_UBO_DDGI_FLAG = 1 << 4
DDGI_UBO_DDGI_MULTI_FLAG = 1 << 5
DDGI_UBO_BAKE_MODE_ON_FLAG = 1 << 11

DDGI_FORMAT_RGBA32F = 0
DDGI_FORMAT_RGBA16F = 1

DDGI_GRID_EDGE_CLAMP = 1 << 0
DDGI_GRID_WRITE_DIRS = 1 << 1
DDGI_GRID_RECORD_HITS = 1 << 2
DDGI_GRID_RAYS_RGBA16F = 1 << 3

DDGI_ELEM_F16 = 0
DDGI_ELEM_BF16 = 1

ERROR_NAMES = {
    DDGI_EINVAL: "DDGI_EINVAL", DDGI_ENOMEM: "DDGI_ENOMEM", DDGI_ETIMEDOUT: "DDGI_ETIMEDOUT",
    DDGI_EDEVICE: "DDGI_EDEVICE", DDGI_EUNSUPPORTED: "DDGI_EUNSUPPORTED", DDGI_EOVERFLOW: "DDGI_EOVERFLOW",
    DDGI_EBUSY: "DDGI_EBUSY",
}

# ---- record dtypes (numpy views of the C structs) -------------------------------------------------
PACKED_VERTEX = np.dtype([("d0", "<f4", 4), ("d1", "<f4", 4), ("d2", "<f4", 4), ("d3", "<f4", 4),
                          ("d4", "<f4", 4), ("d5", "<i4", 4)])
MESH_INFO = np.dtype([("minPos", "<f4", 4), ("maxPos", "<f4", 4), ("vertexOffset", "<u4"),
                      ("indexOffset", "<u4"), ("numIndices", "<u4"), ("numVertices", "<u4")])
MATERIAL_INFO = np.dtype([("baseColFac", "<f4", 4), ("emissive", "<f4", 4), ("bindlessIndices", "<i4", 4),
                          ("metRough", "<f4", 4)])
INSTANCE = np.dtype([("transform", "<f4", 12), ("mesh", "<u4"), ("material", "<u4"), ("reserved", "<u4", 2)])
SURFACE_POINT = np.dtype([("position", "<f4", 3), ("metallic", "<f4"), ("normal", "<f4", 3), ("roughness", "<f4"),
                          ("albedo", "<f4", 3), ("shadow", "<f4")])
assert SURFACE_POINT.itemsize == 48
MIRROR_POINT = np.dtype([("position", "<f4", 3), ("sky", "<f4"), ("normal", "<f4", 3), ("reserved", "<f4")])
assert MIRROR_POINT.itemsize == 32
RAY = np.dtype([("origin", "<f4", 3), ("tmin", "<f4"), ("direction", "<f4", 3), ("tmax", "<f4")])
HIT = np.dtype([("t", "<f4"), ("b1", "<f4"), ("b2", "<f4"), ("triangle", "<i4")])
DDGI_RAY_ANY_HIT = 1
DDGI_SCENE_REFIT = 0
DDGI_SCENE_REBUILD = 1
assert PACKED_VERTEX.itemsize == 96 and MESH_INFO.itemsize == 48
assert MATERIAL_INFO.itemsize == 64 and INSTANCE.itemsize == 64


class SceneDesc(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("numVertices", C.c_uint64),
                ("indices", C.c_void_p), ("numIndices", C.c_uint64),
                ("meshes", C.c_void_p), ("numMeshes", C.c_uint32),
                ("instances", C.c_void_p), ("numInstances", C.c_uint32),
                ("materials", C.c_void_p), ("numMaterials", C.c_uint32)]


class SceneInfo(C.Structure):
    _fields_ = [("numTriangles", C.c_uint64), ("numNodes", C.c_uint64), ("deviceBytes", C.c_uint64),
                ("boundsMin", C.c_float * 3), ("boundsMax", C.c_float * 3)]


class GridDesc(C.Structure):
    _fields_ = [("dims", C.c_int32 * 3), ("step", C.c_float * 3), ("originY", C.c_float),
                ("raysPerProbe", C.c_int32), ("atlasFormat", C.c_int32), ("hysteresis", C.c_float),
                ("options", C.c_uint32)]


class Frame(C.Structure):
    _fields_ = [("cameraPos", C.c_float * 3), ("lightDir", C.c_float * 3), ("sunIntensity", C.c_float),
                ("skyColor", C.c_float * 3), ("skyIntensity", C.c_float), ("flags", C.c_uint32),
                ("rotation", C.c_float * 9), ("layer", C.c_int32), ("bakeTileInfo", C.c_int32 * 3)]


class Tuning(C.Structure):
    _fields_ = [("warpProbes", C.c_int32), ("rayOrder", C.c_int32), ("shadowMode", C.c_int32),
                ("convMode", C.c_int32), ("bvhWidth", C.c_int32), ("refillLanes", C.c_int32),
                ("reserved", C.c_int32 * 2)]


class BatchItem(C.Structure):
    _fields_ = [("grid", C.c_void_p), ("scene", C.c_void_p)]


class BatchTuning(C.Structure):
    _fields_ = [("warpProbes", C.c_int32), ("rayOrder", C.c_int32), ("shadowMode", C.c_int32),
                ("convMode", C.c_int32), ("blocksPerSm", C.c_int32), ("refillLanes", C.c_int32),
                ("useGraph", C.c_int32), ("bvhWidth", C.c_int32)]


class BatchStats(C.Structure):
    _fields_ = [("rays", C.c_uint64), ("translations", C.c_uint32), ("graphLaunches", C.c_uint32),
                ("eagerLaunches", C.c_uint32), ("reserved", C.c_uint32)]


class ServerConfig(C.Structure):
    _fields_ = [("memoryBudget", C.c_uint64), ("maxBatch", C.c_int32), ("inFlight", C.c_int32),
                ("convMode", C.c_int32), ("maxBatchMRays", C.c_uint32), ("policy", C.c_int32),
                ("agingMs", C.c_float), ("reserved", C.c_int32 * 2)]


DDGI_SERVE_FIFO = 0
DDGI_SERVE_SHORTEST_FIRST = 1


class Request(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("grid", GridDesc), ("frame", Frame), ("atlasOut", C.c_void_p),
                ("tag", C.c_uint64)]


class RequestStatus(C.Structure):
    _fields_ = [("state", C.c_int32), ("error", C.c_int32), ("submitSeconds", C.c_double),
                ("admitSeconds", C.c_double), ("doneSeconds", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("rejected", C.c_uint64),
                ("failed", C.c_uint64), ("batches", C.c_uint64), ("rays", C.c_uint64), ("peakBytes", C.c_uint64),
                ("p50LatencyMs", C.c_double), ("p99LatencyMs", C.c_double), ("meanLatencyMs", C.c_double),
                ("maxLatencyMs", C.c_double), ("elapsedSeconds", C.c_double)]


DDGI_REQUEST_QUEUED, DDGI_REQUEST_RUNNING, DDGI_REQUEST_DONE = 0, 1, 2
DDGI_REQUEST_FAILED, DDGI_REQUEST_REJECTED = -1, -2


class GridBuffers(C.Structure):
    _fields_ = [("atlas", C.c_void_p), ("rayRadiance", C.c_void_p), ("rayDirection", C.c_void_p),
                ("rayHit", C.c_void_p), ("lattice", C.c_void_p),
                ("atlasWidth", C.c_int32), ("atlasHeight", C.c_int32),
                ("rayWidth", C.c_int32), ("rayHeight", C.c_int32),
                ("rayBlockW", C.c_int32), ("rayBlockH", C.c_int32), ("atlasBytes", C.c_uint64),
                ("rayBytes", C.c_uint64), ("rayFormat", C.c_int32), ("reserved", C.c_int32)]


class WaitConfig(C.Structure):
    _fields_ = [("spinLimit", C.c_uint32), ("stallTest", C.c_uint32), ("reserved", C.c_uint32 * 2)]


ALLOC_HOOK = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_uint64)


class GridExternal(C.Structure):
    _fields_ = [("atlas", C.c_void_p), ("atlasTemp", C.c_void_p), ("rayRadiance", C.c_void_p),
                ("rayDirection", C.c_void_p), ("atlasBytes", C.c_uint64), ("rayBytes", C.c_uint64)]


# name -> (restype, argtypes); every symbol include/ddgi.h declares
SIGNATURES = {
    "ddgi_abi_version": (C.c_int, []),
    "ddgi_context_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "ddgi_context_destroy": (None, [C.c_void_p]),
    "ddgi_last_error": (C.c_char_p, [C.c_void_p]),
    "ddgi_sync": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ddgi_context_set_waits": (C.c_int, [C.c_void_p, C.POINTER(WaitConfig)]),
    "ddgi_context_set_alloc_hook": (C.c_int, [C.c_void_p, ALLOC_HOOK, C.c_void_p]),
    "ddgi_scene_create": (C.c_int, [C.c_void_p, C.POINTER(SceneDesc), C.c_void_p, C.POINTER(C.c_void_p)]),
    "ddgi_scene_destroy": (None, [C.c_void_p]),
    "ddgi_scene_info": (C.c_int, [C.c_void_p, C.POINTER(SceneInfo)]),
    "ddgi_grid_create": (C.c_int, [C.c_void_p, C.POINTER(GridDesc), C.POINTER(C.c_void_p)]),
    "ddgi_grid_destroy": (None, [C.c_void_p]),
    "ddgi_grid_buffers": (C.c_int, [C.c_void_p, C.POINTER(GridBuffers)]),
    "ddgi_grid_bind_external": (C.c_int, [C.c_void_p, C.POINTER(GridExternal), C.c_void_p]),
    "ddgi_grid_reset": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ddgi_grid_footprint": (C.c_uint64, [C.POINTER(GridDesc), C.c_int]),
    "ddgi_grid_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    "ddgi_grid_set_tuning": (C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    "ddgi_translate": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_int), C.c_void_p]),
    "ddgi_trace": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(Frame), C.c_void_p]),
    "ddgi_convolve": (C.c_int, [C.c_void_p, C.POINTER(Frame), C.c_void_p]),
    "ddgi_update": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(Frame), C.c_void_p]),
    "ddgi_atlas_download": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "ddgi_atlas_download_async": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "ddgi_atlas_download_wait": (C.c_int, [C.c_void_p]),
    "ddgi_atlas_upload": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "ddgi_rays_download": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ddgi_atlas_export_rgba16f": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "ddgi_atlas_import_rgba16f": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "ddgi_scene_update_transforms": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_int, C.c_void_p]),
    "ddgi_scene_update_vertices": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint64, C.c_int, C.c_void_p]),
    "ddgi_trace_rays": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32, C.c_void_p, C.c_void_p]),
    "ddgi_shadow_mask": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p]),
    "ddgi_query_irradiance": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p]),
    "ddgi_mirror_reflections": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p,
                                          C.c_void_p]),
    "ddgi_batch_create": (C.c_int, [C.c_void_p, C.POINTER(BatchItem), C.c_int, C.POINTER(C.c_void_p)]),
    "ddgi_batch_destroy": (None, [C.c_void_p]),
    "ddgi_batch_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(BatchTuning)]),
    "ddgi_batch_set_tuning": (C.c_int, [C.c_void_p, C.POINTER(BatchTuning)]),
    "ddgi_batch_stats": (C.c_int, [C.c_void_p, C.POINTER(BatchStats)]),
    "ddgi_batch_update": (C.c_int, [C.c_void_p, C.POINTER(Frame), C.c_void_p]),
    "ddgi_server_create": (C.c_int, [C.c_void_p, C.POINTER(ServerConfig), C.POINTER(C.c_void_p)]),
    "ddgi_server_submit": (C.c_int, [C.c_void_p, C.POINTER(Request), C.POINTER(C.c_uint64)]),
    "ddgi_server_status": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(RequestStatus)]),
    "ddgi_server_drain": (C.c_int, [C.c_void_p, C.c_double]),
    "ddgi_server_stats": (C.c_int, [C.c_void_p, C.POINTER(ServerStats)]),
    "ddgi_server_destroy": (None, [C.c_void_p]),
    "ddgi_fibonacci_lattice": (C.c_int, [C.c_int, C.POINTER(C.c_float), C.c_void_p, C.c_void_p]),
    "ddgi_convolve_raw": (C.c_int, [C.POINTER(GridDesc), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                    C.c_uint32, C.c_void_p]),
    "ddgi_translate_raw": (C.c_int, [C.POINTER(GridDesc), C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
    "ddgi_convolve_tc_raw": (C.c_int, [C.c_void_p, C.POINTER(GridDesc), C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                       C.c_int, C.c_int, C.c_uint32, C.c_void_p]),
    "ddgi_pack_rays16": (C.c_int, [C.POINTER(GridDesc), C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]),
    "ddgi_convolve_raw_noalloc": (C.c_int, [C.POINTER(GridDesc), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                            C.c_int, C.c_uint32, C.c_void_p]),
}

DDGI_NOALLOC_MAX_RAYS = 512

_lib = None


def load() -> C.CDLL:
    """Loads libddgi.so and binds every signature. Raises if the library is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class DdgiError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code
