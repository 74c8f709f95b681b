"""Seeded synthetic workloads for the probe engine: random-triangle scenes, probe grids and per-frame
parameters with the distributions of the benchmark configurations. Every random number comes from a
counter-based SplitMix64 stream (seed, stream id, counter), so any slice of a workload is reproducible.

The scenes stand in for the reference's Sponza scene, whose assets are not available: equilateral triangles
with uniformly random orientation, side U(0.2, 1.0), centroids uniform in a box, flat normals, vertex colour =
albedo; materials albedo U(0,1)^3, roughness U(0.1,1), metallic Bernoulli(0.2), 5% emissive with per-channel
radiance U(0,10)."""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from ._lib import INSTANCE, MATERIAL_INFO, MESH_INFO, PACKED_VERTEX

_GOLDEN64 = np.uint64(0x9E3779B97F4A7C15)


def splitmix64(x: np.ndarray) -> np.ndarray:
    x = (x + _GOLDEN64).astype(np.uint64)
    z = x
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def uniform(seed: int, stream: int, n: int, offset: int = 0) -> np.ndarray:
    """n doubles in [0, 1) from stream `stream` of `seed`, counters offset .. offset + n - 1."""
    with np.errstate(over="ignore"):
        base = splitmix64(np.array([seed * 0x100000001B3 + stream], dtype=np.uint64))[0]
        ctr = np.arange(offset, offset + n, dtype=np.uint64) + base
        bits = splitmix64(ctr)
    return (bits >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))


@dataclass
class Scene:
    vertices: np.ndarray   # PACKED_VERTEX records
    indices: np.ndarray    # uint32
    meshes: np.ndarray     # MESH_INFO
    instances: np.ndarray  # INSTANCE
    materials: np.ndarray  # MATERIAL_INFO

    @property
    def num_triangles(self) -> int:
        return int(sum(int(self.meshes[i]["numIndices"]) // 3 for i in self.instances["mesh"]))


def random_materials(seed: int, n: int, stream0: int = 100) -> np.ndarray:
    m = np.zeros(n, dtype=MATERIAL_INFO)
    alb = np.stack([uniform(seed, stream0 + k, n) for k in range(3)], 1)
    rough = 0.1 + 0.9 * uniform(seed, stream0 + 3, n)
    metal = (uniform(seed, stream0 + 4, n) < 0.2).astype(np.float64)
    emissive = uniform(seed, stream0 + 5, n) < 0.05
    erad = np.stack([10.0 * uniform(seed, stream0 + 6 + k, n) for k in range(3)], 1)
    m["baseColFac"][:, :3] = alb
    m["baseColFac"][:, 3] = 1.0
    m["emissive"][:, :3] = np.where(emissive[:, None], erad, 0.0)
    m["emissive"][:, 3] = np.where(emissive, 1.0, 0.0)
    m["bindlessIndices"] = -1
    m["metRough"][:, 0] = metal
    m["metRough"][:, 1] = rough
    return m


def random_triangles(seed: int, n: int, box_lo, box_hi, stream0: int = 0) -> np.ndarray:
    """(n, 3, 3) float64 vertices of random equilateral triangles."""
    lo = np.asarray(box_lo, np.float64)
    hi = np.asarray(box_hi, np.float64)
    cen = lo + (hi - lo) * np.stack([uniform(seed, stream0 + k, n) for k in range(3)], 1)
    side = 0.2 + 0.8 * uniform(seed, stream0 + 3, n)
    u1, u2, u3 = (uniform(seed, stream0 + 4 + k, n) for k in range(3))
    # uniform random rotation (Shoemake's quaternion)
    a, b = np.sqrt(1.0 - u1), np.sqrt(u1)
    qx, qy = a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2)
    qz, qw = b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (qy * qy + qz * qz); R[:, 0, 1] = 2 * (qx * qy - qz * qw); R[:, 0, 2] = 2 * (qx * qz + qy * qw)
    R[:, 1, 0] = 2 * (qx * qy + qz * qw); R[:, 1, 1] = 1 - 2 * (qx * qx + qz * qz); R[:, 1, 2] = 2 * (qy * qz - qx * qw)
    R[:, 2, 0] = 2 * (qx * qz - qy * qw); R[:, 2, 1] = 2 * (qy * qz + qx * qw); R[:, 2, 2] = 1 - 2 * (qx * qx + qy * qy)
    ang = np.array([math.pi / 2, math.pi / 2 + 2 * math.pi / 3, math.pi / 2 + 4 * math.pi / 3])
    canon = np.stack([np.cos(ang), np.sin(ang), np.zeros(3)], 1)  # unit circumradius
    r = side / math.sqrt(3.0)
    return cen[:, None, :] + np.einsum("nij,kj->nki", R, canon) * r[:, None, None]


def assemble(tris: np.ndarray, tri_mesh: np.ndarray, mesh_material: np.ndarray, materials: np.ndarray) -> Scene:
    """Builds scene records: triangles grouped into meshes (tri_mesh[i] = mesh of triangle i, meshes in
    increasing order), one identity instance per mesh, flat normals, vertex colour = material albedo."""
    tris = np.asarray(tris, np.float32)
    n = len(tris)
    order = np.argsort(tri_mesh, kind="stable")
    tris = tris[order]
    tri_mesh = np.asarray(tri_mesh)[order]
    num_meshes = int(tri_mesh.max()) + 1 if n else 0
    counts = np.bincount(tri_mesh, minlength=num_meshes)
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64)
    v = np.zeros(3 * n, dtype=PACKED_VERTEX)
    p = tris.reshape(-1, 3)
    e1 = tris[:, 1].astype(np.float64) - tris[:, 0]
    e2 = tris[:, 2].astype(np.float64) - tris[:, 0]
    nrm = np.cross(e1, e2)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm = np.repeat(nrm, 3, axis=0).astype(np.float32)
    alb = materials["baseColFac"][mesh_material[tri_mesh], :3]
    col = np.repeat(alb, 3, axis=0)
    v["d0"][:, :3] = p
    v["d0"][:, 3] = col[:, 0]
    v["d1"][:, 0] = col[:, 1]
    v["d1"][:, 1] = col[:, 2]
    v["d1"][:, 2] = nrm[:, 0]
    v["d1"][:, 3] = nrm[:, 1]
    v["d2"][:, 0] = nrm[:, 2]
    idx = np.empty(3 * n, np.uint32)
    meshes = np.zeros(num_meshes, dtype=MESH_INFO)
    for m in range(num_meshes):
        s, c = int(starts[m]), int(counts[m])
        meshes[m]["vertexOffset"] = 3 * s
        meshes[m]["indexOffset"] = 3 * s
        meshes[m]["numIndices"] = 3 * c
        meshes[m]["numVertices"] = 3 * c
        idx[3 * s: 3 * (s + c)] = np.arange(3 * c, dtype=np.uint32)
        if c:
            pts = p[3 * s: 3 * (s + c)]
            meshes[m]["minPos"][:3] = pts.min(0)
            meshes[m]["maxPos"][:3] = pts.max(0)
    inst = np.zeros(num_meshes, dtype=INSTANCE)
    inst["transform"] = np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], np.float32)
    inst["mesh"] = np.arange(num_meshes)
    inst["material"] = mesh_material[:num_meshes]
    return Scene(v, idx, meshes, inst, materials)


def floor_quad(y: float, half: float) -> np.ndarray:
    a = np.array([[-half, y, -half], [half, y, -half], [half, y, half]])
    b = np.array([[-half, y, -half], [half, y, half], [-half, y, half]])
    return np.stack([a, b])


@dataclass
class Workload:
    name: str
    dims: tuple
    step: tuple
    origin_y: float
    rays: int
    num_tris: int
    box_lo: tuple
    box_hi: tuple
    tris_per_mesh: int
    num_materials: int  # 0: one material per mesh
    floor_y: float | None
    floor_half: float
    frames: int
    hysteresis: float
    move_every: int = 0   # camera +1 in x every `move_every` frames (0: static camera)
    seed: int = 0
    light_dir: tuple = (-0.3, -1.0, -0.2)
    sun: float = 3.0
    sky: tuple = (0.4, 0.5, 0.7)
    sky_intensity: float = 1.0
    extra: dict = field(default_factory=dict)

    @property
    def probes(self) -> int:
        return self.dims[0] * self.dims[1] * self.dims[2]


# Plain DDGI update on the CPU-transcribed reference: 8x4x8 probes at 1.0 spacing around the origin
# (layers at y = -1.5 .. 1.5), 64 rays, 4096 random triangles in [-8, 8]^3 + a 20x20 floor at y = -2,
# one material per triangle, 8 frames, hysteresis 0.97.
CPU_REFERENCE = Workload("ddgi_8x4x8_n64_4k_tris", (8, 4, 8), (1.0, 1.0, 1.0), -1.5, 64, 4096,
                         (-8, -8, -8), (8, 8, 8), 1, 0, -2.0, 10.0, 8, 0.97)
# Plain single-grid GPU form: 32x8x32 probes, step (1,2,1), 256 rays, 262,144 triangles in
# [-30,30]x[0,15]x[-15,15] as 1024 meshes x 256 triangles with 1024 materials, 60 frames, camera +1 in x
# every 10 frames.
SINGLE_GRID = Workload("ddgi_32x8x32_n256_262k_tris", (32, 8, 32), (1.0, 2.0, 1.0), 0.0, 256, 262144,
                       (-30, 0, -15), (30, 15, 15), 256, 0, None, 0.0, 60, 0.97, move_every=10)


def build_scene(w: Workload) -> Scene:
    tris = random_triangles(w.seed, w.num_tris, w.box_lo, w.box_hi)
    tri_mesh = np.arange(w.num_tris) // w.tris_per_mesh
    n_mesh = int(tri_mesh.max()) + 1
    if w.floor_y is not None:
        tris = np.concatenate([tris, floor_quad(w.floor_y, w.floor_half)])
        tri_mesh = np.concatenate([tri_mesh, [n_mesh, n_mesh]])
        n_mesh += 1
    n_mat = w.num_materials or n_mesh
    mats = random_materials(w.seed, n_mat)
    mesh_material = np.arange(n_mesh) % n_mat
    return assemble(tris, tri_mesh, mesh_material, mats)


def rotation(seed: int, frame: int) -> np.ndarray:
    """mat3(glm::rotate(I, radians(angle), axis)) for a seeded axis in {x,y,z} and angle in [0, 360)
    (IrradianceProbeRayTracingPass.cpp:114-135 draws them from std::random_device); column-major float32."""
    u = uniform(seed, 7000, 2, offset=2 * frame)
    ax = min(int(u[0] * 3), 2)
    ang = math.radians(360.0 * u[1])
    a = np.zeros(3)
    a[ax] = 1.0
    c, s = math.cos(ang), math.sin(ang)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    R = c * np.eye(3) + s * K + (1 - c) * np.outer(a, a)
    return R.T.reshape(-1).astype(np.float32)  # column-major


def camera(w: Workload, frame: int) -> tuple:
    """Camera position of a frame: +1 in x every `move_every` frames over the workload's `frames`, then back
    (-1 every `move_every` frames) over as many, and so on. Frames past the first run keep the camera within
    the first run's positions, so a run of any length sees the same scene coverage and only ±1 translations."""
    if not w.move_every:
        return (0.0, 0.0, 0.0)
    legs = max(1, w.frames // w.move_every)  # positions 0 .. legs - 1 on the way out
    p = (frame // w.move_every) % (2 * legs)
    return (float(p if p < legs else 2 * legs - 1 - p), 0.0, 0.0)


@dataclass
class GridSpec:
    dims: tuple
    rays: int
    scene: int
    camera: tuple
    step: tuple = (1.0, 2.0, 1.0)
    origin_y: float = 0.0
    hysteresis: float = 0.97

    @property
    def probes(self) -> int:
        return self.dims[0] * self.dims[1] * self.dims[2]


@dataclass
class BatchWorkload:
    name: str
    num_grids: int
    num_scenes: int
    tri_range: tuple
    dims_choices: tuple
    rays_choices: tuple
    box_lo: tuple = (-30, 0, -15)
    box_hi: tuple = (30, 15, 15)
    seed: int = 0


# Batched form: 64 probe grids of uneven size (each axis from {4, 8, 16, 32}: 64 .. 32,768 probes) with
# rays/probe from {64, 128, 256, 512}, over 8 resident scenes of 10k .. 1M random triangles (log-uniform).
BATCHED = BatchWorkload("ddgi_batch_64grids_8scenes", 64, 8, (10_000, 1_000_000), (4, 8, 16, 32),
                        (64, 128, 256, 512))


def batch_layout(bw: BatchWorkload, tri_scale: float = 1.0, max_dim: int | None = None):
    """(triangle count per scene, GridSpec per grid) of a batched workload, from its seed."""
    u = uniform(bw.seed, 9000, bw.num_scenes)
    lo, hi = np.log(bw.tri_range[0]), np.log(bw.tri_range[1])
    tris = [max(64, int(round(np.exp(lo + (hi - lo) * x) * tri_scale))) for x in u]
    d = uniform(bw.seed, 9001, 3 * bw.num_grids).reshape(bw.num_grids, 3)
    r = uniform(bw.seed, 9002, bw.num_grids)
    sc = uniform(bw.seed, 9003, bw.num_grids)
    cam = uniform(bw.seed, 9004, 3 * bw.num_grids).reshape(bw.num_grids, 3)
    lo3, hi3 = np.asarray(bw.box_lo, float), np.asarray(bw.box_hi, float)
    grids = []
    for i in range(bw.num_grids):
        dims = tuple(int(bw.dims_choices[min(int(x * len(bw.dims_choices)), len(bw.dims_choices) - 1)]) for x in d[i])
        if max_dim:
            dims = tuple(min(v, max_dim) for v in dims)
        rays = int(bw.rays_choices[min(int(r[i] * len(bw.rays_choices)), len(bw.rays_choices) - 1)])
        camera = tuple(float(v) for v in np.round(lo3 + (hi3 - lo3) * cam[i], 3))
        grids.append(GridSpec(dims, rays, min(int(sc[i] * bw.num_scenes), bw.num_scenes - 1), camera))
    return tris, grids


def build_scene_tris(n: int, seed: int, box_lo=(-30, 0, -15), box_hi=(30, 15, 15), tris_per_mesh: int = 256,
                     num_materials: int = 1024) -> Scene:
    """A random-triangle scene of n triangles in a box (the workloads' distributions)."""
    tris = random_triangles(seed, n, box_lo, box_hi)
    tri_mesh = np.arange(n) // tris_per_mesh
    n_mesh = int(tri_mesh.max()) + 1
    mats = random_materials(seed, min(num_materials, n_mesh))
    return assemble(tris, tri_mesh, np.arange(n_mesh) % len(mats), mats)


@dataclass
class ServingWorkload:
    name: str
    num_scenes: int
    tri_range: tuple
    rate: float            # requests per second (Poisson)
    probe_range: tuple     # log-uniform probes per request
    rays_choices: tuple
    budget: int            # device bytes of admitted request grids
    seed: int = 0


# Serving form: 32 resident scenes of 10k .. 1M triangles, Poisson arrivals at 2,000 probe-update requests/s,
# each a grid of 256 .. 65,536 probes (log-uniform) with 64 .. 512 rays/probe, admitted under a 150 GB budget.
SERVING = ServingWorkload("ddgi_serving_32scenes_2000rps", 32, (10_000, 1_000_000), 2000.0, (256, 65536),
                          (64, 128, 256, 512), 150 << 30)


def serving_scene_tris(sw: ServingWorkload) -> list:
    """Triangle count of each resident scene of a serving workload (log-uniform over its range, from its seed)."""
    u = uniform(sw.seed, 9105, sw.num_scenes)
    lo, hi = np.log(sw.tri_range[0]), np.log(sw.tri_range[1])
    return [int(round(np.exp(lo + (hi - lo) * x))) for x in u]


def serving_requests(sw: ServingWorkload, count: int, rate: float | None = None):
    """`count` requests: (arrival time s, scene index, dims, rays, camera, rotation frame)."""
    rate = rate or sw.rate
    gaps = -np.log(1.0 - uniform(sw.seed, 9100, count)) / rate
    t = np.cumsum(gaps)
    lp = np.log2(sw.probe_range[0]) + (np.log2(sw.probe_range[1]) - np.log2(sw.probe_range[0])) * uniform(sw.seed, 9101, count)
    sc = uniform(sw.seed, 9102, count)
    rr = uniform(sw.seed, 9103, count)
    cam = uniform(sw.seed, 9104, 3 * count).reshape(count, 3)
    out = []
    for i in range(count):
        k = int(round(lp[i]))
        ax, rem = k // 3, k % 3
        dims = (1 << (ax + (rem >= 1)), 1 << ax, 1 << (ax + (rem >= 2)))
        rays = int(sw.rays_choices[min(int(rr[i] * len(sw.rays_choices)), len(sw.rays_choices) - 1)])
        camera = tuple(float(v) for v in np.round(np.array([-30, 0, -15]) + np.array([60, 15, 30]) * cam[i], 3))
        out.append((float(t[i]), min(int(sc[i] * sw.num_scenes), sw.num_scenes - 1), dims, rays, camera, i))
    return out
