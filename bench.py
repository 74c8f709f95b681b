"""Benchmark of the DDGI probe update on the 32x8x32-probe / 256-ray / 262,144-triangle single-grid workload.

One step = one probe update of the whole grid: translation (when the camera's probe index changes), the
rotated golden-angle lattice, trace + shade of all 2,097,152 rays, and the convolution + hysteresis of all
8192 probes. The camera moves +1 in x every 10 frames over the workload's 60 frames, as in the workload
definition, then back and forth over the same positions, so a long run stays within the same scene.

  value      probe rays/s, device-timed (CUDA events on the launching stream), inputs resident in HBM
  e2e        the same metric through the C ABI from the host: ddgi_update + ddgi_atlas_download_async into
             pinned host memory, each step's readback overlapping the next update, wall clock over all steps
             (host frame parameters in, every step's atlas out); blocking_readback_value times
             ddgi_update + ddgi_atlas_download, which waits for each atlas
  roofline   of the dominant work, the trace (closest-hit traversal, shading, shadow traversal: three
             kernels in stream order): algorithmic bytes / its event-timed duration vs the
             measured HBM copy bandwidth
  cpu_baseline  the FP64 oracle on all host cores over a bounded sample (rank 0, N = 1 only)

--impl reference times the CPU implementation of the path (the oracle restatement; the reference's GLSL
cannot run on this machine) on the same workload and metric.

Multi-GPU (torchrun): probe grids are independent, so each rank updates its own replica of the grid
(weak scaling, no data-path collective); a barrier brackets the timed region and the max over ranks is
reported."""
from __future__ import annotations

import argparse
import datetime
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

PEAKS_FALLBACK = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}
METRIC = "probe rays/s"
UNIT = "rays/s"
# compulsory bytes of the trace + shade kernel (per primary hit / per miss): 3 indices (12 B), three full
# 96-byte vertex records (288 B), the material (64 B), the 8-probe x 4-texel FP32 atlas gather (512 B) and
# the radiance write (12 B); a miss writes the radiance only.
BYTES_PER_HIT = 12 + 3 * 96 + 64 + 8 * 4 * 16 + 12
BYTES_PER_MISS = 12


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d["bf16_tflops"]), "source": "measured"}
    return dict(PEAKS_FALLBACK, source="fallback")


class ClockSampler:
    """nvidia-smi clock / throttle samples (every 200 ms) during the timed region.

    Each sample carries nvidia-smi's timestamp; stop(t0, t1) keeps the samples taken between the wall-clock
    times t0 and t1 (time.time()) of the timed region, or all samples if none fell inside it."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.out = None

    def start(self):
        try:
            self.out = open(Path(tempfile.gettempdir()) / f".ddgi_clocks_{os.getpid()}.csv", "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.out,
                                         stderr=subprocess.DEVNULL)
            time.sleep(0.5)  # nvidia-smi start-up, so its samples cover the whole timed region
        except (OSError, FileNotFoundError):
            self.proc = None

    @staticmethod
    def parse(lines, t0=None, t1=None):
        """Summary of sample lines: median SM clock, max clock, active slowdown reasons, sample counts."""
        rows = []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                sm, smax = float(f[2]), float(f[3])
            except ValueError:
                continue
            rows.append((ts, sm, smax, {nm for nm, v in zip(names, f[6:10]) if v.lower() == "active"}))
        inside = [r for r in rows if t0 is not None and t0 <= r[0] <= t1]
        use = inside or rows
        if not use:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0,
                    "samples_in_region": 0}
        return {"sm_mhz": statistics.median(r[1] for r in use), "sm_max_mhz": use[-1][2],
                "reasons": sorted(set().union(*(r[3] for r in use))), "samples": len(use),
                "samples_in_region": len(inside)}

    def stop(self, t0=None, t1=None):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        self.proc.wait()
        self.out.close()
        lines = Path(self.out.name).read_text().strip().splitlines()
        Path(self.out.name).unlink(missing_ok=True)
        return self.parse(lines, t0, t1)


def dist_init():
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1 and not dist.is_initialized():
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return rank, local, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_sample(w, arrays, frames: int, threads: int = 0):
    """FP64 oracle on `frames` full probe updates; returns (rays/s, seconds, threads used)."""
    from anerend_gb300 import _lib as L
    from anerend_gb300.ddgi import FrameParams
    from oracle import oracle

    d = L.GridDesc()
    d.dims[:] = list(w.dims)
    d.step[:] = list(w.step)
    d.originY = w.origin_y
    d.raysPerProbe = w.rays
    d.hysteresis = w.hysteresis
    osc = oracle.OracleScene(arrays, L.SceneDesc)
    og = oracle.OracleGrid(d, threads=threads)
    t0 = time.perf_counter()
    from anerend_gb300 import scenes

    for f in range(frames):
        og.update(osc, FrameParams(camera_pos=scenes.camera(w, f), rotation=scenes.rotation(w.seed, f)).to_c())
    dt = time.perf_counter() - t0
    osc.close()
    used = threads if threads > 0 else (os.cpu_count() or 1)
    return frames * w.probes * w.rays / dt, dt, used


def run_reference(args, rank, world):
    """CPU implementation of the path (the FP64 oracle restatement on all host threads), same metric."""
    from anerend_gb300 import scenes

    if rank != 0:
        return
    w = scenes.SINGLE_GRID
    arrays = scenes.build_scene(w)
    # each step: one full probe update of the grid is ~3 s on 8 cores; a step here is one layer (1/8 of a
    # frame: 262,144 rays), so warm-up + steps stay within a few minutes
    from anerend_gb300 import _lib as L
    from anerend_gb300.ddgi import FrameParams
    from oracle import oracle

    d = L.GridDesc()
    d.dims[:] = list(w.dims)
    d.step[:] = list(w.step)
    d.originY = w.origin_y
    d.raysPerProbe = w.rays
    d.hysteresis = w.hysteresis
    osc = oracle.OracleScene(arrays, L.SceneDesc)
    og = oracle.OracleGrid(d)
    times = []
    for s in range(args.warmup + args.steps):
        fp = FrameParams(camera_pos=scenes.camera(w, s), rotation=scenes.rotation(w.seed, s), layer=s % w.dims[1])
        t0 = time.perf_counter()
        og.update(osc, fp.to_c())
        dt = time.perf_counter() - t0
        if s >= args.warmup:
            times.append(dt)
    rays = w.dims[0] * w.dims[2] * w.rays
    total = sum(times)
    value = rays * len(times) / total
    cores = os.cpu_count() or 1
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": w.name, "probes": w.probes, "rays_per_probe": w.rays,
                       "triangles": w.num_tris, "step_unit": "one probe layer (32x32 probes x 256 rays)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{args.steps} single-layer updates of 262,144 rays, FP64 oracle, std::thread x {cores}"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    osc.close()
    print(json.dumps(line))


def _time_updates(torch, fn, frames, reps):
    """Median CUDA-event time (ms) of fn(frame) over reps frames after 2 warm-up calls."""
    for f in range(2):
        fn(frames(f))
    torch.cuda.synchronize()
    ts = []
    for f in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        fr = frames(f + 2)
        e0.record()
        fn(fr)
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return float(np.median(ts))


def _time_back_to_back(torch, fn, reps):
    """CUDA-event time (ms) per call of `reps` calls issued back to back after 2 warm-up calls, so the
    host's launch work overlaps the device's."""
    for _ in range(2):
        fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def _texel_dirs64(np):
    """FP64 directions of the 8 x 8 octahedral texels (probe_conv.comp:283-286 with octDecode)."""
    t = np.arange(64)
    u = (2.0 * (t % 8) + 1.0) / 16.0 * 2.0 - 1.0
    v = (2.0 * (t // 8) + 1.0) / 16.0 * 2.0 - 1.0
    vx, vy, vz = u.copy(), v.copy(), 1.0 - np.abs(u) - np.abs(v)
    neg = vz < 0
    sx, sy = np.where(u >= 0, 1.0, -1.0), np.where(v >= 0, 1.0, -1.0)
    vx[neg], vy[neg] = ((1.0 - np.abs(v)) * sx)[neg], ((1.0 - np.abs(u)) * sy)[neg]
    d = np.stack([vx, vz, vy], 1)  # octDecode swaps y and z
    return d / np.linalg.norm(d, axis=1, keepdims=True)


def _oracle_conv_blocks(R, dirs64):
    """The FP64 oracle's convolution (oracle.convolve, probe_conv.comp:21-90) of K probes with hysteresis 0:
    R is (3, K, n) FP64 radiance, dirs64 the (n, 3) ray directions; returns the (K, 8, 8, 3) interior texels.
    The probes are laid out as a K x 1 x 1 grid, since each probe's convolution depends only on its own rays."""
    from anerend_gb300 import ddgi
    from oracle import oracle

    K, n = R.shape[1], R.shape[2]
    g = oracle.GridGeom(K, 1, 1, n)
    bw, _ = g.block
    rh, rw = g.ray_hw
    img = np.zeros((rh, rw, 4))
    img[..., 3] = 1.0
    j = np.arange(n)
    img[(j // bw)[None, :], np.arange(K)[:, None] * bw + (j % bw)[None, :], :3] = R.transpose(1, 2, 0)
    ah, aw = g.atlas_hw
    atlas = np.zeros((ah, aw, 4))
    atlas[..., 3] = 1.0
    oracle.convolve(ddgi.grid_desc((K, 1, 1), rays_per_probe=n, hysteresis=0.0), img, dirs64, atlas, 0, 1, 0,
                    hysteresis=0.0)
    return atlas[1:9, :, :3].reshape(8, K, 10, 3)[:, :, 1:9, :].transpose(1, 0, 2, 3)


def _atlas_blocks(atlas, dims, probes):
    """(K, 8, 8, 3) interior texels of probes p = (layer * Z + z) * X + x of an RGBA atlas (10 Z Y, 10 X, 4)."""
    X, _, Z = dims
    x, z, layer = probes % X, (probes // X) % Z, probes // (X * Z)
    t = np.arange(8)
    r0, c0 = 10 * (Z * layer + z) + 1, 10 * x + 1
    return atlas[r0[:, None, None] + t[None, :, None], c0[:, None, None] + t[None, None, :], :3]


def _rel_err_stats(pairs):
    """max / p99 / mean per-texel-channel relative error over (got, want) block pairs, each pair's denominator
    floored at 1e-6 x its mean irradiance."""
    e = np.concatenate([(np.abs(got.astype(np.float64) - want) / np.maximum(np.abs(want), 1e-6 * np.abs(want).mean()))
                        .ravel() for got, want in pairs])
    return {"max": float(e.max()), "p99": float(np.percentile(e, 99)), "mean": float(e.mean()),
            "texel_channels": int(e.size)}


def measure_precision(ctx, stream):
    """Convolution of the 65,536-probe / 512-ray precision workload (radiance log-uniform in [1e-3, 1e2] per
    channel, seeded, generated on the device) on tensor cores (FP16, BF16) and on CUDA cores (FP32): time per
    call issued back to back, and per-texel relative error of the convolution result against the same
    formula in FP64 (denominator floor 1e-6 x mean irradiance; hysteresis 0, so the atlas holds the result)."""
    import ctypes as C

    import torch

    from anerend_gb300 import _lib as L
    from anerend_gb300 import ddgi, scenes

    lib = L.load()
    dims, n = (64, 16, 64), 512
    P = dims[0] * dims[1] * dims[2]
    gen = torch.Generator(device="cuda")
    gen.manual_seed(0)
    R32 = torch.exp(torch.empty((3, P, n), device="cuda").uniform_(np.log(1e-3), np.log(1e2), generator=gen))
    dirs = torch.empty(n * 4, dtype=torch.float32, device="cuda")
    lib.ddgi_fibonacci_lattice(n, (C.c_float * 9)(*scenes.rotation(0, 0).tolist()), dirs.data_ptr(), stream)
    atlas = torch.zeros((10 * dims[2] * dims[1], 10 * dims[0], 4), device="cuda")
    prec = {"probes": P, "rays_per_probe": n, "algorithmic_bytes": P * (6 * n + 2048)}
    # FP64 reference of the convolution result: sum_j W[t, j] L_j / s_t with W = max(0, d_j . omega_t), 0 <= 1e-6
    d64 = dirs.view(n, 4)[:, :3].double()
    om = torch.from_numpy(_texel_dirs64(np)).cuda()
    W = torch.clamp(d64 @ om.T, min=0.0)  # n x 64
    W = torch.where(W > 1e-6, W, torch.zeros_like(W))
    ref = (R32.double().reshape(3 * P, n) @ W) / W.sum(0)  # (3P) x 64
    ref = ref.reshape(3, dims[1], dims[2], dims[0], 8, 8)  # c, layer, z, x, ty, tx
    floor = 1e-6 * float(ref.mean())
    rows = (10 * (torch.arange(dims[1]).cuda()[:, None] * dims[2] + torch.arange(dims[2]).cuda()[None, :]))
    ri = (rows[:, :, None, None, None] + 1 + torch.arange(8).cuda()[None, None, None, :, None])
    ci = (10 * torch.arange(dims[0]).cuda()[None, None, :, None, None] + 1 + torch.arange(8).cuda()[None, None, None, None, :])
    ri, ci = torch.broadcast_tensors(ri, ci)

    # the oracle's check: a seeded 1 % subset of the probes, convolved by oracle.convolve in FP64 from the FP32
    # radiance and the device's FP32 lattice
    sub = np.sort(np.random.default_rng(0).choice(P, P // 100, replace=False))
    want_sub = _oracle_conv_blocks(R32[:, torch.from_numpy(sub).cuda(), :].double().cpu().numpy(),
                                   dirs.view(n, 4)[:, :3].double().cpu().numpy())

    def oracle_errors():
        return _rel_err_stats([(_atlas_blocks(atlas.cpu().numpy(), dims, sub), want_sub)])

    def errors():
        got = atlas[ri, ci, :3].permute(5, 0, 1, 2, 3, 4).double()
        e = ((got - ref).abs() / torch.clamp(ref.abs(), min=floor)).flatten()
        q = torch.quantile(e[torch.randperm(e.numel(), device="cuda")[:4_000_000]], 0.99).item()
        return {"max": float(e.max()), "p99": q, "mean": float(e.mean())}

    d0 = ddgi.grid_desc(dims, rays_per_probe=n, hysteresis=0.0)  # error runs: the atlas holds the result
    d = ddgi.grid_desc(dims, rays_per_probe=n, hysteresis=0.97)
    for name, fmt, dt in (("fp16", L.DDGI_ELEM_F16, torch.float16), ("bf16", L.DDGI_ELEM_BF16, torch.bfloat16)):
        r16 = R32.to(dt).contiguous()

        def tc(dd=d, r16=r16, fmt=fmt):
            ctx.check(lib.ddgi_convolve_tc_raw(ctx.handle, C.byref(dd), r16.data_ptr(), fmt, dirs.data_ptr(),
                                               atlas.data_ptr(), 0, dims[1], 0, stream))

        ms = _time_back_to_back(torch, tc, 20)
        prec[f"tc_{name}_ms"] = ms
        prec[f"tc_{name}_gbs"] = prec["algorithmic_bytes"] / ms / 1e6
        atlas.zero_()
        tc(dd=d0)
        torch.cuda.synchronize()
        prec[f"tc_{name}_rel_err"] = oracle_errors()
        prec[f"tc_{name}_rel_err_full_grid"] = errors()
        del r16
    bw, bh = 32, 16
    img = torch.ones((bh * dims[2] * dims[1], bw * dims[0], 4), device="cuda")
    p = torch.arange(P, device="cuda")
    j = torch.arange(n, device="cuda")
    rr = (p // dims[0])[:, None] * bh + (j // bw)[None, :]
    cc = (p % dims[0])[:, None] * bw + (j % bw)[None, :]
    for c in range(3):
        img[rr, cc, c] = R32[c]
    del R32, rr, cc

    def fp32(dd=d):
        assert lib.ddgi_convolve_raw(C.byref(dd), img.data_ptr(), dirs.data_ptr(), atlas.data_ptr(), 0, dims[1], 0,
                                     stream) == 0

    prec["fp32_cuda_core_ms"] = _time_back_to_back(torch, fp32, 10)
    atlas.zero_()
    fp32(dd=d0)
    torch.cuda.synchronize()
    prec["fp32_rel_err"] = oracle_errors()
    prec["fp32_rel_err_full_grid"] = errors()
    prec["tc_fp16_speedup_vs_fp32"] = prec["fp32_cuda_core_ms"] / prec["tc_fp16_ms"]
    prec["error_reference"] = ("*_rel_err: the FP64 oracle (oracle.convolve) on a seeded 1% probe subset "
                               f"({len(sub)} probes); *_rel_err_full_grid: every probe against the same formula "
                               "in FP64 on the device; floor 1e-6 x mean irradiance")
    prec["meets_1e-3"] = {k: prec[f"{k}_rel_err"]["max"] <= 1e-3 for k in ("tc_fp16", "tc_bf16", "fp32")}
    del img, atlas, ref, W
    torch.cuda.empty_cache()
    return prec


def measure_forms(ctx, scene, w, stream, only=None, bvh_width=8):
    """The other forms of the path, each bounded to a few seconds: the plain single-grid FP32 form and the
    tensor-core convolution on the same workload, the tensor-core convolution of the 65,536-probe / 512-ray
    precision workload, the 64-grid batched workload against its plain form, and a short serving run."""
    import ctypes as C

    import torch

    from anerend_gb300 import _lib as L
    from anerend_gb300 import ddgi, scenes

    lib = L.load()
    out = {}
    if only == "precision":
        return {"precision_tc": measure_precision(ctx, stream)}
    if only == "batched":
        return measure_batched(ctx, stream, serving=False)
    if only == "batched_launches":
        return batched_launches(ctx, stream)
    rays = w.probes * w.rays
    g = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis)

    def single(fr):
        g.update(scene, fr, stream)

    def frames1(f):
        return ddgi.FrameParams(camera_pos=scenes.camera(w, f), rotation=scenes.rotation(w.seed, f))

    tuned = dict(shadow_mode=1, ray_order=1, warp_probes=2, bvh_width=bvh_width)
    for name, tun in (("plain_fp32", dict(shadow_mode=0, ray_order=0, warp_probes=32, conv_mode=0, bvh_width=2)),
                      ("tuned_fp32", dict(tuned, conv_mode=0)),
                      ("tuned_tc_fp16", dict(tuned, conv_mode=1)),
                      ("tuned_tc_bf16", dict(tuned, conv_mode=2))):
        g.set_tuning(**tun)
        ms = _time_updates(torch, single, frames1, 5)
        out[f"single_grid_{name}"] = {"ms_per_update": ms, "rays_per_s": rays / ms * 1e3}
    g.close()
    out["single_grid_speedup_vs_plain"] = (out["single_grid_plain_fp32"]["ms_per_update"]
                                           / out["single_grid_tuned_fp32"]["ms_per_update"])
    # the reference's own formats: RGBA16F atlas and RGBA16F ray images, tuned, FP32 convolution
    g = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis, atlas_format=L.DDGI_FORMAT_RGBA16F,
                       options=L.DDGI_GRID_RAYS_RGBA16F)
    g.set_tuning(**dict(tuned, conv_mode=0))
    ms = _time_updates(torch, single, frames1, 5)
    out["single_grid_tuned_fp32_rgba16f"] = {"ms_per_update": ms, "rays_per_s": rays / ms * 1e3,
                                             "formats": "RGBA16F atlas and ray images (the reference's)"}
    g.close()

    out["precision_tc"] = measure_precision(ctx, stream)
    out["mirror"] = measure_mirror(ctx, scene, w, stream)
    out.update(measure_batched(ctx, stream, serving=True))
    return out


def measure_mirror(ctx, scene, w, stream):
    """The specular GI mirror pass (ddgi_mirror_reflections) on a 1920 x 1080 G-buffer of points on the workload's
    triangles (face normals, camera at the grid's camera, 1 in 23 sky pixels), device-resident, with the grid's
    atlas after two updates: ms per pass and reflected rays / s."""
    import torch

    from anerend_gb300 import _lib as L
    from anerend_gb300 import ddgi, scenes

    arrays = scene.arrays
    n = 1920 * 1080
    v = arrays.vertices["d0"][:, :3].astype(np.float64)
    tri = arrays.indices.reshape(-1, 3)
    u = [scenes.uniform(17, 960 + k, n) for k in range(3)]
    k = (u[0] * len(tri)).astype(np.int64) % len(tri)
    a, b = u[1].copy(), u[2].copy()
    flip = a + b > 1
    a[flip], b[flip] = 1 - a[flip], 1 - b[flip]
    pts = np.zeros(n, L.MIRROR_POINT)
    pts["position"] = (v[tri[k, 0]] * (1 - a - b)[:, None] + v[tri[k, 1]] * a[:, None] + v[tri[k, 2]] * b[:, None])
    pts["normal"] = np.cross(v[tri[k, 1]] - v[tri[k, 0]], v[tri[k, 2]] - v[tri[k, 0]])
    pts["sky"][::23] = 1.0
    dp = torch.from_numpy(pts.view(np.uint8).copy()).cuda()
    out = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    g = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis)
    try:
        for f in range(2):
            g.update(scene, ddgi.FrameParams(camera_pos=scenes.camera(w, f), rotation=scenes.rotation(w.seed, f)), stream)
        fp = ddgi.FrameParams(camera_pos=scenes.camera(w, 1))
        for _ in range(3):
            g.mirror_reflections(scene, fp, dp.data_ptr(), n, out.data_ptr(), stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 10
        e0.record()
        for _ in range(reps):
            g.mirror_reflections(scene, fp, dp.data_ptr(), n, out.data_ptr(), stream)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        hit = float((out[:, 3] < 1e6).logical_and(out[:, 3] > 0).float().mean())
    finally:
        g.close()
    return {"points": n, "ms": ms, "reflected_rays_per_s": n / ms * 1e3, "hit_fraction": hit}


def batched_launches(ctx, stream, updates=4):
    """A few eager updates of the 64-grid batched workload (FP16 tensor-core convolution, the autotuned launch
    shape of its last measurement), for a per-kernel launch list under ncu: the per-phase split of the batched
    form. Returns the CUDA-event time of the last update."""
    import torch

    from anerend_gb300 import ddgi, scenes

    bwl = scenes.BATCHED
    tris, specs = scenes.batch_layout(bwl)
    scs = [ddgi.Scene(ctx, scenes.build_scene_tris(t, 1000 + i, bwl.box_lo, bwl.box_hi)) for i, t in enumerate(tris)]
    grids = [ddgi.ProbeGrid(ctx, sp.dims, sp.step, sp.rays, sp.origin_y, sp.hysteresis) for sp in specs]
    batch = ddgi.Batch(ctx, [(g, scs[sp.scene]) for g, sp in zip(grids, specs)])
    batch.set_tuning(conv_mode=1, use_graph=0, bvh_width=8, refill_lanes=16, blocks_per_sm=8, warp_probes=4,
                     ray_order=1, shadow_mode=1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for f in range(updates):
        frames = [ddgi.FrameParams(camera_pos=sp.camera, rotation=scenes.rotation(i, f)) for i, sp in enumerate(specs)]
        e0.record()
        batch.update(frames, stream)
        e1.record()
    torch.cuda.synchronize()
    out = {"batched_launches": {"updates": updates, "last_update_ms": e0.elapsed_time(e1)}}
    batch.close()
    for g in grids:
        g.close()
    for sc in scs:
        sc.close()
    return out


def _batched_conv_error(ctx, stream, specs, scs, tuning, conv_mode, picks=8, probes_per_grid=256):
    """Per-texel error of a batched update's convolution against the FP64 oracle: hysteresis-0 copies of a
    seeded subset of the batched grids run two batched updates with `conv_mode`; on up to probes_per_grid
    seeded probes of each, the atlas texels are compared with oracle.convolve of the same traced FP32 radiance
    and lattice."""
    from anerend_gb300 import ddgi, scenes
    from oracle import oracle

    rng = np.random.default_rng(1)
    sel = sorted(int(i) for i in rng.choice(len(specs), picks, replace=False))
    grids = [ddgi.ProbeGrid(ctx, specs[i].dims, specs[i].step, specs[i].rays, specs[i].origin_y, 0.0) for i in sel]
    batch = ddgi.Batch(ctx, [(g, scs[specs[i].scene]) for g, i in zip(grids, sel)])
    batch.set_tuning(conv_mode=conv_mode, use_graph=0, **tuning)
    for f in range(2):
        batch.update([ddgi.FrameParams(camera_pos=specs[i].camera, rotation=scenes.rotation(i, f)) for i in sel],
                     stream)
    ctx.sync(stream)
    pairs = []
    for g, i in zip(grids, sel):
        X, Y, Z = specs[i].dims
        n = specs[i].rays
        rad, _, lat = g.download_rays()
        atlas = g.download_atlas()
        idx = np.sort(rng.choice(X * Y * Z, min(X * Y * Z, probes_per_grid), replace=False))
        x, z, layer = idx % X, (idx // X) % Z, idx // (X * Z)
        bw, bh = oracle.GridGeom(X, Y, Z, n).block
        j = np.arange(n)
        R = rad[((layer * Z + z) * bh)[:, None] + (j // bw)[None, :], (x * bw)[:, None] + (j % bw)[None, :], :3]
        want = _oracle_conv_blocks(R.astype(np.float64).transpose(2, 0, 1), lat[:, :3].astype(np.float64))
        pairs.append((_atlas_blocks(atlas, specs[i].dims, idx), want))
    batch.close()
    for g in grids:
        g.close()
    return _rel_err_stats(pairs)


def measure_batched(ctx, stream, serving=True):
    """The 64-grid batched workload against its plain one-grid-at-a-time form and, with `serving`, the serving
    loop over the same resident scenes."""
    import torch

    from anerend_gb300 import _lib as L
    from anerend_gb300 import ddgi, scenes

    out = {}
    # batched workload: 64 grids over 8 scenes, batched tensor-core form vs plain one-grid-at-a-time form
    bwl = scenes.BATCHED
    tris, specs = scenes.batch_layout(bwl)
    scs = [ddgi.Scene(ctx, scenes.build_scene_tris(t, 1000 + i, bwl.box_lo, bwl.box_hi)) for i, t in enumerate(tris)]
    grids = [ddgi.ProbeGrid(ctx, sp.dims, sp.step, sp.rays, sp.origin_y, sp.hysteresis) for sp in specs]
    items = [(gg, scs[sp.scene]) for gg, sp in zip(grids, specs)]
    brays = sum(sp.probes * sp.rays for sp in specs)

    def bframes(f):
        return [ddgi.FrameParams(camera_pos=sp.camera, rotation=scenes.rotation(i, f)) for i, sp in enumerate(specs)]

    for gg in grids:
        gg.set_tuning(shadow_mode=0, ray_order=0, warp_probes=32, conv_mode=0, bvh_width=2)

    def plain(fr):
        for (gg, sc), fp in zip(items, fr):
            gg.update(sc, fp, stream)

    plain_ms = _time_updates(torch, plain, bframes, 3)
    batch = ddgi.Batch(ctx, items)
    res_b = {"grids": len(specs), "scenes": len(tris), "triangles": sum(tris), "rays": brays,
             "probes": sum(sp.probes for sp in specs),
             "plain_fp32_ms": plain_ms, "plain_fp32_rays_per_s": brays / plain_ms * 1e3}
    # launch shape from the autotuner, timed on the FP16 tensor-core form (the trace dominates, so the shape
    # carries over to the other convolution modes)
    from anerend_gb300 import autotune

    batch.set_tuning(conv_mode=1, use_graph=1)
    tuned = autotune.tune_batch(batch, bframes, autotune.batch_signature(specs, tris), stream, reps=2, warmup=2,
                                use_cache=False)
    res_b["autotuned"] = {"tuning": tuned["tuning"], "trials": len(tuned["trials"]), "best_ms": tuned["ms"]}
    for name, conv in (("batched_fp32", 0), ("batched_tc_fp16", 1), ("batched_tc_bf16", 2)):
        batch.set_tuning(conv_mode=conv, use_graph=1, **tuned["tuning"])
        ms = _time_updates(torch, lambda fr: batch.update(fr, stream), bframes, 4)
        res_b[f"{name}_ms"] = ms
        res_b[f"{name}_rays_per_s"] = brays / ms * 1e3
        res_b[f"{name}_probe_updates_per_s"] = res_b["probes"] / ms * 1e3
    res_b["graph_launches"] = int(batch.stats.graphLaunches)
    batch.close()
    # the same grids one at a time with the batch's tuned launch shape and the FP16 tensor-core convolution,
    # so the gain of batching itself shows beside the gain of the tuned kernels
    for gg in grids:
        gg.set_tuning(conv_mode=1)
    res_b["tuned_per_grid_fp16_ms"] = _time_updates(torch, plain, bframes, 3)
    # the speed-up claim is made at the FP16 tensor-core form, whose per-texel error against the FP64 oracle
    # stays within 1e-3 (measured below); BF16 is reported beside it only
    res_b["speedup_batched_tc_vs_plain"] = plain_ms / res_b["batched_tc_fp16_ms"]
    res_b["speedup_batched_tc_vs_tuned_per_grid"] = res_b["tuned_per_grid_fp16_ms"] / res_b["batched_tc_fp16_ms"]
    res_b["speedup_batched_tc_bf16_vs_plain"] = plain_ms / res_b["batched_tc_bf16_ms"]
    res_b["speedup_mode"] = "FP16 tensor-core convolution (convMode 1)"
    res_b["conv_rel_err_vs_oracle"] = {
        name: _batched_conv_error(ctx, stream, specs, scs, tuned["tuning"], conv) for name, conv in
        (("tc_fp16", 1), ("tc_bf16", 2), ("fp32", 0))}
    res_b["conv_rel_err_vs_oracle"]["sample"] = ("8 seeded grids of the 64 (hysteresis 0 copies, 2 batched updates), "
                                                 "up to 256 seeded probes each, oracle.convolve in FP64 on the traced "
                                                 "FP32 radiance")
    out["batched"] = res_b
    for gg in grids:
        gg.close()
    for sc in scs:
        sc.close()
    ctx.sync(stream)
    if not serving:
        return out

    # serving: Poisson arrivals over the workload's 32 resident scenes (10k..1M triangles, log-uniform), at the
    # workload's 2,000 req/s and at lower rates down to 500 req/s, to find where the p99 latency crosses one
    # 30 Hz update period. One small request per scene first, untimed, so every scene's light-space shadow BVH
    # exists.
    sw = scenes.SERVING
    stris = scenes.serving_scene_tris(sw)
    scs = [ddgi.Scene(ctx, scenes.build_scene_tris(t, 2000 + i, bwl.box_lo, bwl.box_hi)) for i, t in enumerate(stris)]
    srv = ddgi.Server(ctx, sw.budget, max_batch=64, in_flight=2, conv_mode=1, max_batch_mrays=8)
    for sc in scs:
        srv.submit(sc, ddgi.grid_desc((4, 4, 4), rays_per_probe=64, hysteresis=0.97),
                   ddgi.FrameParams(camera_pos=(0.0, 0.0, 0.0), rotation=scenes.rotation(0, 0)))
    srv.drain(600.0)
    srv.close()
    serv = {"scenes": len(scs), "triangles": sum(stris), "triangles_min": min(stris), "triangles_max": max(stris),
            "conv_mode": "FP16 tensor cores", "policy": "shortest rays first, aging 50 ms", "in_flight": 2,
            "max_batch_mrays": 8, "baseline_policy": "arrival order (fifo_<rate>), same slots"}
    sjf_rates = (2000, 1000, 900, 850, 750, 650, 600, 500)
    runs = [(float(r), 1.5, L.DDGI_SERVE_FIFO, 2, f"fifo_{r}") for r in (2000, 1000, 750, 500)]
    runs += [(float(r), 1.5, L.DDGI_SERVE_SHORTEST_FIRST, 2, f"rate_{r}") for r in sjf_rates]
    for rate, dur, policy, slots, key in runs:
        reqs = scenes.serving_requests(sw, int(rate * dur), rate)
        srv = ddgi.Server(ctx, sw.budget, max_batch=64, in_flight=slots, conv_mode=1, max_batch_mrays=8,
                          policy=policy, aging_ms=50.0)
        t0 = time.perf_counter()
        for (ta, si, dms, rr, cam, k) in reqs:
            now = time.perf_counter() - t0
            if ta > now:
                time.sleep(ta - now)
            srv.submit(scs[si % len(scs)], ddgi.grid_desc(dms, rays_per_probe=rr, hysteresis=0.97),
                       ddgi.FrameParams(camera_pos=cam, rotation=scenes.rotation(k, 0)))
        srv.drain(600.0)
        wall = time.perf_counter() - t0
        st = srv.stats
        offered = sum(int(np.prod(dm)) * rr for (_, _, dm, rr, _, _) in reqs)
        serv[key] = {"requests": len(reqs), "completed": int(st.completed), "batches": int(st.batches),
                                     "offered_rays_per_s": offered / max(reqs[-1][0], 1e-9),
                                     "served_rays_per_s": st.rays / wall, "p50_ms": st.p50LatencyMs,
                                     "p99_ms": st.p99LatencyMs, "peak_gb": st.peakBytes / 2**30}
        srv.close()
    # the knee: the highest offered rate (of those run, shortest first) whose p99 stays within one 30 Hz period
    ok = [r for r in sjf_rates if serv[f"rate_{r}"]["p99_ms"] < 33.0]
    serv["knee_req_per_s"] = max(ok) if ok else None
    out["serving"] = serv
    for sc in scs:
        sc.close()
    ctx.sync(stream)
    return out


def run_ours(args, rank, local, world):
    import torch

    from anerend_gb300 import _lib as L
    from anerend_gb300 import ddgi, scenes

    torch.cuda.set_device(local)
    w = scenes.SINGLE_GRID
    arrays = scenes.build_scene(w)
    ctx = ddgi.Context(local)
    scene = ddgi.Scene(ctx, arrays)
    stream = torch.cuda.current_stream().cuda_stream

    # hit fraction of the workload's rays (for the algorithmic bytes), from one recorded trace
    probe_grid = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis,
                                options=L.DDGI_GRID_RECORD_HITS)
    probe_grid.trace(scene, ddgi.FrameParams(rotation=scenes.rotation(w.seed, 0)), stream)
    ctx.sync(stream)
    _, hits, _ = probe_grid.download_rays(hits=True)
    hit_frac = float((hits >= 0).mean())
    probe_grid.close()

    grid = ddgi.ProbeGrid(ctx, w.dims, w.step, w.rays, w.origin_y, w.hysteresis)
    grid.set_tuning(warp_probes=args.warp_probes, ray_order=1, shadow_mode=1, conv_mode=0, bvh_width=args.bvh_width,
                    refill_lanes=args.refill_lanes)  # FP32 throughout
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > L2 (129 MB)
    rays_per_step = w.probes * w.rays

    def frame(f):
        return ddgi.FrameParams(camera_pos=scenes.camera(w, f), rotation=scenes.rotation(w.seed, f))

    f = 0
    for _ in range(args.warmup):
        grid.update(scene, frame(f), stream)
        f += 1
    torch.cuda.synchronize()

    # ---- device-timed steps (per-phase events on the launching stream, L2 flushed between steps) ----
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
    launches = 0
    sampler = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    sampler.start()
    t_region0 = time.time()
    t_wall0 = time.perf_counter()
    for s in range(args.steps):
        flush.zero_()
        fp = frame(f)
        e = ev[s]
        e[0].record()
        moved = grid.translate(fp.camera_pos, stream)
        e[1].record()
        grid.trace(scene, fp, stream)
        e[2].record()
        grid.convolve(fp, stream)
        e[3].record()
        # lattice, seed map, closest hit, shade, shadow, shadow resolve, weights, convolve (+ translate)
        launches += 8 + (1 if moved else 0)
        f += 1
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall0
    t_region1 = time.time()
    barrier(world)
    clocks = sampler.stop(t_region0, t_region1)
    ctx.sync(stream)
    step_ms = [e[0].elapsed_time(e[3]) for e in ev]
    trace_ms = [e[1].elapsed_time(e[2]) for e in ev]
    conv_ms = [e[2].elapsed_time(e[3]) for e in ev]
    total_ms = max_over_ranks(sum(step_ms), world)
    ms_per_step = total_ms / args.steps
    value = world * rays_per_step * args.steps / (total_ms / 1e3)

    # ---- end to end through the C ABI: host frame in, atlas out into pinned host memory ----
    # Per step: ddgi_update, then a wait for the previous step's atlas to reach the host, then this step's
    # readback started behind its update (ddgi_atlas_download_async), so each readback runs during the next
    # update. Every step's atlas is on the host before the timed region ends.
    nb = grid.buffers.atlasBytes
    atlas_host = [torch.empty(nb // 4, dtype=torch.float32).pin_memory() for _ in range(2)]
    lib = L.load()
    fps = [frame(f + s).to_c() for s in range(args.steps)]
    f += args.steps
    ctx.sync(stream)
    barrier(world)
    t0 = time.perf_counter()
    for s in range(args.steps):
        ctx.check(lib.ddgi_update(grid.handle, scene.handle, fps[s], stream))
        if s:
            ctx.check(lib.ddgi_atlas_download_wait(grid.handle))
        ctx.check(lib.ddgi_atlas_download_async(grid.handle, atlas_host[s & 1].data_ptr(), nb, stream))
    ctx.check(lib.ddgi_atlas_download_wait(grid.handle))
    e2e_total = max_over_ranks(time.perf_counter() - t0, world)
    e2e_value = world * rays_per_step * args.steps / e2e_total
    # the same with the blocking readback (ddgi_atlas_download returns once the atlas is on the host)
    e2e_times = []
    barrier(world)
    for s in range(args.steps):
        fp = frame(f).to_c()
        t0 = time.perf_counter()
        ctx.check(lib.ddgi_update(grid.handle, scene.handle, fp, stream))
        ctx.check(lib.ddgi_atlas_download(grid.handle, atlas_host[0].data_ptr(), nb, stream))
        e2e_times.append(time.perf_counter() - t0)
        f += 1
    e2e_blocking = world * rays_per_step * args.steps / max_over_ranks(sum(e2e_times), world)

    peaks = load_peaks()
    trace_avg_s = sum(trace_ms) / len(trace_ms) / 1e3
    alg_bytes = rays_per_step * (hit_frac * BYTES_PER_HIT + (1 - hit_frac) * BYTES_PER_MISS)
    achieved = alg_bytes / trace_avg_s / 1e9
    # DRAM bytes of one trace launch: copied from the ncu capture of the same kernels on the same workload that
    # profiles/trace_wavefront_single_grid.md summarises (ncu does not run inside the bench), so it is not a
    # figure of this run; the line says so in roofline.traffic_source
    traffic = None
    tp = ROOT / "profiles" / "trace_wavefront_single_grid.md"
    if tp.exists():
        import re

        m = re.search(r"^traffic_bytes_per_launch:\s*(\d+)", tp.read_text(), re.M)
        traffic = int(m.group(1)) if m else None
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        frames = 4
        v, dt, cores = cpu_sample(w, arrays, frames)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{frames} full probe updates ({frames * rays_per_step} rays), FP64 oracle, {dt:.1f} s"}
        # the CPU reference workload run in full (8x4x8 probes, 64 rays, 4,098 triangles, all 8 frames)
        w1 = scenes.CPU_REFERENCE
        v1, dt1, _ = cpu_sample(w1, scenes.build_scene(w1), w1.frames)
        cpu["cpu_reference_workload_full"] = {"value": v1, "unit": UNIT, "frames": w1.frames,
                                              "rays": w1.frames * w1.probes * w1.rays, "seconds": dt1}
    forms = None
    if rank == 0 and world == 1 and not args.no_extras:
        forms = measure_forms(ctx, scene, w, stream, bvh_width=args.bvh_width)
    if rank == 0:
        srt = sorted(step_ms)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": w.name, "probes": w.probes, "grid": list(w.dims), "rays_per_probe": w.rays,
                       "triangles": w.num_tris, "materials": 1024, "atlas": "RGBA32F", "hysteresis": w.hysteresis,
                       "camera": "+1 x every 10 frames", "l2": "flushed between steps (256 MB write)",
                       "parallelism": f"replicas x{world}"},
            "probe_updates_per_s": value / w.rays,
            "p50_ms": srt[len(srt) // 2], "p99_ms": srt[min(len(srt) - 1, int(0.99 * len(srt)))],
            "phase_ms": {"trace_shade": sum(trace_ms) / len(trace_ms), "convolve": sum(conv_ms) / len(conv_ms),
                         "translate_and_lattice": sum(e[0].elapsed_time(e[1]) for e in ev) / len(ev)},
            "hit_fraction": hit_frac,
            "wall_s": wall,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 116,
                    "d2h_bytes_per_step": int(grid.buffers.atlasBytes),
                    "readback": "ddgi_atlas_download_async, overlapping the next update",
                    "blocking_readback_value": e2e_blocking},
            "roofline": {"kernel": "trace (k_trace_closest + k_shade + k_trace_shadow + k_shadow_resolve)", "bound": "hbm",
                         "achieved": achieved,
                         "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                         "traffic": traffic,
                         "traffic_source": "copied from the ncu capture in profiles/trace_wavefront_single_grid.md, "
                                           "not measured in this run",
                         "peak_source": peaks["source"],
                         "algorithmic_bytes_per_launch": alg_bytes},
            "cpu_baseline": cpu,
            "gpu_launches": launches,
            "clocks": clocks,
            "tuning": {"warpProbes": int(grid.tuning.warpProbes), "rayOrder": int(grid.tuning.rayOrder),
                       "shadowMode": int(grid.tuning.shadowMode), "convMode": int(grid.tuning.convMode),
                       "bvhWidth": int(grid.tuning.bvhWidth), "refillLanes": int(grid.tuning.refillLanes)},
            "forms": forms,
        }
        print(json.dumps(line))
    grid.close()
    scene.close()
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # 600 updates are about 1 s of device time: enough 200 ms clock samples inside the timed region
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the other forms (batched, precision, serving)")
    ap.add_argument("--form", choices=["precision", "batched", "batched_launches"],
                    help="run only this form and print its measurements (batched_launches: four eager batched updates, "
                         "for an ncu launch list)")
    ap.add_argument("--bvh-width", type=int, default=8, choices=[2, 8], help="traversal tree (8-wide or binary)")
    ap.add_argument("--refill-lanes", type=int, default=8, help="idle lanes before a traversal warp refills (1..32)")
    ap.add_argument("--warp-probes", type=int, default=2, help="probes per traversal warp (1, 2, 4, ... 32)")
    args = ap.parse_args()
    rank, local, world = dist_init()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        from anerend_gb300 import build

        if rank == 0:
            build.build()
        barrier(world)
        if args.form:
            import torch

            from anerend_gb300 import ddgi

            torch.cuda.set_device(local)
            with ddgi.Context(local) as ctx:
                print(json.dumps(measure_forms(ctx, None, None, torch.cuda.current_stream().cuda_stream, args.form)))
        else:
            run_ours(args, rank, local, world)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
