"""Writes tests/golden/ref_shader_pin.npz: outputs of the reference's own DDGI shader code (irradiance_probe
_update.rgen / .rchit / .rmiss and probe_conv.comp; mirror_reflections.rgen / .rchit / .rmiss; shadow.rgen /
.rchit / .rmiss; deferred_tiled.comp's doLight; compiled as FP64 C++ by oracle/ref_shader/build_ref.py from the
reference sources) on the seeded pin workload of oracle/ref_shader/pin_workload.py.

Run where the reference sources are present:  python tests/golden/make_ref_shader_golden.py
Per frame (camera_relative, bake_tile) it stores, for every compared rectangle, the traced radiance and
direction texels (RGB, FP64) and the convolved 8 x 8 interior texels (RGBA, FP64) of the rectangle's
probes; per G-buffer pass frame (DDGI flag on, off) the mirror pass's (radiance, distance), the shadow pass's
visibility and the deferred DDGI block's ambient term of the workload's points. The oracle is checked against
this file by tests/test_oracle_vs_reference_shaders.py on any machine.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

OUT = Path(__file__).resolve().parent / "ref_shader_pin.npz"


def conv_probes(rect):
    x0, y0, x1, y1 = rect
    return [(px, pz) for pz in range(y0 // 8, y1 // 8) for px in range(x0 // 8, x1 // 8)]


def interior(atlas, layer, px, pz, Z=64):
    ty, tx = 10 * Z * layer + 10 * pz + 1, 10 * px + 1
    return atlas[ty:ty + 8, tx:tx + 8]


def generate() -> dict:
    from oracle.ref_shader import RefShaders
    from oracle.ref_shader import pin_workload as W

    arrays = W.scene_arrays()
    desc = W.scene_desc(arrays)
    ref = RefShaders()
    ref.set_scene(desc)
    prev = W.atlas_prev()
    out = {}
    for name, fp, layer in W.frames():
        f = fp.to_c()
        for k, rect in enumerate(W.TRACE_RECTS):
            irr, dirs = ref.trace(f, fp.rotation, layer, prev, *rect)
            out[f"{name}/trace{k}/radiance"] = irr[..., :3].copy()
            out[f"{name}/trace{k}/direction"] = dirs[..., :3].copy()
        irr_img, dir_img, _ = W.conv_inputs(fp.rotation)
        atlas = prev.copy()
        for k, rect in enumerate(W.CONV_RECTS):
            ref.convolve(f, layer, irr_img, dir_img, atlas, *rect)
            out[f"{name}/conv{k}/texels"] = np.stack([interior(atlas, layer, px, pz) for px, pz in conv_probes(rect)])
    mpts, spts, qpts = W.mirror_points(arrays), W.shadow_points(arrays), W.surface_points()
    for name, fp in W.pass_frames():
        f = fp.to_c()
        out[f"{name}/mirror"] = ref.mirror(f, prev, mpts)
        out[f"{name}/shadow"] = ref.shadow_mask(f, spts)
        out[f"{name}/consumer"] = ref.query_irradiance(f, prev, qpts)
    return out


if __name__ == "__main__":
    data = generate()
    np.savez_compressed(OUT, **data)
    print(OUT, sum(v.nbytes for v in data.values()), "bytes")
