"""Pins the oracle restatement to the reference's own shader code.

The reference's irradiance_probe_update.rgen / .rchit / .rmiss and probe_conv.comp, compiled from their
sources as FP64 C++ (oracle/ref_shader), run on the seeded pin workload (oracle/ref_shader/pin_workload.py:
the reference's 64 x 8 x 64 / 256-ray grid, a 3,000-triangle scene, a camera-relative frame and a bake-tile
frame, interior probes and the +x / +z corner probes whose lookups wrap). Which triangle a ray hits comes
from the oracle's exact closest hit on both sides (the reference's own hit is made by closed RT hardware),
so the comparison covers ray generation, hit reconstruction, shading, the shadow-ray decision, the
previous-frame probe lookup with its REPEAT wrap, the miss shader and the convolution.

Tolerances: traced radiance and directions within 1e-10 relative (both sides FP64, the orders of operations
differ); convolved texels within 1e-12 relative. Floating literals are read at their decimal value on both
sides (the convolution is given the hysteresis 0.96 as a double); the shader itself rounds its literals to
float32, which moves the golden-angle lattice by up to about 3e-5 rad at 256 rays, a deviation the product
shares with the oracle (its lattice is FP64 from the decimal constants).

The committed fixture tests/golden/ref_shader_pin.npz (tests/golden/make_ref_shader_golden.py) holds the
reference code's outputs, so the oracle is pinned on machines without the reference sources too; where they
are present, the fixture is also regenerated and must match bit for bit.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "tests" / "golden"))

from anerend_gb300 import _lib as L  # noqa: E402
from oracle import oracle  # noqa: E402
from oracle.ref_shader import pin_workload as W  # noqa: E402

FIXTURE = ROOT / "tests" / "golden" / "ref_shader_pin.npz"


def rel(a, b, floor=1e-9):
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


@pytest.fixture(scope="module")
def oracle_outputs():
    """The oracle on the pin workload: traced layer per frame and the convolved atlases."""
    import make_ref_shader_golden as G

    arrays = W.scene_arrays()
    osc = oracle.OracleScene(arrays, L.SceneDesc)
    prev = W.atlas_prev()
    out = {}
    try:
        for name, fp, layer in W.frames():
            f = fp.to_c()
            og = oracle.OracleGrid(W.grid_desc())
            og.atlas[:] = prev
            og.trace(osc, f)
            rows = slice(layer * 1024, (layer + 1) * 1024)
            for k, (x0, y0, x1, y1) in enumerate(W.TRACE_RECTS):
                out[f"{name}/trace{k}/radiance"] = og.ray_rad[rows][y0:y1, x0:x1, :3].copy()
                j = (np.arange(y1 - y0)[:, None] % 16) * 16 + (np.arange(x1 - x0)[None, :] % 16)
                out[f"{name}/trace{k}/direction"] = og.dirs[j]
                out[f"{name}/trace{k}/uncertain"] = og.uncertain[rows][y0:y1, x0:x1].copy()
            irr_img, _, dirs = W.conv_inputs(fp.rotation)
            rr = np.zeros_like(og.ray_rad)
            rr[rows] = irr_img
            atlas = prev.copy()
            oracle.convolve(W.grid_desc(), rr, dirs, atlas, layer, layer + 1, f.flags, hysteresis=W.HYSTERESIS)
            for k, rect in enumerate(W.CONV_RECTS):
                out[f"{name}/conv{k}/texels"] = np.stack([G.interior(atlas, layer, px, pz)
                                                         for px, pz in G.conv_probes(rect)])
    finally:
        osc.close()
    return out


def test_fixture_exists_and_is_small():
    assert FIXTURE.exists(), "run tests/golden/make_ref_shader_golden.py where the reference sources are present"
    assert FIXTURE.stat().st_size < 700_000


@pytest.mark.parametrize("frame", ["camera_relative", "bake_tile"])
def test_oracle_matches_reference_code_fixture(oracle_outputs, frame):
    gold = np.load(FIXTURE)
    for k in range(len(W.TRACE_RECTS)):
        key = f"{frame}/trace{k}"
        assert np.max(rel(oracle_outputs[key + "/radiance"], gold[key + "/radiance"])) <= 1e-10, key
        assert np.max(np.abs(oracle_outputs[key + "/direction"] - gold[key + "/direction"])) <= 1e-12, key
        # the oracle decides every ray here without an FP32 ambiguity, so nothing is excused
        assert oracle_outputs[key + "/uncertain"].mean() < 0.01
    for k in range(len(W.CONV_RECTS)):
        key = f"{frame}/conv{k}/texels"
        assert np.max(rel(oracle_outputs[key], gold[key])) <= 1e-12, key
    # the workload exercises hits and misses on both frames
    rad = np.concatenate([gold[f"{frame}/trace{k}/radiance"].reshape(-1, 3) for k in range(len(W.TRACE_RECTS))])
    c = np.float32([0.4, 0.5, 0.7]).astype(np.float64)  # toLinear(skyIntensity * skyColor), rmiss:20
    sky = np.where(c < 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4)
    missed = np.all(np.abs(rad - sky) <= 1e-12, axis=1)
    assert 0.05 < missed.mean() < 0.95


@pytest.mark.parametrize("frame", ["ddgi_on", "ddgi_off"])
def test_gbuffer_pass_oracles_match_reference_code_fixture(frame):
    """The oracle's restatements of the other passes against the reference's own stages (mirror_reflections.rgen
    / .rchit / .rmiss, shadow.rgen / .rchit / .rmiss, the DDGI block of deferred_tiled.comp's doLight), on the
    same scene, atlas and seeded G-buffer points; hits are the oracle's exact closest hits on both sides."""
    gold = np.load(FIXTURE)
    arrays = W.scene_arrays()
    fp = dict(W.pass_frames())[frame]
    f = fp.to_c()
    prev = W.atlas_prev()
    osc = oracle.OracleScene(arrays, L.SceneDesc)
    try:
        mpts = W.mirror_points(arrays)
        got, unc = oracle.mirror_reflections(osc, W.grid_desc(), f, prev, mpts)
        want = gold[f"{frame}/mirror"]
        assert np.max(rel(got, want)) <= 1e-10
        sky = mpts["sky"] != 0
        assert np.all(want[sky] == 0.0) and 0.1 < np.mean(want[~sky, 3] < 1e6) < 0.99  # hits and misses
        # the RT shadow pass: a ray along -lightDir over [0.1, 50]; lit (1) on a miss, 0 on a hit, sky pixels 1
        spts = W.shadow_points(arrays)
        d = -np.array(f.lightDir[:], np.float64)
        lit = np.array([1.0 if p[3] != 0 or osc.closest_hit(p[:3].astype(np.float64), d)[0] < 0 else 0.0
                        for p in spts])
        assert np.array_equal(lit, gold[f"{frame}/shadow"])
        assert 0.01 < gold[f"{frame}/shadow"].mean() < 0.99  # shadowed and lit points
        # the deferred pass's ambient term of its DDGI block (CLAMP_TO_EDGE sampler, far points use the sky term)
        qpts = W.surface_points()
        got = oracle.query_irradiance(W.grid_desc(), f, prev, qpts)
        assert np.max(rel(got, gold[f"{frame}/consumer"])) <= 1e-10
    finally:
        osc.close()


def test_fixture_regenerates_from_reference_sources():
    """Where the reference sources are present the fixture is rebuilt from the compiled shader code and must
    equal the committed one bit for bit."""
    from oracle.ref_shader import build_if_available

    if build_if_available() is None:
        pytest.skip("reference shader sources not present on this machine")
    import make_ref_shader_golden as G

    fresh = G.generate()
    gold = np.load(FIXTURE)
    assert sorted(fresh) == sorted(gold.files)
    for k, v in fresh.items():
        assert np.array_equal(v, gold[k]), k
