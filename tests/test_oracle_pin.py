"""Pins the C oracle against the reference's own code.

* "ieee" mode vs the reference kernels compiled for the host (golden fixtures made by
  tests/golden/make_golden.py host): every plane bit-exact.
* "fma" mode vs the reference kernels compiled by nvcc for sm_103a and run on a GB300
  (tests/golden/ref_gpu.npz, made by make_golden.py gpu): hit, primitive, t and normal
  bit-exact; RGBA8 within 1 LSB and float RGBA within 2e-6 (powf differs between the
  host and device libraries).
* Live comparison against the host build when the reference sources are present.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, load_cases, scene_text, ulp_equal

HOST_CASES = load_cases(GOLDEN / "ref_host.npz")
GPU_NPZ = GOLDEN / "ref_gpu.npz"
GPU_CASES = load_cases(GPU_NPZ) if GPU_NPZ.exists() else {}


def _render(oracle, case, g, mode, thf=None):
    nodes, prims = oracle.parse(scene_text(case))
    w, h = (int(v) for v in g["size"])
    return oracle.render(nodes, prims, g["camera"], g["light"], w, h, mode=mode, tan_half_fov=thf)


@pytest.mark.parametrize("case", sorted(HOST_CASES))
def test_oracle_ieee_matches_reference_host_build(oracle, case):
    g = HOST_CASES[case]
    out = _render(oracle, case, g, "ieee")
    assert (out["hit"] == g["hit"]).all()
    m = g["hit"] == 1
    assert (out["prim"][m] == g["prim"][m]).all()
    assert ulp_equal(out["t"][m], g["t"][m]).all()
    assert ulp_equal(out["normal"][m], g["normal"][m]).all()
    assert (out["rgba8"] == g["rgba8"]).all()
    assert out["capped"] == 0


@pytest.mark.skipif(not GPU_CASES, reason="reference GPU fixtures not generated yet")
@pytest.mark.parametrize("case", sorted(GPU_CASES))
def test_oracle_fma_matches_reference_cuda_kernel(oracle, case):
    g = GPU_CASES[case]
    out = _render(oracle, case, g, "fma", thf=float(g["thf"][0]))
    assert (out["hit"] == g["hit"]).all()
    m = g["hit"] == 1
    assert (out["prim"][m] == g["prim"][m]).all()
    assert ulp_equal(out["t"][m], g["t"][m]).all()
    assert ulp_equal(out["normal"][m], g["normal"][m]).all()
    d = np.abs(out["rgba8"].view(np.uint8).astype(int) - g["rgba8"].view(np.uint8).astype(int))
    assert d.max() <= 1
    if "rgba_hit" in g:
        assert np.abs(out["rgba"][m] - g["rgba_hit"]).max(initial=0) <= 2e-6


def test_oracle_parse_matches_reference_parser(oracle):
    data = np.load(GOLDEN / "ref_parse.npz")
    stems = sorted({k.split("/")[0] for k in data.files})
    assert len(stems) == 21
    for stem in stems:
        nodes, prims = oracle.parse((GOLDEN / "scenes" / f"{stem}.txt").read_bytes())
        assert (nodes.view(np.uint8).ravel() == data[f"{stem}/nodes"].ravel()).all(), stem
        assert (prims.view(np.uint8).ravel() == data[f"{stem}/prims"].ravel()).all(), stem


def test_oracle_camera_matches_reference(oracle):
    data = np.load(GOLDEN / "ref_camera.npz")
    eq = lambda a, b: (np.asarray(a, np.float32).view(np.uint32) == np.asarray(b, np.float32).view(np.uint32)).all()
    assert eq(oracle.camera(), data["default"])
    assert eq(oracle.camera(fov_deg=60), data["fov60"])
    assert eq(oracle.camera(position=(1, 2, 3), rotation=(0.3, -1.2), fov_deg=45), data["posrot"])
    assert eq(oracle.camera(rotation=(2.0, 7.0)), data["clamped"])
    c = oracle.camera_move(oracle.camera_rotate(oracle.camera(fov_deg=75), 0.21, -0.33), 0.7, -0.4, 0.25)
    assert eq(c, data["moved"])
    for i in range(16):
        a = data[f"lookat{i}/args"]
        assert eq(oracle.camera(position=a[:3], rotation=a[3:5], fov_deg=60), data[f"lookat{i}"])
    assert eq(oracle.light_dir(), data["light_default"])
    assert eq(oracle.light_dir(0.4, 1.1), data["light_custom"])


def test_oracle_ieee_live_vs_reference_host():
    """Seeded synthetic scenes of every configuration, rendered by both (where the
    reference sources are present)."""
    from oracle import Oracle, RefHost, quantize_rgba8
    if not RefHost.available():
        pytest.skip("reference host build not present")
    from csgrt import scenes
    import csgrt
    O, R = Oracle(), RefHost()
    rng = np.random.default_rng(3)
    texts = [scenes.write_text(scenes.wikipedia_tree()), scenes.write_text(scenes.cheese_tree(5, 128))]
    texts += [scenes.write_text(scenes.random_tree(s, 2, 600, 12)) for s in range(6)]
    for text in texts:
        cam = csgrt.Camera.look_at_origin(scenes.seeded_direction(rng), 3.5).floats()
        light = csgrt.light_dir()
        on, op = O.parse(text)
        rn, rp = R.parse(text)
        a = O.render(on, op, cam, light, 80, 60, mode="ieee")
        b = R.render(rn, rp, cam, light, 80, 60)
        m = b["hit"] == 1
        assert (a["hit"] == b["hit"]).all()
        assert (a["prim"][m] == b["prim"][m]).all()
        assert ulp_equal(a["t"][m], b["t"][m]).all()
        assert ulp_equal(a["normal"][m], b["normal"][m]).all()
        assert (a["rgba8"] == quantize_rgba8(b["rgba"])).all()


def test_oracle_counts_and_fma_mode_are_consistent(oracle):
    """The two arithmetic modes differ only in the last bits: hit masks agree on almost
    every pixel, and the work counters are plausible."""
    from csgrt import scenes
    nodes, prims = oracle.parse(scenes.write_text(scenes.cheese_tree(1, 64)))
    cam = oracle.camera(position=(0.5, 0.7, 3.6), rotation=(-0.19, 0.14), fov_deg=60)
    light = oracle.light_dir()
    a = oracle.render(nodes, prims, cam, light, 64, 48, mode="ieee", counts=True)
    b = oracle.render(nodes, prims, cam, light, 64, 48, mode="fma")
    assert (a["hit"] != b["hit"]).mean() < 0.01
    c = a["counts"]
    assert (c["iters"] >= 1).all()
    assert c["aabb"].sum() >= 2 * c["iters"].astype(np.int64).sum() // 4
    assert (c["aabb"] % 2 == 0).all()


def test_oracle_f64_states_the_fp32_error(oracle):
    """The FP64 restatement agrees with the FP32 ("fma" = engine = reference kernel) results
    on hit and primitive for these samples, and bounds their t and normal error."""
    from csgrt import scenes
    from report_f64_errors import error_stats
    for text, view in ((scenes.config_scene_text(1), scenes.config_views(1)[0]),
                       (scenes.config_scene_text(3, 0), scenes.config_views(3, 0)[0])):
        s = error_stats(oracle, text, view, 320, 180, n_pix=1500)
        assert s["hit_mismatch"] <= 2 and s["prim_mismatch"] <= 2, s
        assert s["t_rel_p99"] < 1e-4 and s["normal_p99"] < 1e-3, s
        assert s["rgba8_max"] <= 1, s


def test_oracle_ieee_random_tree_sweep_vs_reference_host():
    """150 seeded random trees of up to 2,048 leaves (sphere, cylinder and cube leaves,
    all three operators, depth <= 12) from random look-at views: the oracle's ieee mode and
    the reference's host build agree on every plane, float RGBA included."""
    from oracle import Oracle, RefHost
    if not RefHost.available():
        pytest.skip("reference host build not present")
    from csgrt import scenes
    import csgrt
    O, R = Oracle(), RefHost()
    rng = np.random.default_rng(12)
    light = csgrt.light_dir()
    hits = 0
    for s in range(150):
        text = scenes.write_text(scenes.random_tree(30000 + s, 2, 2048, 12))
        cam = csgrt.Camera.look_at_origin(scenes.seeded_direction(rng), float(rng.uniform(2.5, 4.0))).floats()
        on, op = O.parse(text)
        rn, rp = R.parse(text)
        a = O.render(on, op, cam, light, 32, 24, mode="ieee")
        b = R.render(rn, rp, cam, light, 32, 24)
        m = b["hit"] == 1
        assert (a["hit"] == b["hit"]).all(), s
        assert (a["prim"][m] == b["prim"][m]).all(), s
        assert ulp_equal(a["t"][m], b["t"][m]).all(), s
        assert ulp_equal(a["normal"][m], b["normal"][m]).all(), s
        assert ulp_equal(a["rgba"], b["rgba"]).all(), s
        hits += int(m.sum())
    assert hits > 3000
