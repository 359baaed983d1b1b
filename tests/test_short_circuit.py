"""The engine's operator short-circuit, checked on the CPU against the reference's own
algorithm: the oracle renders random trees (depth <= 12, so no stack can overflow) with and
without the rule -- a Difference whose left child, or an Intersection with a child, is a
Miss known at GoTo, and a Difference / Intersection whose left subtree returned a Miss, go
straight to Compute -- and every plane is the same, bit for bit, while the iteration count
falls."""
from __future__ import annotations

import numpy as np


def _render(oracle, text, cam, light, w, h, sc):
    nodes, prims = oracle.parse(text)
    oracle.set_short_circuit(sc)
    try:
        thf = oracle.tan_half_fov(float(cam[5]))
        return oracle.render(nodes, prims, cam, light, w, h, mode="fma", tan_half_fov=thf,
                             want=("hit", "t", "prim", "normal", "rgba8"), counts=True)
    finally:
        oracle.set_short_circuit(False)


def test_short_circuit_keeps_every_plane(csg, oracle):
    from csgrt import scenes
    rng = np.random.default_rng(42)
    light = np.float32(csg.light_dir())
    iters = [0, 0]
    hits = 0
    w, h = 48, 36
    for seed in range(24):
        leaves = int(np.exp(rng.uniform(np.log(2), np.log(600))))
        text = scenes.write_text(scenes.random_tree(7000 + seed, 2, leaves, 12))
        cam = csg.Camera.look_at_origin(scenes.seeded_direction(rng), float(rng.uniform(2.5, 4.0))).floats()
        ref = _render(oracle, text, cam, light, w, h, False)
        sc = _render(oracle, text, cam, light, w, h, True)
        assert ref["capped"] == 0 and sc["capped"] == 0
        for k in ("hit", "t", "prim", "normal", "rgba8"):
            a, b = ref[k], sc[k]
            if k in ("t", "normal"):
                a, b = a.view(np.uint32), b.view(np.uint32)
            if k == "prim":  # defined only where the ray hits
                a, b = np.where(ref["hit"] != 0, a, -1), np.where(sc["hit"] != 0, b, -1)
            assert np.array_equal(a, b), (seed, k)
        iters[0] += int(ref["counts"]["iters"].sum())
        iters[1] += int(sc["counts"]["iters"].sum())
        hits += int(ref["hit"].sum())
    assert hits > 300  # the frames see surfaces (many random trees are empty sets)
    assert iters[1] < iters[0]  # the rule skips work


def test_short_circuit_is_off_by_default(csg, oracle):
    """The oracle is the reference's algorithm unless a test switches the rule on."""
    from csgrt import scenes
    text = scenes.write_text(scenes.random_tree(91, 2, 200, 12))
    cam = csg.Camera.look_at_origin(scenes.seeded_direction(np.random.default_rng(3)), 3.0).floats()
    light = np.float32(csg.light_dir())
    nodes, prims = oracle.parse(text)
    thf = oracle.tan_half_fov(float(cam[5]))
    a = oracle.render(nodes, prims, cam, light, 24, 18, mode="fma", tan_half_fov=thf, want=("hit",), counts=True)
    b = _render(oracle, text, cam, light, 24, 18, False)
    assert np.array_equal(a["counts"]["iters"], b["counts"]["iters"])
