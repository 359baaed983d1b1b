"""The engine's single-leaf shortcut (trace.cuh child_test), checked on the CPU against
the reference's own traversal: the oracle renders seeded random trees, cheese scenes and
the benchmark frames with and without the rule (on top of the live-leaf pruning and the
operator short-circuit), and every plane is the same, bit for bit, while the iterations
fall.  The rule: an operator child of at most 256 leaves with exactly one live leaf is not
descended into; its result is that leaf's own (tested with its box) when every operator on
the path down to it is a Union or a Difference entered on its left, and a Miss otherwise."""
from __future__ import annotations

import numpy as np

from test_live_pruning import _differ

PLANES = ("hit", "t", "prim", "normal", "rgba8")
SHORTCUT_LEAVES = 256  # the engine's kShortcutLeaves


def _render(oracle, nodes, prims, cam, light, w, h, shortcut, sc=True, pix=None):
    oracle.set_live_pruning(4)
    oracle.set_short_circuit(sc)
    oracle.set_leaf_shortcut(SHORTCUT_LEAVES if shortcut else 0)
    try:
        thf = oracle.tan_half_fov(float(cam[5]))
        if pix is not None:
            return oracle.render_list(nodes, prims, cam, light, w, h, pix, mode="fma", tan_half_fov=thf,
                                      want=("hit", "t", "prim", "normal", "rgba8"), counts=True)
        return oracle.render(nodes, prims, cam, light, w, h, mode="fma", tan_half_fov=thf, want=PLANES,
                             counts=True)
    finally:
        oracle.set_live_pruning(0)
        oracle.set_short_circuit(False)
        oracle.set_leaf_shortcut(0)


def test_leaf_shortcut_keeps_every_plane(csg, oracle):
    from csgrt import scenes
    rng = np.random.default_rng(29)
    light = np.float32(csg.light_dir())
    iters = [0, 0]
    cases = [scenes.random_tree(8200 + s, 2, 2048, 12) for s in range(60)]
    cases += [scenes.cheese_tree(s) for s in range(3)]
    for i, tree in enumerate(cases):
        nodes, prims = oracle.parse(scenes.write_text(tree))
        cam = csg.Camera.look_at_origin(scenes.seeded_direction(rng), float(rng.uniform(2.5, 4.0))).floats()
        for sc in (False, True):
            ref = _render(oracle, nodes, prims, cam, light, 40, 30, False, sc)
            got = _render(oracle, nodes, prims, cam, light, 40, 30, True, sc)
            assert ref["capped"] == 0 and got["capped"] == 0
            assert _differ(ref, got) == 0, (i, sc)
            iters[0] += int(ref["counts"]["iters"].sum())
            iters[1] += int(got["counts"]["iters"].sum())
    assert iters[1] < 0.8 * iters[0]


def test_leaf_shortcut_on_the_benchmark_frames(csg, oracle):
    """The cheese frame and a random-tree frame, on sampled warp tiles: the planes of the
    reference's traversal, and far fewer iterations (4x fewer on the cheese frame)."""
    from csgrt import scenes
    for cfg, seed, sc, gain in ((2, 0, False, 3.0), (3, 0, True, 1.5)):
        text = scenes.config_scene_text(cfg, seed)
        v = scenes.config_views(cfg, seed)[0]
        nodes, prims = oracle.parse(text)
        rng = np.random.default_rng(3)
        wx = rng.integers(0, v.w // 8, 300)
        wy = rng.integers(0, v.h // 4, 300)
        lane = np.arange(32)
        pix = ((wy[:, None] * 4 + lane // 8) * v.w + wx[:, None] * 8 + lane % 8).ravel()
        oracle.set_live_pruning(0)
        base = oracle.render_list(nodes, prims, v.camera, v.light, v.w, v.h, pix, mode="fma",
                                  want=("hit", "t", "prim", "normal", "rgba8"))
        off = _render(oracle, nodes, prims, v.camera, v.light, v.w, v.h, False, sc, pix)
        on = _render(oracle, nodes, prims, v.camera, v.light, v.w, v.h, True, sc, pix)
        for k in ("hit", "prim", "rgba8"):
            assert np.array_equal(on[k], base[k]), (cfg, k)
        for k in ("t", "normal"):
            assert np.array_equal(on[k].view(np.uint32), base[k].view(np.uint32)), (cfg, k)
        assert off["counts"]["iters"].sum() > gain * on["counts"]["iters"].sum(), cfg
