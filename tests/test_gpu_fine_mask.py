"""Single-view renders of large rolled trees with the one-bit-per-leaf live mask (the
scene's fine mask, CSG_SCENE_FINE_MASK): every plane still equals the reference kernel's,
bit for bit, for trees of 1,173, 1,694 and 1,852 leaves; the scene holds what the host-side
plan says."""
from __future__ import annotations

import numpy as np
import pytest

from test_gpu_parity import assert_bit_exact, engine_render

pytestmark = pytest.mark.gpu

CASES = [79, 191, 93]  # tree seeds of the batched workload (1,173, 1,694 and 1,852 leaves)


def test_fine_mask_trees_vs_reference_kernel(csg):
    from oracle import RefCuda, quantize_rgba8
    from conftest import ulp_equal
    from csgrt import scenes
    if not RefCuda.available():
        pytest.skip("reference cubin not built on this machine")
    G = RefCuda()
    rng = np.random.default_rng(11)
    hits = 0
    for seed in CASES:
        text = scenes.write_text(scenes.random_tree(seed, 2, 2048, 12))
        with csg.Scene(text, fine_mask=True) as sc:
            info = sc.info()
        assert info == csg.plan_tree(text, fine_mask=True)  # the host-side plan is what the scene holds
        assert info["n_prims"] > 1024 and info["rolled"] == 1 and info["live_shift"] == 1, (seed, info)
        assert info["fine_words"] == (info["n_prims"] + 31) // 32, (seed, info)
        for _ in range(2):
            cam = csg.Camera.look_at_origin(scenes.seeded_direction(rng), float(rng.uniform(2.5, 4.0))).floats()
            light = csg.light_dir()
            w, h = 256, 192
            eng = engine_render(csg, text, cam, light, w, h, fine_mask=True)
            nodes44, prims48, _ = csg.parse_tree(text)
            ref = G.render(nodes44, prims48, cam, light, w, h)
            ref["rgba8"] = quantize_rgba8(ref["rgba"])
            assert_bit_exact(eng, ref, f"tree {seed}")
            assert ulp_equal(eng["rgba32f"], ref["rgba"]).all(), seed
            hits += int(ref["hit"].sum())
    assert hits > 5000  # the frames see surfaces, not only empty sets
