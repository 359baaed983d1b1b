"""A wider sweep of the engine against the reference's own CUDA kernel: 64 random trees of
the batched and random-tree workloads (2 to 4,096 leaves, depth up to 12, mixed
primitives and operators), one seeded camera each, every plane compared bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

from test_gpu_parity import assert_bit_exact, engine_render

pytestmark = pytest.mark.gpu


def test_random_trees_vs_reference_kernel(csg):
    from oracle import RefCuda, quantize_rgba8
    from conftest import ulp_equal
    from csgrt import scenes
    if not RefCuda.available():
        pytest.skip("reference cubin not built on this machine")
    G = RefCuda()
    rng = np.random.default_rng(2024)
    cases = [(f"batch-{i}", text, views[0]) for i, (text, views) in enumerate(scenes.config_batch(7, n_scenes=48))]
    for seed in range(100, 116):
        cases.append((f"random-{seed}", scenes.config_scene_text(3, seed), scenes.config_views(3, seed)[0]))
    hits = 0
    for name, text, view in cases:
        cam = csg.Camera.look_at_origin(scenes.seeded_direction(rng), float(rng.uniform(2.5, 4.5)))
        w, h = 160, 120
        eng = engine_render(csg, text, cam.floats(), view.light, w, h)
        nodes44, prims48, _ = csg.parse_tree(text)
        ref = G.render(nodes44, prims48, cam.floats(), view.light, w, h)
        ref["rgba8"] = quantize_rgba8(ref["rgba"])
        assert_bit_exact(eng, ref, name)
        assert ulp_equal(eng["rgba32f"], ref["rgba"]).all(), name
        hits += int(ref["hit"].sum())
    assert hits > 10000  # the sweep sees surfaces, not only empty sets
