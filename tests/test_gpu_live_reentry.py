"""Rays on which the reference re-enters a subtree with a tmin below one the subtree has
already looped to (a node returns its closer child's t, below a tmin its other child's
subtree reached, and an ancestor's loop re-descends with it).  A live-leaf mask that keeps
bits cleared at the higher tmin changes these rays; the engine marks the looped child's
leaves live again and must match the oracle and the reference kernel bit for bit.  The
trees and views are ones where the oracle without that restore differs
(tests/test_live_pruning.py).  Also: trees deeper than 15 operator levels, whose 32-entry
stacks can overflow, where the engine skips work only while no push has been dropped and
where the skipped traversal could not drop one: against the oracle on chains whose stacks
overflow, and against the reference kernel on drilled blocks whose stacks do not."""
from __future__ import annotations

import numpy as np
import pytest

from test_gpu_parity import assert_bit_exact, engine_render
from test_live_pruning import DEEP_SEEDS, REENTRY_DIR, REENTRY_DIST, REENTRY_TREE, deep_tree

pytestmark = pytest.mark.gpu


def _cases():
    import csgrt
    from csgrt import scenes
    out = [(REENTRY_TREE, csgrt.Camera.look_at_origin(np.array(REENTRY_DIR), REENTRY_DIST).floats())]
    # two more trees of a seeded sweep (tree seed 20000 + i, the i-th view of that sweep)
    rng = np.random.default_rng(20000)
    for i in range(142):
        d, dist = scenes.seeded_direction(rng), float(rng.uniform(2.5, 4.0))
        if i in (113, 141):
            out.append((20000 + i, csgrt.Camera.look_at_origin(d, dist).floats()))
    return out


@pytest.mark.parametrize("size", [(48, 36), (96, 72)])
def test_reentry_rays_match_oracle_and_reference_kernel(csg, oracle, size):
    from oracle import RefCuda, quantize_rgba8
    from csgrt import scenes
    w, h = size
    light = np.float32(csg.light_dir())
    G = RefCuda() if RefCuda.available() else None
    for seed, cam in _cases():
        text = scenes.write_text(scenes.random_tree(seed, 2, 2048, 12))
        eng = engine_render(csg, text, cam, light, w, h)
        nodes, prims = oracle.parse(text)
        thf = csg.device_tan_half_fov(float(cam[5]))
        ref = oracle.render(nodes, prims, cam, light, w, h, mode="fma", tan_half_fov=thf)
        assert_bit_exact(eng, ref, f"tree {seed} {w}x{h} vs oracle")
        if G is not None:
            nodes44, prims48, _ = csg.parse_tree(text)
            k = G.render(nodes44, prims48, cam, light, w, h)
            k["rgba8"] = quantize_rgba8(k["rgba"])
            assert_bit_exact(eng, k, f"tree {seed} {w}x{h} vs reference kernel")


def test_deep_trees_with_overflowing_stacks_match_oracle(csg, oracle):
    """The reference kernel is not run here: its stacks read uninitialised slots when
    they overflow; the oracle defines those slots as the engine does."""
    from csgrt import scenes
    light = np.float32(csg.light_dir())
    cases = [deep_tree(seed) for seed in DEEP_SEEDS + (0, 1, 4, 7)]
    cases += [(scenes.drilled_block(seed, n), scenes.seeded_direction(np.random.default_rng(seed)))
              for seed, n in ((2, 40), (3, 33))]
    for seed, (tree, direction) in enumerate(cases):
        text = scenes.write_text(tree)
        with csg.Scene(text) as sc:
            assert sc.info()["stack_class"] == 32
        cam = csg.Camera.look_at_origin(direction, 3.0).floats()
        eng = engine_render(csg, text, cam, light, 80, 60)
        nodes, prims = oracle.parse(text)
        thf = csg.device_tan_half_fov(float(cam[5]))
        ref = oracle.render(nodes, prims, cam, light, 80, 60, mode="fma", tan_half_fov=thf)
        assert_bit_exact(eng, ref, f"deep tree {seed}")


@pytest.mark.parametrize("n_holes", [16, 20, 24, 28])
def test_drilled_blocks_match_reference_kernel(csg, oracle, n_holes):
    """Drilled blocks of 16-28 holes: deeper than 15 operator levels (the 32-entry class,
    where skips are guarded), and shallow enough that no stack overflows, so the reference
    kernel's output is defined: the engine matches it and the oracle bit for bit."""
    from oracle import RefCuda, quantize_rgba8
    from csgrt import scenes
    light = np.float32(csg.light_dir())
    for seed in range(2):
        tree = scenes.drilled_block(100 + seed, n_holes)
        text = scenes.write_text(tree)
        with csg.Scene(text) as sc:
            assert sc.info()["stack_class"] == 32
        cam = csg.Camera.look_at_origin(scenes.seeded_direction(np.random.default_rng(seed)), 3.5).floats()
        eng = engine_render(csg, text, cam, light, 96, 72)
        assert int(eng["hit"].sum()) > 1000
        nodes, prims = oracle.parse(text)
        thf = csg.device_tan_half_fov(float(cam[5]))
        ref = oracle.render(nodes, prims, cam, light, 96, 72, mode="fma", tan_half_fov=thf)
        assert_bit_exact(eng, ref, f"drilled block {n_holes} seed {seed} vs oracle")
        if RefCuda.available():
            nodes44, prims48, _ = csg.parse_tree(text)
            k = RefCuda().render(nodes44, prims48, cam, light, 96, 72)
            k["rgba8"] = quantize_rgba8(k["rgba"])
            assert_bit_exact(eng, k, f"drilled block {n_holes} seed {seed} vs reference kernel")
