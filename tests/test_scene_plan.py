"""The scene compiler's host-side decisions (csg_tree_plan, no device work): stack class
from the operator depth, rolled GoTo for trees of more than 2 primitives,
live-mask words and granularity, the fine mask of single-view renders (on request) for
rolled trees of 1,025-2,048 leaves, the operator short-circuit for trees where Differences and
Intersections are common, and the device layout size."""
from __future__ import annotations

import pytest


def _count_kinds(tree, c=None):
    c = c if c is not None else {}
    c[tree[0]] = c.get(tree[0], 0) + 1
    if tree[0] in ("Union", "Intersection", "Difference"):
        _count_kinds(tree[1], c)
        _count_kinds(tree[2], c)
    return c


def _depth(tree):
    if tree[0] in ("Union", "Intersection", "Difference"):
        return 1 + max(_depth(tree[1]), _depth(tree[2]))
    return 0


@pytest.mark.parametrize("seed,leaves", [(3, 2), (11, 9), (21, 300), (79, 2048), (191, 2048), (93, 2048),
                                         (5, 4096), (8, 40)])
def test_plan_matches_the_rules(csg, seed, leaves):
    from csgrt import scenes
    tree = scenes.random_tree(seed, 2, leaves, 12)
    text = scenes.write_text(tree)
    plan = csg.plan_tree(text)
    kinds = _count_kinds(tree)
    n = sum(kinds.get(k, 0) for k in ("Sphere", "Cylinder", "Cube"))
    assert plan["n_prims"] == n and plan["n_nodes"] == 2 * n - 1
    assert plan["op_depth"] == _depth(tree)
    d = plan["op_depth"]
    assert plan["stack_class"] == (4 if d <= 4 else 8 if d <= 8 else 12 if d <= 12 else 16 if d <= 15 else 32)
    assert plan["rolled"] == int(n > 2)
    shift = 0
    while (n + (1 << shift) - 1) >> shift > 32 * 32:
        shift += 1
    assert plan["live_shift"] == shift
    assert plan["live_words"] == (((n + (1 << shift) - 1) >> shift) + 31) // 32 <= 32
    possible = bool(plan["rolled"]) and shift > 0 and n <= 2048
    if plan["fine_words"]:  # by default only where the build's threshold allows
        assert possible and plan["fine_words"] == (n + 31) // 32
    asked = csg.plan_tree(text, fine_mask=True)  # CSG_SCENE_FINE_MASK
    assert asked["fine_words"] == ((n + 31) // 32 if possible else 0)
    assert {k: v for k, v in asked.items() if k != "fine_words"} == {k: v for k, v in plan.items() if k != "fine_words"}
    assert plan["device_bytes"] > 16 * plan["n_nodes"]
    ops = sum(kinds.get(k, 0) for k in ("Union", "Intersection", "Difference"))
    decisive = kinds.get("Intersection", 0) + kinds.get("Difference", 0)
    assert plan["short_circuit"] == int(8 * decisive >= ops)


def test_plan_of_the_reference_files(csg):
    from conftest import GOLDEN
    for f in sorted((GOLDEN / "scenes").glob("*.txt")):
        plan = csg.plan_tree(f.read_text())
        assert plan["n_nodes"] == 2 * plan["n_prims"] - 1
        assert plan["fine_words"] == 0  # the reference's own scenes are small


def test_plan_errors_are_parse_errors(csg):
    with pytest.raises(csg.CsgError) as e:
        csg.plan_tree("Sphere 0 0 0 FF0000")
    assert e.value.code == csg.CSG_E_PARSE
    assert csg.lib().csg_tree_plan(b"Sphere 0 0 0 FF0000 1", 21, 0, None, None, 0) == csg.CSG_E_ARG


def test_plan_of_the_benchmark_scenes(csg):
    from csgrt import scenes
    cheese = csg.plan_tree(scenes.config_scene_text(2, 0))
    assert cheese["short_circuit"] == 0 and cheese["rolled"] == 1  # one Difference over a Union of spheres
    # the README tree: a Difference and an Intersection among four operators (unrolled)
    assert csg.plan_tree(scenes.config_scene_text(1, 0))["short_circuit"] == 1
    assert csg.plan_tree(scenes.config_scene_text(3, 0))["short_circuit"] == 1
