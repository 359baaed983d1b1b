"""Scene writer and seeded generators of the benchmark configurations."""
from __future__ import annotations

import numpy as np

from csgrt import scenes


def test_writer_round_trip(csg, oracle):
    for seed in range(5):
        tree = scenes.random_tree(seed, 2, 300)
        text = scenes.write_text(tree)
        nodes, prims, depth = csg.parse_tree(text)
        n = len(nodes) // 44
        assert n == 2 * scenes.count_leaves(tree) - 1
        assert depth == scenes.op_depth(tree)
        # writing the same tree twice gives the same bytes
        assert scenes.write_text(tree) == text


def test_readme_tree_equals_reference_file(csg):
    from conftest import GOLDEN
    a = csg.parse_tree(scenes.write_text(scenes.wikipedia_tree()))
    b = csg.parse_tree((GOLDEN / "scenes" / "testWikipedia.txt").read_text())
    assert (a[0] == b[0]).all() and (a[1] == b[1]).all()


def test_cheese_config():
    tree = scenes.cheese_tree(0)
    assert scenes.count_leaves(tree) == 513
    assert scenes.op_depth(tree) == 10
    assert tree[0] == "Difference" and tree[1][0] == "Cube"


def test_random_tree_bounds():
    for seed in range(40):
        tree = scenes.random_tree(seed, 2, 4096, 12)
        n = scenes.count_leaves(tree)
        assert 2 <= n <= 4096
        assert scenes.op_depth(tree) <= 12
    assert scenes.count_leaves(scenes.random_tree(0, n_leaves=4096)) == 4096
    assert scenes.op_depth(scenes.random_tree(0, n_leaves=4096)) == 12


def test_seeded_directions_respect_pitch_clamp():
    rng = np.random.default_rng(0)
    for _ in range(500):
        d = scenes.seeded_direction(rng)
        assert abs(np.degrees(np.arcsin(-d[1]))) <= 89.0
        assert abs(np.linalg.norm(d) - 1) < 1e-12


def test_look_at_camera_faces_origin(csg):
    rng = np.random.default_rng(1)
    for _ in range(50):
        d = scenes.seeded_direction(rng)
        c = csg.Camera.look_at_origin(d, 4.0).floats()
        assert np.allclose(c[:3], 4 * d, atol=1e-5)
        assert np.allclose(c[6:9], -d, atol=1e-5)
