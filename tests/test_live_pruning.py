"""The engine's live-leaf pruning, checked on the CPU against the reference's own
algorithm: the oracle renders seeded random trees and cheese scenes with and without the
rule (a mask of the leaves live at tmin = 0; children without a live leaf are Misses;
culls and leaf Misses clear bits; each region of four mask words records the largest tmin
at which one of its live bits was cleared, and a loop to a tmin below a region's record
marks the looped child's leaves in that region live again: the oracle's pruning mode 4),
and every plane is the same, bit for bit, while the iteration count falls.  The engine's
earlier rule, one record per ray (mode 1), is sound too and is checked beside it.

Without the loop restore the rule is unsound: a node can return its closer child's t, below
a tmin its other child's subtree has already looped to, and an ancestor's loop then re-enters
that subtree with the lower tmin, where a leaf cleared at the higher tmin can hit.  On trees
deeper than 15 operator levels, whose 32-entry stacks can overflow, skipping a subtree
can change which pushes are dropped, so the engine skips there only under a guard: while no
push of the ray has been dropped, and under an operator whose height leaves the stacks room
for the skipped traversal.  Tests render trees and views where each part of the rule
matters and show the difference."""
from __future__ import annotations

import numpy as np

PLANES = ("hit", "t", "prim", "normal", "rgba8")

# A random tree (seed 5174, up to 2,048 leaves, 74 drawn) seen from this look-at camera at
# 48 x 36: three rays re-enter a subtree below a tmin it had already looped to.
REENTRY_TREE = 5174
REENTRY_DIR = (0.8142095647293127, -0.17626529223304066, -0.5531666398629836)
REENTRY_DIST = 2.5151785211371585


# Deep trees: a chain of 30 operators whose other children are leaves or small subtrees.
DEEP_SEEDS = (3, 11)


def deep_tree(seed: int, n_ops: int = 30):
    """(tree, view direction) for a seeded chain of n_ops operators."""
    from csgrt import scenes
    r = np.random.default_rng(seed)
    t = scenes._random_leaf(r)
    for _ in range(n_ops):
        op = scenes.OPERATORS[int(r.integers(0, 3))]
        other = scenes._random_leaf(r) if r.random() < 0.7 else scenes._random_shape(r, int(r.integers(2, 6)), 3)
        t = (op, t, other) if r.random() < 0.5 else (op, other, t)
    return t, scenes.seeded_direction(r)


def _render(oracle, nodes, prims, cam, light, w, h, live, sc):
    oracle.set_live_pruning(live)
    oracle.set_short_circuit(sc)
    try:
        thf = oracle.tan_half_fov(float(cam[5]))
        return oracle.render(nodes, prims, cam, light, w, h, mode="fma", tan_half_fov=thf,
                             want=PLANES, counts=True)
    finally:
        oracle.set_live_pruning(0)
        oracle.set_short_circuit(False)


def _differ(a, b) -> int:
    bad = np.zeros(a["hit"].shape, bool)
    for k in PLANES:
        x, y = a[k], b[k]
        if k in ("t", "normal"):
            x, y = x.view(np.uint32), y.view(np.uint32)
        if k == "prim":  # defined only where the ray hits
            x, y = np.where(a["hit"] != 0, x, -1), np.where(b["hit"] != 0, y, -1)
        if x.ndim > 1:
            bad |= (x != y).any(axis=tuple(range(1, x.ndim)))
        else:
            bad |= x != y
    return int(bad.sum())


def test_live_pruning_keeps_every_plane(csg, oracle):
    from csgrt import scenes
    rng = np.random.default_rng(17)
    light = np.float32(csg.light_dir())
    iters = [0, 0]
    cases = [(scenes.random_tree(6000 + s, 2, 2048, 12), rng) for s in range(60)]
    cases += [(scenes.cheese_tree(s), rng) for s in range(2)]
    for i, (tree, r) in enumerate(cases):
        nodes, prims = oracle.parse(scenes.write_text(tree))
        cam = csg.Camera.look_at_origin(scenes.seeded_direction(r), float(r.uniform(2.5, 4.0))).floats()
        for sc in (False, True):
            ref = _render(oracle, nodes, prims, cam, light, 40, 30, 0, sc)
            got = _render(oracle, nodes, prims, cam, light, 40, 30, 4, sc)  # the engine's rule
            assert ref["capped"] == 0 and got["capped"] == 0
            assert _differ(ref, got) == 0, (i, sc)
            per_ray = _render(oracle, nodes, prims, cam, light, 40, 30, 1, sc)  # one record per ray
            assert _differ(ref, per_ray) == 0, (i, sc)
            iters[0] += int(ref["counts"]["iters"].sum())
            iters[1] += int(got["counts"]["iters"].sum())
    assert iters[1] < 0.9 * iters[0]  # the rule skips work


def test_live_pruning_reentry_case(csg, oracle):
    """The rule keeps the planes where tmin falls on re-entry; without its loop restore the
    same rule changes them."""
    from csgrt import scenes
    nodes, prims = oracle.parse(scenes.write_text(scenes.random_tree(REENTRY_TREE, 2, 2048, 12)))
    cam = csg.Camera.look_at_origin(np.array(REENTRY_DIR), REENTRY_DIST).floats()
    light = np.float32(csg.light_dir())
    for sc in (False, True):
        ref = _render(oracle, nodes, prims, cam, light, 48, 36, 0, sc)
        assert _differ(ref, _render(oracle, nodes, prims, cam, light, 48, 36, 1, sc)) == 0
        assert _differ(ref, _render(oracle, nodes, prims, cam, light, 48, 36, 4, sc)) == 0
        assert _differ(ref, _render(oracle, nodes, prims, cam, light, 48, 36, 2, sc)) > 0


def test_deep_trees_prune_under_the_guard(csg, oracle):
    """Trees deeper than 15 operator levels: the rule with its guard (mode 4; the
    short-circuit carries the same guard) keeps every plane of the reference's traversal,
    with its drop-on-full stacks, on chains whose action stack fills; pruning them without
    the guard (mode 3) changes the renders wherever a 32-entry stack overflows."""
    from csgrt import scenes
    light = np.float32(csg.light_dir())
    changed = 0
    for seed in range(12):
        tree, direction = deep_tree(seed)
        assert scenes.op_depth(tree) > 15
        nodes, prims = oracle.parse(scenes.write_text(tree))
        cam = csg.Camera.look_at_origin(direction, 3.0).floats()
        ref = _render(oracle, nodes, prims, cam, light, 40, 30, 0, False)
        assert int(ref["counts"]["max_actions"].max()) >= 31  # the action stack (nearly) fills
        for sc in (False, True):
            got = _render(oracle, nodes, prims, cam, light, 40, 30, 4, sc)
            assert _differ(ref, got) == 0, (seed, sc)
            assert _differ(ref, _render(oracle, nodes, prims, cam, light, 40, 30, 0, sc)) == 0, (seed, sc)
        changed += _differ(ref, _render(oracle, nodes, prims, cam, light, 40, 30, 3, False)) > 0
        if seed in DEEP_SEEDS:
            assert int(ref["hit"].sum()) > 50
            assert _differ(ref, _render(oracle, nodes, prims, cam, light, 40, 30, 3, False)) > 0
    assert changed >= 6


def test_drilled_block_prunes_below_the_overflow(csg, oracle):
    """A cube with holes cut one after another (a left-deep Difference chain): with 20 holes
    the stacks never fill and the guarded rule skips a third of the iterations (with 24, where
    only the lowest eight levels leave the stacks room, 14%), every plane unchanged; with 40 the reference's action stack overflows on every ray that enters the
    chain (the reference then renders the block wrongly: almost no hits), and the guarded rule
    reproduces that render too."""
    from csgrt import scenes
    light = np.float32(csg.light_dir())
    for seed, n_holes in ((0, 20), (1, 24), (2, 40)):
        tree = scenes.drilled_block(seed, n_holes)
        assert scenes.op_depth(tree) == n_holes
        nodes, prims = oracle.parse(scenes.write_text(tree))
        rng = np.random.default_rng(seed)
        cam = csg.Camera.look_at_origin(scenes.seeded_direction(rng), 3.5).floats()
        ref = _render(oracle, nodes, prims, cam, light, 64, 48, 0, False)
        got = _render(oracle, nodes, prims, cam, light, 64, 48, 4, True)
        assert _differ(ref, got) == 0, (seed, n_holes)
        it0, it4 = int(ref["counts"]["iters"].sum()), int(got["counts"]["iters"].sum())
        if n_holes <= 24:
            assert int(ref["counts"]["max_actions"].max()) < 32
            assert int(ref["hit"].sum()) > 500
            assert it4 < (0.8 if n_holes == 20 else 0.95) * it0  # less room under 24 levels
        else:
            assert int(ref["counts"]["max_actions"].max()) == 32
            assert int(ref["hit"].sum()) < 50


def test_live_pruning_with_non_finite_parameters(csg, oracle):
    """Scenes whose text carries nan, inf or huge values (the parser accepts them, as the
    reference's std::stof does): hits with NaN t and loops to a NaN tmin keep the rule
    exact (a NaN tmin counts as below every clear, so the looped child is re-enabled).
    Some such scenes have rays whose traversal never ends (the oracle stops them at its
    iteration cap, as the engine does; the reference has none): those scenes are left out."""
    from csgrt import scenes
    rng = np.random.default_rng(3)
    light = np.float32(csg.light_dir())
    specials = ["nan", "inf", "-inf", "1e38", "-1e38", "0"]
    rendered = nan_hits = 0
    for s in range(80):
        toks = scenes.write_text(scenes.random_tree(9000 + s, 2, 200, 10)).split()
        slots = [i for i, t in enumerate(toks) if t not in scenes.OPERATORS + scenes.PRIMITIVES and len(t) != 6]
        for _ in range(int(rng.integers(1, 4))):
            toks[slots[int(rng.integers(len(slots)))]] = specials[int(rng.integers(len(specials)))]
        cam = csg.Camera.look_at_origin(scenes.seeded_direction(rng), 3.0).floats()
        try:
            nodes, prims = oracle.parse(" ".join(toks))
        except Exception:  # an out-of-range rotation: the reference rejects it too
            continue
        sc = bool(s & 1)
        ref = _render(oracle, nodes, prims, cam, light, 32, 24, 0, sc)
        if ref["capped"]:
            continue  # rays that never end: the reference's loop has no iteration cap
        got = _render(oracle, nodes, prims, cam, light, 32, 24, 4, sc)
        assert got["capped"] == 0
        assert _differ(ref, got) == 0, s
        rendered += 1
        nan_hits += int(np.isnan(ref["t"][ref["hit"] != 0]).sum())
    assert rendered >= 40 and nan_hits > 0


def test_region_records_restore_less_on_the_cheese_frame(csg, oracle):
    """On the 3840x2160 cheese frame (every 16th pixel each way) one restore record per
    ray (mode 1) re-enables whole subtrees that held no stale bit; per-region records
    (mode 4, the engine's rule) re-enable far less, with the same planes.  What set the
    GPU time was the slowest rays: their warps ran for most of the launch.  With one record
    per ray they took 2.8x the iterations of the rule without the restore; with per-region
    records, within 5% of it."""
    from csgrt import scenes
    text = scenes.config_scene_text(2, 0)
    view = scenes.config_views(2, 0)[0]
    nodes, prims = oracle.parse(text)
    ys = np.arange(8, view.h, 16)
    xs = np.arange(8, view.w, 16)
    pix = (ys[:, None] * view.w + xs[None, :]).ravel()
    out = {}
    for mode in (0, 1, 2, 4):
        oracle.set_live_pruning(mode)
        try:
            out[mode] = oracle.render_list(nodes, prims, view.camera, view.light, view.w, view.h, pix,
                                           mode="fma", want=("t", "prim"), counts=True)
        finally:
            oracle.set_live_pruning(0)
    for mode in (1, 2, 4):
        assert np.array_equal(out[mode]["t"].view(np.uint32), out[0]["t"].view(np.uint32))
        assert np.array_equal(out[mode]["prim"], out[0]["prim"])
    it = {m: int(out[m]["counts"]["iters"].sum()) for m in out}
    mx = {m: int(out[m]["counts"]["iters"].max()) for m in out}
    assert it[2] <= it[4] < it[1] < it[0]
    assert it[4] < 1.02 * it[2] and it[1] > 1.1 * it[2]
    assert mx[4] < 1.05 * mx[2] and mx[1] > 2.5 * mx[2]


def test_single_cylinder_root(csg, oracle):
    """A root leaf is tested without its box, and a cylinder's box (BVHNode.cuh:34-49)
    does not contain the cylinder: here a quarter of the hits lie outside it.  Trees this
    small start all live (no pre-pass), so the rule keeps every one of them."""
    text = "Cylinder 0 0 0 FF0000 0.6 1.6 30 20 10"
    nodes, prims = oracle.parse(text)
    d = np.array([0.2, 0.3, 1.0])
    cam = csg.Camera.look_at_origin(d / np.linalg.norm(d), 3.0).floats()
    light = np.float32(csg.light_dir())
    ref = _render(oracle, nodes, prims, cam, light, 96, 72, 0, False)
    pos = oracle.render(nodes, prims, cam, light, 96, 72, mode="fma", want=("hit", "pos"))
    outside = (np.abs(pos["pos"][pos["hit"] != 0]) > 0.8).any(axis=1).sum()
    assert outside > 100
    for mode in (1, 4):
        assert _differ(ref, _render(oracle, nodes, prims, cam, light, 96, 72, mode, False)) == 0
