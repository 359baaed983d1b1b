"""Kensler's Intersection table (LookUpActions, RaycastingKernels.cu:666-677) is symmetric
in its two children, ties included, so the traversal may visit an Intersection's children
in either order: checked on the CPU with the oracle, which renders random trees as written
and with every Intersection whose children are both operators swapped so that the child
with fewer leaves comes first.  The planes are the same once primitive indices are mapped
back; with the engine's live-leaf pruning and operator short-circuit, a Miss from the
smaller child then skips the larger one and the traversal takes fewer iterations."""
from __future__ import annotations

import numpy as np

PLANES = ("hit", "t", "prim", "normal", "rgba8")


def _leaves(tree) -> int:
    from csgrt import scenes
    return scenes.count_leaves(tree)


def reorder(tree, order):
    """(tree with reordered Intersections, order[i] = the original preorder index of the
    primitive now at preorder position i)."""
    from csgrt import scenes
    counter = [0]

    def tag(t):
        if t[0] in scenes.OPERATORS:
            return (t[0], tag(t[1]), tag(t[2]))
        counter[0] += 1
        return ("leaf", counter[0] - 1, t)

    def build(t):
        if t[0] == "leaf":
            order.append(t[1])
            return t[2]
        a, b = t[1], t[2]
        if t[0] == "Intersection" and a[0] != "leaf" and b[0] != "leaf" and _leaves(untag(b)) < _leaves(untag(a)):
            a, b = b, a
        return (t[0], build(a), build(b))

    def untag(t):
        return t[2] if t[0] == "leaf" else (t[0], untag(t[1]), untag(t[2]))

    return build(tag(tree))


def _render(oracle, text, cam, light, w, h, engine_rules):
    nodes, prims = oracle.parse(text)
    oracle.set_live_pruning(4 if engine_rules else 0)
    oracle.set_short_circuit(engine_rules)
    try:
        thf = oracle.tan_half_fov(float(cam[5]))
        return oracle.render(nodes, prims, cam, light, w, h, mode="fma", tan_half_fov=thf, want=PLANES,
                             counts=True)
    finally:
        oracle.set_live_pruning(0)
        oracle.set_short_circuit(False)


def _same(a, b, order) -> bool:
    hit = a["hit"] != 0
    if not np.array_equal(a["hit"], b["hit"]):
        return False
    prim_b = np.where(b["hit"] != 0, order[np.clip(b["prim"], 0, None)], -1)
    if not np.array_equal(np.where(hit, a["prim"], -1), prim_b):
        return False
    for k in ("t", "normal"):
        if not np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)):
            return False
    return np.array_equal(a["rgba8"], b["rgba8"])


def test_intersection_children_commute(csg, oracle):
    from csgrt import scenes
    rng = np.random.default_rng(8)
    light = np.float32(csg.light_dir())
    iters = [0, 0]
    swapped_trees = 0
    for s in range(200):
        tree = scenes.random_tree(7100 + s, 2, 2048, 12)
        order: list[int] = []
        tree2 = reorder(tree, order)
        order = np.array(order)
        swapped_trees += int((order != np.arange(len(order))).any())
        cam = csg.Camera.look_at_origin(scenes.seeded_direction(rng), float(rng.uniform(2.5, 4.0))).floats()
        t1, t2 = scenes.write_text(tree), scenes.write_text(tree2)
        # the reference's own traversal on the first 40 trees, the engine's rules on all
        for rules in ((False, True) if s < 40 else (True,)):
            a = _render(oracle, t1, cam, light, 40, 30, rules)
            b = _render(oracle, t2, cam, light, 40, 30, rules)
            assert _same(a, b, order), (s, rules)
            if rules:
                iters[0] += int(a["counts"]["iters"].sum())
                iters[1] += int(b["counts"]["iters"].sum())
    assert swapped_trees >= 50
    assert iters[1] < 0.95 * iters[0]  # 0.93 on this sample


def engine_order(nodes):
    """The scene compiler's Intersection order applied to a parsed node array: an
    Intersection of two operators lists the child with fewer leaves first.  Leaves keep
    their numbers (every subtree's leaves stay contiguous), so the planes, primitive
    indices included, must not change."""
    nodes = nodes.copy()
    n = len(nodes)
    leaves = np.zeros(n, np.int64)
    for i in range(n - 1, -1, -1):
        leaves[i] = 1 if nodes[i]["prim"] != -1 else leaves[nodes[i]["left"]] + leaves[nodes[i]["right"]]
    swapped = 0
    for i in range(n):
        l, r = int(nodes[i]["left"]), int(nodes[i]["right"])
        if nodes[i]["type"] == 2 and nodes[l]["prim"] == -1 and nodes[r]["prim"] == -1 and leaves[r] < leaves[l]:
            nodes[i]["left"], nodes[i]["right"] = r, l
            swapped += 1
    return nodes, swapped


def test_engine_order_keeps_every_plane(csg, oracle):
    """The engine's rule on node arrays (children swapped in place, no renumbering): every
    plane identical under the reference's traversal and under the engine's rules, and ~20%
    fewer iterations with them on the batched workload's trees."""
    from csgrt import scenes
    light = np.float32(csg.light_dir())
    work = scenes.config_batch(0, n_scenes=96)
    iters = [0, 0]
    swapped_trees = 0
    for s, (text, views) in enumerate(work):
        nodes, prims = oracle.parse(text)
        nodes2, k = engine_order(nodes)
        swapped_trees += k > 0
        cam = views[0].camera
        for rules in ((False, True) if s < 24 else (True,)):
            outs = []
            for nd in (nodes, nodes2):
                oracle.set_live_pruning(4 if rules else 0)
                oracle.set_short_circuit(rules)
                try:
                    outs.append(oracle.render(nd, prims, cam, light, 40, 30, mode="fma", want=PLANES, counts=True))
                finally:
                    oracle.set_live_pruning(0)
                    oracle.set_short_circuit(False)
            assert _same(outs[0], outs[1], np.arange(len(prims))), (s, rules)
            if rules:
                iters[0] += int(outs[0]["counts"]["iters"].sum())
                iters[1] += int(outs[1]["counts"]["iters"].sum())
    assert swapped_trees >= 20
    assert iters[1] < 0.9 * iters[0]
