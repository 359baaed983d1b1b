"""Scene text writer and seeded scene generators for the benchmark configurations.

Scenes are produced as text in the reference's preorder format (README.md:37-61, parsed
by CSGTree::Parse, CSGTree.cu:5-152), so every engine and every oracle reads the same
bytes.  Numbers are written with 9 significant digits, which round-trips float32.

Trees are nested tuples:
    ("Union" | "Difference" | "Intersection", left, right)
    ("Sphere", x, y, z, "RRGGBB", radius)
    ("Cylinder", x, y, z, "RRGGBB", radius, height, rotX, rotY, rotZ)
    ("Cube", x, y, z, "RRGGBB", edge)
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

OPERATORS = ("Union", "Difference", "Intersection")
PRIMITIVES = ("Sphere", "Cylinder", "Cube")


def _num(v) -> str:
    return format(float(np.float32(v)), ".9g")


def write_text(tree, indent: str = "\t") -> str:
    """Pretty-print a tree in preorder, one node per line, children indented."""
    lines: list[str] = []
    stack = [(tree, 0)]
    while stack:
        node, depth = stack.pop()
        kind = node[0]
        pad = indent * depth
        if kind in OPERATORS:
            lines.append(pad + kind)
            stack.append((node[2], depth + 1))
            stack.append((node[1], depth + 1))
        elif kind in ("Sphere", "Cube"):
            _, x, y, z, col, s = node
            lines.append(f"{pad}{kind} {_num(x)} {_num(y)} {_num(z)} {col} {_num(s)}")
        elif kind == "Cylinder":
            _, x, y, z, col, r, h, rx, ry, rz = node
            lines.append(f"{pad}Cylinder {_num(x)} {_num(y)} {_num(z)} {col} {_num(r)} {_num(h)} "
                         f"{_num(rx)} {_num(ry)} {_num(rz)}")
        else:
            raise ValueError(f"unknown node kind {kind!r}")
    return "\n".join(lines) + "\n"


def count_leaves(tree) -> int:
    if tree[0] in OPERATORS:
        return count_leaves(tree[1]) + count_leaves(tree[2])
    return 1


def op_depth(tree) -> int:
    if tree[0] in OPERATORS:
        return 1 + max(op_depth(tree[1]), op_depth(tree[2]))
    return 0


def _color(rng) -> str:
    return "%06X" % int(rng.integers(0, 1 << 24))


# ---- configuration 1: the README / testWikipedia tree ---------------------------------
def wikipedia_tree():
    """Difference(Intersection(Cube 0 edge 2, Sphere 0 r 1.35), Union(Union(Cylinder r .7 h 2
    rot 90,0,0; Cylinder rot 0,0,0), Cylinder rot 0,0,90))."""
    cyl = lambda rx, ry, rz: ("Cylinder", 0, 0, 0, "00FF00", 0.7, 2, rx, ry, rz)
    return ("Difference",
            ("Intersection", ("Cube", 0, 0, 0, "FF0000", 2), ("Sphere", 0, 0, 0, "0000FF", 1.35)),
            ("Union", ("Union", cyl(90, 0, 0), cyl(0, 0, 0)), cyl(0, 0, 90)))


# ---- configuration 2: cheese ---------------------------------------------------------
def _balanced(leaves):
    if len(leaves) == 1:
        return leaves[0]
    mid = len(leaves) // 2
    return ("Union", _balanced(leaves[:mid]), _balanced(leaves[mid:]))


def cheese_tree(seed: int, n_spheres: int = 512):
    """Difference(Cube centre 0 edge 2, balanced Union of n spheres), centres U[-1,1]^3,
    radii U[0.05, 0.2]."""
    rng = np.random.default_rng(seed)
    spheres = []
    for _ in range(n_spheres):
        c = rng.uniform(-1, 1, 3)
        r = rng.uniform(0.05, 0.2)
        spheres.append(("Sphere", c[0], c[1], c[2], _color(rng), r))
    return ("Difference", ("Cube", 0, 0, 0, _color(rng), 2), _balanced(spheres))


# ---- configuration 3: random trees ------------------------------------------------------
def drilled_block(seed: int, n_holes: int = 40):
    """A cube of edge 2 with n_holes holes cut one after another: a left-deep chain of
    Differences, Difference(...Difference(Difference(Cube, hole 1), hole 2)..., hole n), so
    n_holes operator levels (the shape sequential modelling produces).  Holes are
    axis-aligned cylinders through the block (radius U[0.04, 0.12], height 2.4, centre
    U[-0.9, 0.9] on the other two axes) and, one in four, spheres (radius U[0.1, 0.3],
    centre U[-1, 1]^3)."""
    rng = np.random.default_rng(seed)
    t = ("Cube", 0.0, 0.0, 0.0, _color(rng), 2.0)
    rots = ((0.0, 0.0, 0.0), (90.0, 0.0, 0.0), (0.0, 0.0, 90.0))
    for _ in range(n_holes):
        col = _color(rng)
        if rng.random() < 0.25:
            c = rng.uniform(-1, 1, 3)
            hole = ("Sphere", c[0], c[1], c[2], col, rng.uniform(0.1, 0.3))
        else:
            c = rng.uniform(-0.9, 0.9, 3)
            rot = rots[int(rng.integers(0, 3))]
            hole = ("Cylinder", c[0], c[1], c[2], col, rng.uniform(0.04, 0.12), 2.4, *rot)
        t = ("Difference", t, hole)
    return t


def _random_leaf(rng):
    kind = PRIMITIVES[int(rng.integers(0, 3))]
    c = rng.uniform(-1, 1, 3)
    col = _color(rng)
    if kind == "Sphere":
        return ("Sphere", c[0], c[1], c[2], col, rng.uniform(0.1, 0.8))
    if kind == "Cube":
        return ("Cube", c[0], c[1], c[2], col, rng.uniform(0.1, 0.8))
    rot = rng.uniform(0, 360, 3)
    return ("Cylinder", c[0], c[1], c[2], col, rng.uniform(0.1, 0.8), rng.uniform(0.1, 0.8),
            rot[0], rot[1], rot[2])


def _random_shape(rng, n: int, depth: int):
    """A tree with n leaves and at most `depth` operator levels (n <= 2**depth): each split
    is uniform among the splits that still fit, so it is near-balanced when n is close
    to 2**depth and free otherwise."""
    if n == 1:
        return _random_leaf(rng)
    half = 1 << (depth - 1)
    lo, hi = max(1, n - half), min(n - 1, half)
    k = int(rng.integers(lo, hi + 1))
    op = OPERATORS[int(rng.integers(0, 3))]
    return (op, _random_shape(rng, k, depth - 1), _random_shape(rng, n - k, depth - 1))


def random_tree(seed: int, min_leaves: int = 2, max_leaves: int = 4096, max_depth: int = 12,
                n_leaves: int | None = None):
    """Leaf count log-uniform in [min_leaves, max_leaves], operators uniform over
    {Union, Difference, Intersection}, primitives uniform over {sphere, cylinder, cube},
    positions U[-1,1]^3, sizes U[0.1, 0.8], cylinder rotations U[0, 360) per axis."""
    rng = np.random.default_rng(seed)
    if n_leaves is None:
        n_leaves = int(round(math.exp(rng.uniform(math.log(min_leaves), math.log(max_leaves)))))
    n_leaves = max(1, min(n_leaves, 1 << max_depth))
    return _random_shape(rng, n_leaves, max_depth)


# ---- cameras ----------------------------------------------------------------------------
def seeded_direction(rng) -> np.ndarray:
    """A unit direction whose look-at pitch stays within the camera's +-89 degree clamp."""
    while True:
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        if abs(math.degrees(math.asin(-d[1]))) <= 89.0:
            return d


@dataclass
class View:
    camera: np.ndarray  # 15 floats, reference Camera layout
    light: np.ndarray   # 3 floats
    w: int
    h: int


def config_views(config: int, seed: int = 0, n: int = 1):
    """Camera/light/resolution for the benchmark configurations (needs libcsgrt for the
    camera maths, which must be the engine's own)."""
    from . import Camera, light_dir
    rng = np.random.default_rng(seed + 1000 * config)
    views = []
    for _ in range(n):
        if config == 1:
            cam = Camera().set_fov(60)
            views.append(View(cam.floats(), np.array([-1, -1, -1], np.float32), 1280, 720))
            continue
        cam = Camera.look_at_origin(seeded_direction(rng), 4.0, 60.0)
        res = {2: (3840, 2160), 3: (1920, 1080)}.get(config)
        if res is None:
            s = [256, 512, 768, 1024] if config == 4 else [256, 512, 1024, 2048]
            r = s[int(rng.integers(0, 4))]
            res = (r, r)
        views.append(View(cam.floats(), light_dir(), res[0], res[1]))
    return views


def config_scene_text(config: int, seed: int = 0) -> str:
    if config == 1:
        return write_text(wikipedia_tree())
    if config == 2:
        return write_text(cheese_tree(seed))
    if config == 3:
        return write_text(random_tree(seed, 2, 4096, 12))
    return write_text(random_tree(seed, 2, 2048, 12))


def config_batch(seed: int = 0, n_scenes: int = 256, per_scene: int = 4):
    """The batched workload: n_scenes random trees (leaf counts log-uniform 2..2048, depth
    <= 12), each seen by per_scene seeded cameras at resolutions uniform over 256^2,
    512^2, 768^2 and 1024^2.  Returns [(scene text, [View, ...]), ...]."""
    out = []
    for s in range(n_scenes):
        sid = seed * 100003 + s
        out.append((write_text(random_tree(sid, 2, 2048, 12)), config_views(4, sid, per_scene)))
    return out
