"""The cost-ordered dispatch's order (csrc/render.cu: order_grid, order_count, order_scatter),
restated in numpy (with the view shift that makes a tile read the recorded cost of the tile
it came from): the positions the two kernels compute (a class's start, plus the same
class's tiles in earlier blocks, which each order_scatter block sums from order_count's
per-block counts, plus the same class's earlier tiles inside the block) form a permutation
of the tiles, longest class first, centre-out order within a class, on grids from one tile
to the largest frames.  The GPU tests check the kernels' own
output (tests/test_gpu_dispatch.py); this pins the arithmetic and the buffer bounds."""
from __future__ import annotations

import numpy as np
import pytest

THREADS, CLASSES, BLOCKS_MAX, KEY_TOP = 256, 32, 256, 45


def tile_row(k, c, n):
    """tile_row (render_tiled.cuh), vectorised over k."""
    k = np.asarray(k, np.int64)
    m = min(c, n - 1 - c)
    near = np.where(k & 1, c - ((k + 1) >> 1), c + (k >> 1))
    far = (c + m + (k - 2 * m)) if c - m == 0 else (c - m - (k - 2 * m))
    return np.where(k <= 2 * m, near, far)


def cost_class(c):
    c = np.asarray(c, np.uint64)
    l = np.floor(np.log2((c | 1).astype(np.float64))).astype(np.int64)
    nxt = np.where(l > 0, (c >> np.maximum(l - 1, 0).astype(np.uint64)) & 1, 0).astype(np.int64)
    return np.clip(KEY_TOP - (2 * l + nxt), 0, CLASSES - 1)


def order_grid(n):
    g = min(BLOCKS_MAX, (n + THREADS - 1) // THREADS) or 1
    per = (n + g - 1) // g
    return g, (per + THREADS - 1) // THREADS * THREADS


def dispatch_order(tiles_x, tiles_y, center_row, cost, shift_x=0, shift_y=0):
    n = tiles_x * tiles_y
    g, chunk = order_grid(n)
    assert g <= BLOCKS_MAX and chunk % THREADS == 0 and g * chunk >= n
    k = np.arange(n)
    row = tile_row(k // tiles_x, center_row, tiles_y)
    tile = row * tiles_x + k % tiles_x                 # row-major index of position k
    packed = (row << 16) | (k % tiles_x)               # what order[] holds
    # cost_source: the recorded entry standing for each tile once the view moved by the shift
    src = (np.clip(row - shift_y, 0, tiles_y - 1) * tiles_x + np.clip(k % tiles_x - shift_x, 0, tiles_x - 1))
    cls = cost_class(cost[src])
    block = k // chunk
    counts = np.zeros((g, CLASSES), np.int64)
    np.add.at(counts, (block, cls), 1)
    start = np.concatenate([[0], np.cumsum(counts.sum(0))[:-1]])          # per class
    bases = start[None, :] + np.cumsum(counts, 0) - counts                 # each block's first positions
    # inside a block the kernel places a tile after the same class's earlier tiles
    # (earlier slabs, warps of the slab, lanes of the warp: earlier positions k)
    rank = np.zeros(n, np.int64)
    seen = np.zeros((g, CLASSES), np.int64)
    for b in range(g):
        sel = np.nonzero(block == b)[0]
        for c in np.unique(cls[sel]):
            idx = sel[cls[sel] == c]
            rank[idx] = np.arange(len(idx))
            seen[b, c] = len(idx)
    assert (seen == counts).all()
    pos = bases[block, cls] + rank
    assert pos.min() >= 0 and pos.max() < n
    order = np.full(n, -1, np.int64)
    order[pos] = packed
    return order, tile, cls, k, src


@pytest.mark.parametrize("tiles_x,tiles_y,center_row,shift_x,shift_y", [
    (1, 1, 0, 0, 0), (7, 3, 1, 0, 0), (33, 17, 16, 5, -3), (100, 61, 0, 0, 0), (100, 61, 60, -99, 60),
    (480, 135, 67, 23, 0), (240, 270, 135, 0, 0), (13, 5000, 2500, 0, -4999), (257, 257, 3, 1, 1),
    (512, 128, 64, -17, 2)])
def test_positions_are_a_stable_class_order(tiles_x, tiles_y, center_row, shift_x, shift_y):
    rng = np.random.default_rng(tiles_x * 7919 + tiles_y)
    n = tiles_x * tiles_y
    for cost in (np.exp(rng.uniform(0, 22, n)).astype(np.uint64).clip(0, 2 ** 32 - 1),
                 np.zeros(n, np.uint64), np.full(n, 2 ** 32 - 1, np.uint64),
                 rng.integers(0, 2 ** 32, n, dtype=np.uint64)):
        order, tile, cls, k, src = dispatch_order(tiles_x, tiles_y, center_row, cost, shift_x, shift_y)
        assert src.min() >= 0 and src.max() < n                     # reads stay inside the array
        assert (order >= 0).all()
        rows, cols = order >> 16, order & 0xFFFF
        assert rows.max() < tiles_y and cols.max() < tiles_x
        raster = rows * tiles_x + cols
        assert (np.sort(raster) == np.arange(n)).all()               # every tile once
        pos_of = np.empty(n, np.int64)
        pos_of[tile] = k                                             # centre-out position of a tile
        src_of = np.empty(n, np.int64)
        src_of[tile] = src
        c = cost_class(cost[src_of[raster]])
        assert (np.diff(c) >= 0).all()                               # longest class first
        same = np.diff(c) == 0
        assert (np.diff(pos_of[raster])[same] > 0).all()             # centre-out within a class


def test_cost_classes_are_half_octaves():
    c = np.array([0, 1, 2, 3, 4, 5, 6, 7, 8, 12, 2 ** 20, 3 * 2 ** 19, 3 * 2 ** 22, 2 ** 32 - 1], np.uint64)
    cls = cost_class(c)
    assert (np.diff(cls) <= 0).all()                                 # longer is never a later class
    assert cls[-1] == 0 and cls[-2] == 0 and cls[0] == CLASSES - 1
    assert cls[list(c).index(2 ** 20)] == KEY_TOP - 40
    assert cls[list(c).index(3 * 2 ** 19)] == KEY_TOP - 41
