"""The batched persistent launch (csg_batch_*) writes, for every view, exactly the bytes a
per-view csg_render_planes writes -- for every warp tile shape, after autotuning, and on
graph replay."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _views(csg, torch, n_scenes=6, per_scene=2, seed=0, deep=False):
    from csgrt import scenes
    rng = np.random.default_rng(seed)
    sc_list, views = [], []
    for s in range(n_scenes):
        text = scenes.write_text(scenes.random_tree(100 + s, 2, 300 if s % 2 else 60, 12))
        if s == 0:
            text = scenes.write_text(scenes.cheese_tree(7, 64))  # spheres and a cube only
        sc_list.append(csg.Scene(text))
    if deep:
        tree = ("Sphere", 0, 0, 0, "FF0000", 0.9)
        for i in range(20):
            tree = ("Union" if i % 3 else "Difference", tree, ("Sphere", *rng.uniform(-1, 1, 3), "00FF00", 0.3))
        sc_list.append(csg.Scene(scenes.write_text(tree)))
    for sc in sc_list:
        for _ in range(per_scene):
            w, h = int(rng.integers(40, 200)), int(rng.integers(30, 150))
            cam = csg.Camera.look_at_origin(scenes.seeded_direction(rng), 3.0)
            views.append((sc, cam, csg.light_dir(), w, h))
    return sc_list, views


def _alloc(torch, w, h):
    n = w * h
    return {"rgba8": torch.zeros(n, dtype=torch.int32, device="cuda"),
            "t": torch.zeros(n, dtype=torch.float32, device="cuda"),
            "prim": torch.zeros(n, dtype=torch.int32, device="cuda"),
            "normal": torch.zeros(3 * n, dtype=torch.float32, device="cuda"),
            "rgba32f": torch.zeros(4 * n, dtype=torch.float32, device="cuda")}


@pytest.mark.parametrize("deep", [False, True])
def test_batch_equals_per_view_renders(csg, deep):
    import torch
    torch.cuda.set_device(0)
    scenes_, views = _views(csg, torch, deep=deep)
    ref, out, bviews = [], [], []
    for sc, cam, light, w, h in views:
        r = _alloc(torch, w, h)
        sc.render_ptrs(cam, light, w, h, **{k: v.data_ptr() for k, v in r.items()})
        ref.append(r)
        o = _alloc(torch, w, h)
        out.append(o)
        bviews.append((sc, cam, light, w, h, {k: v.data_ptr() for k, v in o.items()}))
    torch.cuda.synchronize()
    b = csg.Batch(bviews)
    info = b.info()
    assert info["n_views"] == len(views)
    if deep:
        assert info["stack_class"] == 32
    for tw in (8, 4, 16, 32, None):
        for o in out:
            for v in o.values():
                v.zero_()
        if tw is None:
            tw, ms = b.tune()
            assert tw in (4, 8, 16, 32) and ms > 0
            for o in out:
                for v in o.values():
                    v.zero_()
        else:
            b.set_tile(tw)
        b.render()
        b.render()  # graph replay
        torch.cuda.synchronize()
        assert b.check() == 0
        for r, o in zip(ref, out):
            for k in r:
                assert torch.equal(r[k], o[k]), (tw, k)
    b.close()
    for sc in scenes_:
        sc.close()


def test_batch_rejects_bad_views(csg):
    import ctypes
    arr = (csg.csg_view * 1)()
    h = ctypes.c_void_p()
    assert csg.lib().csg_batch_create(arr, 1, ctypes.byref(h)) == csg.CSG_E_ARG
    assert csg.lib().csg_batch_create(arr, 0, ctypes.byref(h)) == csg.CSG_E_ARG
