"""The batched persistent launch (csg_batch_*) writes, for every view, exactly the bytes a
per-view csg_render_planes writes -- for every warp tile shape, every block shape (warps
per block, stack placement), after autotuning, and on graph replay."""
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


SHAPES = [(4, False), (2, False), (8, False), (4, True)]


@pytest.mark.parametrize("deep", [False, True])
def test_batch_block_shapes_equal_per_view_renders(csg, deep):
    """Every block shape, at two tile widths, and the autotuned configuration per class."""
    import torch
    torch.cuda.set_device(0)
    scenes_, views = _views(csg, torch, n_scenes=5, deep=deep, seed=3)
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
    assert b.info()["n_classes"] == len(b.classes()) >= 1

    def run_and_compare(tag):
        for o in out:
            for v in o.values():
                v.zero_()
        b.render()
        b.render()
        torch.cuda.synchronize()
        assert b.check() == 0
        for r, o in zip(ref, out):
            for k in r:
                assert torch.equal(r[k], o[k]), (tag, k)

    for warps, local in SHAPES:
        b.set_shape(warps, local)
        for tw in (8, 16):
            b.set_tile(tw)
            run_and_compare((warps, local, tw))
            for c in b.classes():
                assert (c["warps_per_block"], bool(c["local_stacks"]), c["warp_tile_w"]) == (warps, local, tw)
                assert c["grid"] >= 1 and c["n_items"] >= 1
    tw, ms = b.tune()
    assert ms > 0
    classes = b.classes()
    assert tw == classes[0]["warp_tile_w"]
    assert sum(c["n_views"] for c in classes) == len(views)
    for c in classes:
        assert (c["warps_per_block"], bool(c["local_stacks"])) in SHAPES
        assert c["tuned_ms"] > 0
    info = b.info()
    assert (info["warps_per_block"], bool(info["local_stacks"])) == (classes[0]["warps_per_block"],
                                                                      bool(classes[0]["local_stacks"]))
    run_and_compare("tuned")
    b.close()
    for sc in scenes_:
        sc.close()


def test_batch_rejects_bad_shapes(csg):
    import ctypes
    import torch
    torch.cuda.set_device(0)
    sc = csg.Scene("Sphere 0 0 0 FF0000 1")
    o = torch.zeros(16 * 16, dtype=torch.int32, device="cuda")
    b = csg.Batch([(sc, csg.Camera(), csg.light_dir(), 16, 16, {"rgba8": o.data_ptr()})])
    for warps, local in ((3, 0), (1, 0), (16, 0), (2, 1), (8, 1), (4, 2)):
        assert csg.lib().csg_batch_set_shape(b.h, warps, local) == csg.CSG_E_ARG
    assert csg.lib().csg_batch_set_shape(None, 4, 0) == csg.CSG_E_ARG
    n = b.info()["n_classes"]
    for k, tw, warps, local in ((-1, 8, 4, 0), (n, 8, 4, 0), (0, 6, 4, 0), (0, 8, 3, 0), (0, 8, 8, 1)):
        assert csg.lib().csg_batch_set_class(b.h, k, tw, warps, local) == csg.CSG_E_ARG, (k, tw, warps, local)
    assert csg.lib().csg_batch_set_class(b.h, 0, 16, 2, 0) == csg.CSG_OK
    assert (b.classes()[0]["warp_tile_w"], b.classes()[0]["warps_per_block"]) == (16, 2)
    info = csg.csg_batch_class_info()
    assert csg.lib().csg_batch_get_class(b.h, n, ctypes.byref(info)) == csg.CSG_E_ARG
    b.close()
    sc.close()


def test_batch_rejects_bad_views(csg):
    import ctypes
    arr = (csg.csg_view * 1)()
    h = ctypes.c_void_p()
    assert csg.lib().csg_batch_create(arr, 1, ctypes.byref(h)) == csg.CSG_E_ARG
    assert csg.lib().csg_batch_create(arr, 0, ctypes.byref(h)) == csg.CSG_E_ARG


def test_batch_writes_page_locked_host_planes(csg):
    """Views whose planes are page-locked host memory: the kernel writes them directly, the
    bytes equal the device renders; a copied configuration (copy_config) is the tuned one;
    pageable host planes are refused."""
    import ctypes
    import torch
    torch.cuda.set_device(0)
    scenes_, views = _views(csg, torch, n_scenes=4, seed=7)
    ref, dev_views, host_out, host_views = [], [], [], []
    for sc, cam, light, w, h in views:
        r = _alloc(torch, w, h)
        sc.render_ptrs(cam, light, w, h, **{k: v.data_ptr() for k, v in r.items()})
        ref.append(r)
        dev_views.append((sc, cam, light, w, h, {"rgba8": r["rgba8"].data_ptr()}))
        o = {"rgba8": torch.zeros(w * h, dtype=torch.int32, pin_memory=True),
             "t": torch.zeros(w * h, dtype=torch.float32, pin_memory=True)}
        host_out.append(o)
        host_views.append((sc, cam, light, w, h, {k: v.data_ptr() for k, v in o.items()}))
    torch.cuda.synchronize()
    tuned = csg.Batch(dev_views)
    tuned.tune()
    b = csg.Batch(host_views)
    b.copy_config(tuned)
    for mine, theirs in zip(b.classes(), tuned.classes()):
        for k in ("warp_tile_w", "warps_per_block", "local_stacks"):
            assert mine[k] == theirs[k]
    b.render()
    torch.cuda.synchronize()
    assert b.check() == 0
    for r, o in zip(ref, host_out):
        assert torch.equal(r["rgba8"].cpu(), o["rgba8"])
        assert torch.equal(r["t"].cpu(), o["t"])
    b.close()
    tuned.close()
    # pageable host memory cannot be written by a kernel
    import numpy as np
    sc, cam, light, w, h = views[0]
    page = np.zeros(w * h, dtype=np.int32)
    arr = (csg.csg_view * 1)()
    arr[0].scene = sc.h
    ctypes.memmove(ctypes.byref(arr[0].cam), ctypes.byref(cam.c), 60)
    for k in range(3):
        arr[0].light_dir[k] = float(light[k])
    arr[0].w, arr[0].h = w, h
    arr[0].out = csg.csg_planes(page.ctypes.data, None, None, None, None)
    hb = ctypes.c_void_p()
    assert csg.lib().csg_batch_create(arr, 1, ctypes.byref(hb)) == csg.CSG_E_ARG
    for sc in scenes_:
        sc.close()
