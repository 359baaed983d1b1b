"""csg_render_views_noalloc (the batched render whose scratch is a fixed device array)
writes, on two calls in a row, exactly the bytes the allocating entry points write --
csg_render_planes per view and csg_batch_render for the whole set -- writes page-locked
host planes directly, and rejects view counts beyond its fixed capacity and pageable host
planes before enqueuing anything.  Collected last on purpose:
it must pass after every other test has used the device, as well as alone."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest


def _view_array(csg, views):
    arr = (csg.csg_view * len(views))()
    for i, (scene, cam, light, w, h, planes) in enumerate(views):
        v = arr[i]
        v.scene = scene.h
        ctypes.memmove(ctypes.byref(v.cam), ctypes.byref(cam.c), 60)
        for k in range(3):
            v.light_dir[k] = float(light[k])
        v.w, v.h = int(w), int(h)
        v.out = csg.csg_planes(planes.get("rgba8"), planes.get("rgba32f"), planes.get("t"), planes.get("prim"),
                               planes.get("normal"))
    return arr


def test_noalloc_rejects_bad_counts_without_gpu(csg):
    lib = csg.lib()
    cap = 4096
    assert lib.csg_render_views_noalloc(None, 1, 8, None) == csg.CSG_E_ARG
    arr = (csg.csg_view * 1)()
    assert lib.csg_render_views_noalloc(arr, 0, 8, None) == csg.CSG_E_ARG
    assert lib.csg_render_views_noalloc(arr, -3, 8, None) == csg.CSG_E_ARG
    big = (csg.csg_view * (cap + 1))()
    assert lib.csg_render_views_noalloc(big, cap + 1, 8, None) == csg.CSG_E_CAPACITY
    assert "too small" in lib.csg_status_string(csg.CSG_E_CAPACITY).decode()


@pytest.mark.gpu
def test_noalloc_matches_allocating_entry_points_twice_in_a_row(csg):
    import torch
    from csgrt import scenes

    torch.cuda.set_device(0)
    rng = np.random.default_rng(77)
    texts = [scenes.write_text(scenes.wikipedia_tree()), scenes.write_text(scenes.cheese_tree(5, 48)),
             scenes.write_text(scenes.random_tree(31, 2, 400, 12)), scenes.write_text(scenes.random_tree(8, 2, 40, 6))]
    objs = [csg.Scene(t) for t in texts]
    names = ("rgba8", "rgba32f", "t", "prim", "normal")

    def planes_for(w, h):
        n = w * h
        return {"rgba8": torch.zeros(n, dtype=torch.int32, device="cuda"),
                "rgba32f": torch.zeros(4 * n, dtype=torch.float32, device="cuda"),
                "t": torch.zeros(n, dtype=torch.float32, device="cuda"),
                "prim": torch.zeros(n, dtype=torch.int32, device="cuda"),
                "normal": torch.zeros(3 * n, dtype=torch.float32, device="cuda")}

    specs = []
    for sc in objs:
        for _ in range(3):
            w, h = int(rng.integers(17, 180)), int(rng.integers(9, 140))
            cam = csg.Camera.look_at_origin(scenes.seeded_direction(rng), 3.5)
            specs.append((sc, cam, csg.light_dir(), w, h))

    # allocating entry points: per-view renders and one csg_batch render
    ref = []
    for sc, cam, light, w, h in specs:
        r = planes_for(w, h)
        sc.render_ptrs(cam, light, w, h, **{k: r[k].data_ptr() for k in names})
        ref.append(r)
    bout = [planes_for(w, h) for _, _, _, w, h in specs]
    batch = csg.Batch([(sc, cam, light, w, h, {k: o[k].data_ptr() for k in names})
                       for (sc, cam, light, w, h), o in zip(specs, bout)])
    batch.render()
    torch.cuda.synchronize()
    for r, o in zip(ref, bout):
        for k in names:
            assert torch.equal(r[k], o[k]), k

    out = [planes_for(w, h) for _, _, _, w, h in specs]
    arr = _view_array(csg, [(sc, cam, light, w, h, {k: o[k].data_ptr() for k in names})
                            for (sc, cam, light, w, h), o in zip(specs, out)])
    stream = torch.cuda.current_stream().cuda_stream
    for call, tw in enumerate((8, 16)):
        for o in out:
            for v in o.values():
                v.fill_(-7)
        rc = csg.lib().csg_render_views_noalloc(arr, len(specs), tw, stream)
        assert rc == csg.CSG_OK, (call, csg.lib().csg_status_string(rc))
        torch.cuda.synchronize()
        for i, (r, o) in enumerate(zip(ref, out)):
            for k in names:
                assert torch.equal(r[k], o[k]), (call, i, k)
    for sc in objs:
        assert sc.check() == 0

    # page-locked host planes are written by the kernel; pageable ones are refused up front
    sc, cam, light, w, h = specs[0]
    pinned = torch.zeros(w * h, dtype=torch.int32, pin_memory=True)
    harr = _view_array(csg, [(sc, cam, light, w, h, {"rgba8": pinned.data_ptr()})])
    assert csg.lib().csg_render_views_noalloc(harr, 1, 8, stream) == csg.CSG_OK
    torch.cuda.synchronize()
    assert torch.equal(pinned, ref[0]["rgba8"].cpu())
    pageable = np.zeros(w * h, dtype=np.int32)
    parr = _view_array(csg, [(sc, cam, light, w, h, {"rgba8": pageable.ctypes.data})])
    assert csg.lib().csg_render_views_noalloc(parr, 1, 8, stream) == csg.CSG_E_ARG
    batch.close()
    for sc in objs:
        sc.close()
