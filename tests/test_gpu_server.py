"""The render server (csg_server_*): every request's planes are the bytes csg_render_planes
writes for that request alone -- in a batch, in the unbatched form, from several submitting
threads, under an open-loop replay and under a budget small enough to force evictions."""
from __future__ import annotations

import threading

import numpy as np
import pytest

ALL_PLANES = 1 | 2 | 4 | 8 | 16


class _DevArray:
    """A raw device pointer viewed as a 1-D array (CUDA array interface)."""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (int(ptr), False), "version": 3}


def _dev(torch, ptr, n, typestr):
    return torch.as_tensor(_DevArray(ptr, n, typestr), device="cuda")


def _scene_texts():
    from csgrt import scenes
    return [scenes.write_text(scenes.wikipedia_tree()), scenes.write_text(scenes.cheese_tree(3, 40)),
            scenes.write_text(scenes.random_tree(11, 2, 300, 12)), scenes.write_text(scenes.random_tree(12, 2, 60, 8)),
            scenes.write_text(scenes.random_tree(13, 2, 1200, 12))]


def _alone(csg, torch, scene_obj, cam, light, w, h):
    n = w * h
    r = {"rgba8": torch.zeros(n, dtype=torch.int32, device="cuda"),
         "t": torch.zeros(n, dtype=torch.float32, device="cuda"),
         "prim": torch.zeros(n, dtype=torch.int32, device="cuda"),
         "normal": torch.zeros(3 * n, dtype=torch.float32, device="cuda"),
         "rgba32f": torch.zeros(4 * n, dtype=torch.float32, device="cuda")}
    scene_obj.render_ptrs(cam, light, w, h, **{k: v.data_ptr() for k, v in r.items()})
    torch.cuda.synchronize()
    return r


def _served(torch, res, w, h):
    n = w * h
    p = res.planes
    return {"rgba8": _dev(torch, p.rgba8, n, "<i4"), "t": _dev(torch, p.t, n, "<f4"),
            "prim": _dev(torch, p.prim, n, "<i4"), "normal": _dev(torch, p.normal, 3 * n, "<f4"),
            "rgba32f": _dev(torch, p.rgba32f, 4 * n, "<f4")}


def _requests(csg, n, n_scenes, seed, alone_every=0):
    from csgrt import scenes
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        sid = int(rng.integers(0, n_scenes))
        w, h = int(rng.integers(8, 160)), int(rng.integers(8, 120))
        cam = csg.Camera.look_at_origin(scenes.seeded_direction(rng), 3.5)
        alone = bool(alone_every) and i % alone_every == 0
        out.append((sid, cam, csg.light_dir(), w, h, alone))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("order", [0, 2])
def test_server_results_equal_alone_renders(csg, order):
    """order 0: arrival order; 2: size-aware (deadline order, priority streams, blocks that
    retire every few warp tiles)."""
    import torch
    torch.cuda.set_device(0)
    texts = _scene_texts()
    objs = [csg.Scene(t) for t in texts]
    with csg.Server(planes=ALL_PLANES, keep_results=True, slots=3, max_batch_views=8, order=order) as srv:
        ids = [srv.add_scene(t) for t in texts]
        assert ids == list(range(len(texts)))
        reqs = _requests(csg, 40, len(texts), 5, alone_every=5)
        tickets = [srv.submit(csg.Server.request(sid, cam, light, w, h, alone=a))
                   for sid, cam, light, w, h, a in reqs]
        batched_sizes = []
        for t, (sid, cam, light, w, h, a) in zip(tickets, reqs):
            res = srv.wait(t, 60.0)
            assert res.status == csg.CSG_OK
            assert res.t_arrive <= res.t_launch <= res.t_done
            if a:
                assert res.batch_views == 1
            else:
                batched_sizes.append(res.batch_views)
            ref = _alone(csg, torch, objs[sid], cam, light, w, h)
            got = _served(torch, res, w, h)
            for k in ref:
                assert torch.equal(ref[k], got[k]), (k, sid, w, h, a)
            srv.release(t)
        assert max(batched_sizes) > 1  # requests were batched together
        st = srv.stats()
        assert st["requests_done"] == 40 and st["output_bytes"] == 0
    for o in objs:
        o.close()


@pytest.mark.gpu
def test_server_threads_and_host_copies(csg):
    import torch
    torch.cuda.set_device(0)
    texts = _scene_texts()
    objs = [csg.Scene(t) for t in texts]
    reqs = _requests(csg, 32, len(texts), 9)
    hosts = [torch.zeros(w * h, dtype=torch.int32, pin_memory=True) for _, _, _, w, h, _ in reqs]
    with csg.Server(slots=2, max_batch_views=6) as srv:
        for t in texts:
            srv.add_scene(t)
        tickets = [None] * len(reqs)

        def worker(k):
            for i in range(k, len(reqs), 4):
                sid, cam, light, w, h, _ = reqs[i]
                tickets[i] = srv.submit(csg.Server.request(sid, cam, light, w, h, host_rgba8=hosts[i].data_ptr()))

        th = [threading.Thread(target=worker, args=(k,)) for k in range(4)]
        for x in th:
            x.start()
        for x in th:
            x.join()
        for i, t in enumerate(tickets):
            res = srv.wait(t, 60.0)
            assert res.status == csg.CSG_OK
            srv.release(t)
    for i, (sid, cam, light, w, h, _) in enumerate(reqs):
        ref = _alone(csg, torch, objs[sid], cam, light, w, h)["rgba8"].cpu()
        assert torch.equal(ref, hosts[i]), i
    for o in objs:
        o.close()


@pytest.mark.gpu
def test_server_replay_and_budget_evictions(csg):
    import torch
    torch.cuda.set_device(0)
    from csgrt import scenes
    texts = [scenes.write_text(scenes.random_tree(40 + i, n_leaves=n)) for i, n in enumerate((1500, 900, 600, 300))]
    objs = [csg.Scene(t) for t in texts]
    with csg.Server() as probe:
        ids = [probe.add_scene(t) for t in texts]
        for i in ids:
            probe.preload(i)
        scene_bytes = probe.stats()["scene_bytes"]
    sizes = [o.info()["device_bytes"] for o in objs]
    assert scene_bytes == sum(sizes)
    # room for the largest scene, the outputs of two batches in flight and half of the second
    # largest scene: the two largest never fit together, so requests cycling over the scenes
    # force evictions
    reqs = [(sid, cam, light, min(w, 64), min(h, 64), a) for sid, cam, light, w, h, a in _requests(csg, 30, 4, 21)]
    max_out = 64 * 64 * 4 + 256
    budget = sorted(sizes)[-1] + 2 * 4 * max_out + sorted(sizes)[-2] // 2
    assert budget < sum(sizes)
    hosts = [torch.zeros(w * h, dtype=torch.int32, pin_memory=True) for _, _, _, w, h, _ in reqs]
    with csg.Server(hbm_budget=budget, slots=2, max_batch_views=4) as srv:
        for t in texts:
            srv.add_scene(t)
        rq = [csg.Server.request(sid, cam, light, w, h, host_rgba8=hosts[i].data_ptr())
              for i, (sid, cam, light, w, h, _) in enumerate(reqs)]
        arrivals = np.cumsum(np.random.default_rng(2).exponential(1e-3, len(rq)))
        res, _, wall = srv.replay(rq, arrivals)
        assert wall > 0
        for r in res:
            assert r.status == csg.CSG_OK
            assert r.t_done >= r.t_launch >= r.t_arrive - 1e-6
        st = srv.stats()
        assert st["evictions"] > 0 and st["peak_bytes"] <= budget
        # a request whose outputs alone exceed the budget is refused, not queued forever
        big = csg.Server.request(0, reqs[0][1], reqs[0][2], 4096, 4096)
        t = srv.submit(big)
        assert srv.wait(t, 30.0).status == csg.CSG_E_BUDGET
        srv.release(t)
    for i, (sid, cam, light, w, h, _) in enumerate(reqs):
        ref = _alone(csg, torch, objs[sid], cam, light, w, h)["rgba8"].cpu()
        assert torch.equal(ref, hosts[i]), i
    for o in objs:
        o.close()


@pytest.mark.gpu
def test_server_release_while_batch_runs(csg):
    """Requests retire one by one (per-view completion flags) and may be released while the
    rest of their batch is still rendering; with several threads submitting, waiting and
    releasing, every result is right when read and the server ends with no memory held."""
    import torch
    torch.cuda.set_device(0)
    texts = _scene_texts()
    objs = [csg.Scene(t) for t in texts]
    reqs = _requests(csg, 120, len(texts), 33)
    errors = []
    with csg.Server(planes=1 | 4, keep_results=True, slots=2, max_batch_views=64) as srv:
        for t in texts:
            srv.add_scene(t)

        def worker(k):
            try:
                for i in range(k, len(reqs), 4):
                    sid, cam, light, w, h, _ = reqs[i]
                    t = srv.submit(csg.Server.request(sid, cam, light, w, h))
                    res = srv.wait(t, 60.0)
                    assert res.status == csg.CSG_OK
                    if i % 7 == 0:  # check some results before releasing them
                        got = _dev(torch, res.planes.prim, w * h, "<i4").clone()
                        ref = _alone(csg, torch, objs[sid], cam, light, w, h)["prim"]
                        assert torch.equal(got, ref), i
                    srv.release(t)
            except Exception as e:  # noqa: BLE001 -- reported below
                errors.append(repr(e))

        th = [threading.Thread(target=worker, args=(k,)) for k in range(4)]
        for x in th:
            x.start()
        for x in th:
            x.join()
        assert not errors, errors
        import time
        deadline = time.time() + 30.0
        while srv.stats()["output_bytes"] and time.time() < deadline:
            time.sleep(0.01)  # launches whose requests were released early are still ending
        st = srv.stats()
        assert st["requests_done"] == len(reqs)
        assert st["output_bytes"] == 0
    for o in objs:
        o.close()


@pytest.mark.gpu
@pytest.mark.parametrize("order", [0, 1, 2])
def test_server_result_is_complete_when_reported_done(csg, order):
    """A request counts as done only once its frame is in place: each RGBA8 frame goes to
    pinned host memory (written by the kernel), pre-filled with a sentinel, and is read on
    the CPU the moment wait() returns, with no GPU synchronisation in between.  Large views
    of large trees, alone and batched, in every admission order."""
    import torch
    from csgrt import scenes
    torch.cuda.set_device(0)
    texts = [scenes.write_text(scenes.random_tree(900 + i, 200, 2048, 12)) for i in range(3)]
    objs = [csg.Scene(t) for t in texts]
    rng = np.random.default_rng(31)
    reqs = []
    for i in range(18):
        side = int(rng.choice([64, 512, 1024]))
        cam = csg.Camera.look_at_origin(scenes.seeded_direction(rng), 3.0)
        reqs.append((i % 3, cam, csg.light_dir(), side, side, i % 4 == 0))
    sentinel = np.int32(0x5A5A5A5A)
    hosts = [torch.full((w * h,), int(sentinel), dtype=torch.int32, pin_memory=True) for *_, w, h, _ in reqs]
    with csg.Server(slots=3, max_batch_views=4, order=order) as srv:
        for t in texts:
            srv.add_scene(t)
        tickets = [srv.submit(csg.Server.request(sid, cam, light, w, h, alone=a, host_rgba8=hosts[i].data_ptr()))
                   for i, (sid, cam, light, w, h, a) in enumerate(reqs)]
        frames = []
        for t, hb in zip(tickets, hosts):
            res = srv.wait(t, 120.0)
            assert res.status == csg.CSG_OK
            frames.append(hb.numpy().copy())  # at once: no synchronisation with the GPU
            srv.release(t)
    for i, (sid, cam, light, w, h, _) in enumerate(reqs):
        ref = _alone(csg, torch, objs[sid], cam, light, w, h)["rgba8"].cpu().numpy()
        assert np.array_equal(frames[i], ref), (i, w, int((frames[i] == sentinel).sum()))
    for o in objs:
        o.close()
