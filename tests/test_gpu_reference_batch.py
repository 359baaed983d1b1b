"""Batched and served renders checked against the reference's own kernels (RefCuda:
RaycastKernel + LightningKernel as Raycaster::Raycast launches them, Raycaster.cu:23-34),
not through the engine's single-view kernel.

The batch is the batched workload's kind: random trees of 2..2,048 leaves, four seeded
cameras each, one scene from every tree-size class the full 256-scene batch holds (stack
classes 4 to 12, both GoTo variants, live masks of 1 to 32 words) plus its heaviest tree,
and a chain deeper than 15 operator levels (the 32-entry class).  Views are a quarter of
the workload's size each way, so the reference's planes fit on the host.  They run
through csg_batch_tune's choice and through forced shapes: 32x1, 16x2 and 4x8 warp tiles,
2, 4 and 8 warps per block, stacks in shared and in local memory.  The served mix is the serving
workload's kind: requests of differing scenes and sizes, batched by the render server with
the size-aware order the benchmark uses.

Every plane of every view: hit mask and primitive index, t and normal bit for bit, float
RGBA bit for bit (RGBA8 follows).  The deep chain, whose 32-entry stacks overflow (the
reference kernel then reads stack slots it never wrote), is checked against the oracle's
fma mode instead: hit, primitive, t and normal bit for bit, RGBA8 within 1 LSB."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# One scene of each (stack class, GoTo variant, live-mask words) class of the 256-scene
# batch of seed 0, and its heaviest tree (191).
BATCH_SCENES = (3, 71, 25, 2, 139, 18, 19, 1, 0, 21, 4, 10, 191)


def _deep_chain():
    from csgrt import scenes
    rng = np.random.default_rng(4)
    tree = ("Sphere", 0.0, 0.0, 0.0, "FF0000", 0.9)
    for i in range(20):
        tree = ("Union" if i % 3 else "Difference", tree, ("Sphere", *rng.uniform(-1, 1, 3), "00FF00", 0.3))
    return scenes.write_text(tree), scenes.seeded_direction(rng)


def _alloc(torch, n):
    return {"rgba8": torch.zeros(n, dtype=torch.int32, device="cuda"),
            "t": torch.zeros(n, dtype=torch.float32, device="cuda"),
            "prim": torch.zeros(n, dtype=torch.int32, device="cuda"),
            "normal": torch.zeros(3 * n, dtype=torch.float32, device="cuda"),
            "rgba32f": torch.zeros(4 * n, dtype=torch.float32, device="cuda")}


def _host(planes):
    return {k: v.cpu().numpy() for k, v in planes.items()}


def _reference(csg, G, text, cam, light, w, h):
    nodes44, prims48, _ = csg.parse_tree(text)
    return G.render(nodes44, prims48, cam.floats(), light, w, h)


def _same_as_reference(ref, got, w, h):
    """Every plane of an engine render against the reference kernel's planes; returns the
    name of the first plane that differs, or None."""
    from oracle import quantize_rgba8
    n = w * h
    hit = ref["hit"] != 0
    if not np.array_equal(got["prim"], np.where(hit, ref["prim"], -1)):
        return "prim"
    t = got["t"].view(np.uint32)
    if not (np.array_equal(t[hit], ref["t"][hit].view(np.uint32)) and np.isposinf(got["t"][~hit]).all()):
        return "t"
    nrm = got["normal"].reshape(3, n).T
    if not np.array_equal(nrm[hit].view(np.uint32), ref["normal"][hit].view(np.uint32)) or nrm[~hit].any():
        return "normal"
    if not np.array_equal(got["rgba32f"].reshape(n, 4).view(np.uint32), ref["rgba"].view(np.uint32)):
        return "rgba32f"
    if not np.array_equal(got["rgba8"].view(np.uint32), quantize_rgba8(ref["rgba"])):
        return "rgba8"
    return None


def _same_as_oracle(oracle, csg, text, cam, light, got, w, h):
    nodes, prims = oracle.parse(text)
    thf = csg.device_tan_half_fov(float(cam.floats()[5]))
    ref = oracle.render(nodes, prims, cam.floats(), light, w, h, mode="fma", tan_half_fov=thf)
    n = w * h
    hit = ref["hit"] != 0
    assert hit.sum() > 0
    assert np.array_equal(got["prim"], np.where(hit, ref["prim"], -1))
    assert np.array_equal(got["t"][hit].view(np.uint32), ref["t"][hit].view(np.uint32))
    nrm = got["normal"].reshape(3, n).T
    assert np.array_equal(nrm[hit].view(np.uint32), ref["normal"][hit].view(np.uint32))
    d = np.abs(got["rgba8"].view(np.uint8).astype(int) - ref["rgba8"].view(np.uint8).astype(int))
    assert d.max() <= 1


def test_batch_against_reference_kernel(csg, oracle):
    import torch
    from csgrt import scenes
    from oracle import RefCuda
    if not RefCuda.available():
        pytest.skip("reference cubin not built")
    torch.cuda.set_device(0)
    G = RefCuda()
    work = scenes.config_batch(0, n_scenes=max(BATCH_SCENES) + 1)
    items = []  # (text, Camera, light, w, h, reference planes or None)
    for s in BATCH_SCENES:
        text, views = work[s]
        for v in views:
            w, h = v.w // 4, v.h // 4
            cam = csg.Camera.from_floats(v.camera)
            items.append((text, cam, v.light, w, h, _reference(csg, G, text, cam, v.light, w, h)))
    deep_text, direction = _deep_chain()
    for k in range(2):
        cam = csg.Camera.look_at_origin(direction if k == 0 else -direction, 3.0)
        items.append((deep_text, cam, csg.light_dir(), 96, 72, None))
    objs = {}
    outs, bviews = [], []
    for text, cam, light, w, h, _ in items:
        sc = objs.get(text) or objs.setdefault(text, csg.Scene(text))
        o = _alloc(torch, w * h)
        outs.append(o)
        bviews.append((sc, cam, light, w, h, {k: v.data_ptr() for k, v in o.items()}))
    b = csg.Batch(bviews)
    assert b.info()["stack_class"] == 32
    classes = b.classes()
    assert len(classes) >= 10
    configs = [("tuned", None), ("32x1, 4 warps, local stacks", (32, 4, True)),
               ("16x2, 2 warps, shared stacks", (16, 2, False)), ("4x8, 8 warps, shared stacks", (4, 8, False))]
    for name, cfg in configs:
        for o in outs:
            for v in o.values():
                v.fill_(-7)
        if cfg is None:
            b.tune()
        else:
            b.set_tile(cfg[0])
            b.set_shape(cfg[1], cfg[2])
        b.render()
        b.render()  # graph replay
        torch.cuda.synchronize()
        assert b.check() == 0
        for (text, cam, light, w, h, ref), o in zip(items, outs):
            got = _host(o)
            if ref is None:
                _same_as_oracle(oracle, csg, text, cam, light, got, w, h)
            else:
                bad = _same_as_reference(ref, got, w, h)
                assert bad is None, (name, bad, w, h)
    for sc in objs.values():
        sc.close()


def test_served_mix_against_reference_kernel(csg):
    import torch
    from csgrt import scenes
    from oracle import RefCuda
    from test_gpu_server import ALL_PLANES, _served
    if not RefCuda.available():
        pytest.skip("reference cubin not built")
    torch.cuda.set_device(0)
    G = RefCuda()
    rng = np.random.default_rng(21)
    texts = [scenes.write_text(scenes.random_tree(7000 + s, 2, 2048, 12)) for s in range(6)]
    texts.append(scenes.write_text(scenes.cheese_tree(5, 128)))
    reqs = []
    for i in range(36):
        sid = int(rng.integers(0, len(texts)))
        side = int(rng.choice([64, 128, 256]))
        w, h = side, int(side * rng.choice([0.5, 0.75, 1.0]))
        reqs.append((sid, csg.Camera.look_at_origin(scenes.seeded_direction(rng), float(rng.uniform(2.5, 4))), w, h))
    light = csg.light_dir()
    with csg.Server(planes=ALL_PLANES, keep_results=True, slots=3, max_batch_views=8, order=2) as srv:
        for t in texts:
            srv.add_scene(t)
        tickets = [srv.submit(csg.Server.request(sid, cam, light, w, h)) for sid, cam, w, h in reqs]
        batched = 0
        for t, (sid, cam, w, h) in zip(tickets, reqs):
            res = srv.wait(t, 120.0)
            assert res.status == csg.CSG_OK
            batched += res.batch_views > 1
            got = {k: v.cpu().numpy() for k, v in _served(torch, res, w, h).items()}
            ref = _reference(csg, G, texts[sid], cam, light, w, h)
            bad = _same_as_reference(ref, got, w, h)
            assert bad is None, (bad, sid, w, h)
            srv.release(t)
        assert batched > 0  # requests shared launches
