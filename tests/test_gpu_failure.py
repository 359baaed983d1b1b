"""Device-side failure detection without a GPU fault: the traversal's per-ray iteration cap
(the kernels' only bounded loop) is lowered until rays run out of it; they are written as
misses and counted, csg_scene_check / csg_batch_check report CSG_E_TIMEOUT, every other
pixel is the uncapped render's, and the context stays usable."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_iteration_cap_runs_out_and_is_reported(csg):
    import torch
    from csgrt import scenes
    torch.cuda.set_device(0)
    text = scenes.config_scene_text(2, 0)
    view = scenes.config_views(2, 0)[0]
    cam = csg.Camera.from_floats(view.camera)
    w, h = 384, 216
    lib = csg.lib()
    try:
        with csg.Scene(text) as sc:
            ref = sc.render_torch(cam, view.light, w, h, planes=("rgba8", "prim"))
            torch.cuda.synchronize()
            assert sc.check() == 0
            assert lib.csg_set_iteration_cap(4) == csg.CSG_OK
            out = sc.render_torch(cam, view.light, w, h, planes=("rgba8", "prim"))
            torch.cuda.synchronize()
            n_capped = sc.check()
            assert n_capped > 0
            rp, op = ref["prim"].cpu().numpy(), out["prim"].cpu().numpy()
            diff = rp != op
            assert 0 < diff.sum() <= n_capped
            assert (op[diff] == -1).all()  # a capped ray is a miss
            background = out["rgba8"].cpu().numpy()[diff]
            assert (background == background[0]).all()
            same = ~diff
            assert np.array_equal(ref["rgba8"].cpu().numpy()[same], out["rgba8"].cpu().numpy()[same])

            # a batch created under the lowered cap keeps it
            o = torch.zeros(w * h, dtype=torch.int32, device="cuda")
            b = csg.Batch([(sc, cam, view.light, w, h, {"rgba8": o.data_ptr()})])
            b.render()
            torch.cuda.synchronize()
            assert b.check() > 0
            assert torch.equal(o, out["rgba8"])
            b.close()

            # restored: the context is usable and nothing is capped
            assert lib.csg_set_iteration_cap(0) == csg.CSG_OK
            again = sc.render_torch(cam, view.light, w, h, planes=("rgba8", "prim"))
            torch.cuda.synchronize()
            assert sc.check() == 0
            assert torch.equal(again["rgba8"], ref["rgba8"]) and torch.equal(again["prim"], ref["prim"])
    finally:
        lib.csg_set_iteration_cap(0)


def test_server_counts_capped_rays(csg):
    """Served requests (batched and one launch each) whose rays reach the cap still complete;
    the server's statistics count the capped rays."""
    from csgrt import scenes
    text = scenes.config_scene_text(2, 0)
    view = scenes.config_views(2, 0)[0]
    cam = csg.Camera.from_floats(view.camera)
    lib = csg.lib()
    srv = csg.Server(hbm_budget=2 << 30, slots=2, max_batch_views=16)
    try:
        sid = srv.add_scene(text)
        res, _, _ = srv.replay([csg.Server.request(sid, cam, view.light, 128, 96, alone=a) for a in (False, True)],
                               [0.0, 0.0])
        assert all(r.status == 0 for r in res)
        assert srv.stats()["capped_rays"] == 0
        assert lib.csg_set_iteration_cap(4) == csg.CSG_OK
        res, _, _ = srv.replay([csg.Server.request(sid, cam, view.light, 128, 96, alone=a) for a in (False, True)],
                               [0.0, 0.0])
        assert all(r.status == 0 for r in res)
        capped = srv.stats()["capped_rays"]
        assert capped > 0
        lib.csg_set_iteration_cap(0)
        res, _, _ = srv.replay([csg.Server.request(sid, cam, view.light, 128, 96, alone=a) for a in (False, True)],
                               [0.0, 0.0])
        assert all(r.status == 0 for r in res)
        assert srv.stats()["capped_rays"] == capped  # no new ones
    finally:
        lib.csg_set_iteration_cap(0)
        srv.close()
