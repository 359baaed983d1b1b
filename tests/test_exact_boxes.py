"""Optional exact-box mode (csg_scene_create_ex / csg_tree_parse_ex with
CSG_SCENE_EXACT_BOXES): boxes that contain their primitive, computed identically by the
engine's scene compiler and the oracle, and off by default."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN


def _texts():
    from csgrt import scenes
    out = [scenes.write_text(scenes.wikipedia_tree()), scenes.write_text(scenes.random_tree(3, n_leaves=200)),
           scenes.write_text(scenes.cheese_tree(2, 64))]
    out += [p.read_text() for p in sorted((GOLDEN / "scenes").glob("*.txt"))[:6]]
    return out


def test_engine_and_oracle_compute_the_same_exact_boxes(csg, oracle):
    for text in _texts():
        n_exact, _, _ = csg.parse_tree(text, exact_boxes=True)
        n_ref, _, _ = csg.parse_tree(text)
        o_nodes, _ = oracle.parse(text, exact_boxes=True)
        assert n_exact.tobytes() == o_nodes.tobytes()
        o_ref, _ = oracle.parse(text)
        assert n_ref.tobytes() == o_ref.tobytes()  # default: the reference's boxes


def test_exact_boxes_contain_their_primitives(csg, oracle):
    from csgrt import scenes
    rng = np.random.default_rng(1)
    text = scenes.write_text(scenes.random_tree(9, n_leaves=300))
    nodes, prims = oracle.parse(text, exact_boxes=True)
    ref_nodes, _ = oracle.parse(text)
    tighter = 0
    for i, n in enumerate(nodes):
        if n["prim"] < 0:
            continue
        p = prims[n["prim"]]
        c = p["pos"].astype(np.float64)
        lo, hi = n["box"][:3].astype(np.float64), n["box"][3:].astype(np.float64)
        u = rng.normal(size=(400, 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        if n["type"] == 3:  # sphere surface
            pts = c + float(p["p"][0]) * u
        elif n["type"] == 4:  # cylinder: rim circles and side, about axis V from C = c - h/2 V
            V = np.array(p["p"][2:5], np.float64)
            r, h = float(p["p"][0]), float(p["p"][1])
            w = u - (u @ V)[:, None] * V[None, :] / (V @ V)
            w /= np.linalg.norm(w, axis=1, keepdims=True)
            s = rng.uniform(0, h, 400)
            s[:100], s[100:200] = 0.0, h
            pts = c - h / 2 * V + s[:, None] * V + r * w
        else:
            continue
        assert (pts >= lo - 1e-9).all() and (pts <= hi + 1e-9).all(), (i, n["type"])
        rb = ref_nodes[i]["box"].astype(np.float64)
        tighter += (hi - lo).sum() < (rb[3:] - rb[:3]).sum()
    assert tighter > 0


@pytest.mark.gpu
def test_exact_mode_engine_equals_oracle(csg, oracle):
    """The engine in exact-box mode equals the oracle given the same boxes, bit for bit in
    hit, primitive, t and normal; cylinder scenes gain hits the reference's boxes cut."""
    import torch
    from csgrt import scenes
    torch.cuda.set_device(0)
    for text in _texts()[:3]:
        for exact in (True, False):
            sc = csg.Scene(text, exact_boxes=exact)
            cam = csg.Camera.look_at_origin(scenes.seeded_direction(np.random.default_rng(4)), 3.2)
            w, h = 96, 64
            out = sc.render_torch(cam, csg.light_dir(), w, h, planes=("rgba8", "t", "prim", "normal"))
            nodes, prims = oracle.parse(text, exact_boxes=exact)
            thf = csg.device_tan_half_fov(float(cam.floats()[5]))
            ref = oracle.render(nodes, prims, cam.floats(), csg.light_dir(), w, h, mode="fma", tan_half_fov=thf,
                                want=("hit", "t", "prim", "normal"))
            hit = ref["hit"].astype(bool)
            assert np.array_equal(out["prim"].cpu().numpy() >= 0, hit)
            assert np.array_equal(out["prim"].cpu().numpy()[hit], ref["prim"][hit])
            assert np.array_equal(out["t"].cpu().numpy().view(np.uint32)[hit], ref["t"][hit].view(np.uint32))
            sc.close()
