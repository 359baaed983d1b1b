"""Edge cases against the reference kernel and the oracle: degenerate and coincident
geometry (ties, zero radius or height, tangent primitives, a 10-level chain of identical
spheres), cameras on the coordinate axes (direction components exactly zero, so the box
tests take their exact fallback), inside a primitive and facing away, and ragged or
one-pixel frames.

One-pixel-wide or -high frames make the reference's ray generation divide by zero
(u = (x + 0.5) / (W - 1)), so every ray is NaN; they are checked against the oracle only
(the engine stops any ray at its iteration cap, the reference kernel has no cap)."""
from __future__ import annotations

import numpy as np
import pytest

from test_gpu_parity import assert_bit_exact, engine_render

pytestmark = pytest.mark.gpu


def _scenes():
    s = lambda x, y, z, c, r: f"Sphere {x} {y} {z} {c} {r}"
    chain = s(0, 0, 0, "FF0000", 0.8)
    for i in range(10):
        chain = f"{['Union', 'Intersection', 'Difference'][i % 3]}\n{chain}\n{s(0, 0, 0, '00FF00', 0.8)}"
    return {
        "union-identical": f"Union\n{s(0, 0, 0, 'FF0000', 1)}\n{s(0, 0, 0, '00FF00', 1)}",
        "intersection-identical": f"Intersection\n{s(0, 0, 0, 'FF0000', 1)}\n{s(0, 0, 0, '00FF00', 1)}",
        "difference-identical": f"Difference\n{s(0, 0, 0, 'FF0000', 1)}\n{s(0, 0, 0, '00FF00', 1)}",
        "zero-radius": f"Union\n{s(0, 0, 0, 'FF0000', 0)}\n{s(0.5, 0, 0, '00FF00', 0.5)}",
        "zero-height-cylinder": "Union\nCylinder 0 0 0 FF0000 0.7 0 90 0 0\nSphere 0 0 0 00FF00 0.3",
        "tangent-spheres": f"Union\n{s(-0.5, 0, 0, 'FF0000', 0.5)}\n{s(0.5, 0, 0, '00FF00', 0.5)}",
        "cube-sphere-tangent": "Difference\nCube 0 0 0 FF0000 2\nSphere 0 0 0 00FF00 1",
        "identical-chain": chain,
    }


def _cameras(csg):
    return {
        "axis": csg.Camera().set_fov(60).floats(),                                 # (0,0,5) looking down -z
        "axis-x": csg.Camera().set_position(5, 0, 0).set_rotation(0, np.pi / 2).set_fov(60).floats(),
        "inside": csg.Camera().set_position(0, 0, 0.1).set_fov(90).floats(),
        "away": csg.Camera().set_position(0, 0, 5).set_rotation(0, np.pi).set_fov(60).floats(),
    }


SIZES = [(2, 2), (17, 13), (64, 48), (3, 64)]


def test_degenerate_scenes_vs_reference_kernel(csg, oracle):
    from oracle import RefCuda, quantize_rgba8
    from conftest import ulp_equal
    if not RefCuda.available():
        pytest.skip("reference cubin not built on this machine")
    G = RefCuda()
    light = np.float32([-1, -1, -1])
    for sname, text in _scenes().items():
        nodes44, prims48, _ = csg.parse_tree(text)
        for cname, cam in _cameras(csg).items():
            for w, h in SIZES:
                name = f"{sname}/{cname}/{w}x{h}"
                eng = engine_render(csg, text, cam, light, w, h)
                ref = G.render(nodes44, prims48, cam, light, w, h)
                ref["rgba8"] = quantize_rgba8(ref["rgba"])
                assert_bit_exact(eng, ref, name)
                assert ulp_equal(eng["rgba32f"], ref["rgba"]).all(), name


def test_one_pixel_frames_vs_oracle(csg, oracle):
    """W or H of 1: NaN rays.  The engine's planes equal the oracle's (all misses here)."""
    import torch
    light = np.float32([-1, -1, -1])
    for sname, text in list(_scenes().items())[:4]:
        nodes, prims = oracle.parse(text)
        for w, h in ((1, 1), (1, 9), (9, 1)):
            cam = csg.Camera().set_fov(60)
            with csg.Scene(text) as sc:
                out = sc.render_torch(cam, light, w, h, planes=("rgba8", "t", "prim"))
                torch.cuda.synchronize()
                sc.check()
            thf = csg.device_tan_half_fov(float(cam.floats()[5]))
            ref = oracle.render(nodes, prims, cam.floats(), light, w, h, mode="fma", tan_half_fov=thf,
                                want=("hit", "t", "prim", "rgba8"))
            prim = out["prim"].cpu().numpy()
            assert np.array_equal(prim >= 0, ref["hit"].astype(bool)), (sname, w, h)
            assert np.array_equal(prim, ref["prim"]), (sname, w, h)
            assert np.array_equal(out["rgba8"].cpu().numpy().view(np.uint32), ref["rgba8"]), (sname, w, h)
