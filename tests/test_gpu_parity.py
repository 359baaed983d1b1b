"""GPU parity of the engine (libcsgrt, through the C ABI) against

* the CPU oracle's "fma" mode (the reference algorithm with nvcc's contraction): hit
  mask, hit primitive, t and normal bit-exact; RGBA8 within 1 LSB (the device powf of the
  shading is the only transcendental the host cannot reproduce);
* the reference's own CUDA kernels (compiled from the reference sources for sm_103a and
  launched as Raycaster::Raycast does), where that cubin was built: every plane
  bit-exact, float RGBA included.

Full-size frames are checked against the reference kernel in full and against the
oracle on a seeded pixel sample.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, load_cases, scene_text, ulp_equal

pytestmark = pytest.mark.gpu

HOST_CASES = load_cases(GOLDEN / "ref_host.npz")
GPU_NPZ = GOLDEN / "ref_gpu.npz"
GPU_CASES = load_cases(GPU_NPZ) if GPU_NPZ.exists() else {}


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    torch.cuda.set_device(0)
    return torch


@pytest.fixture(scope="module")
def refcuda():
    from oracle import RefCuda
    if not RefCuda.available():
        pytest.skip("reference cubin not built on this machine")
    return RefCuda()


def engine_render(csg, text, cam_floats, light, w, h, planes=("rgba8", "t", "prim", "normal", "rgba32f"),
                  fine_mask=False):
    import torch
    cam = csg.Camera.from_floats(cam_floats)
    with csg.Scene(text, fine_mask=fine_mask) as sc:
        out = sc.render_torch(cam, light, w, h, planes=planes)
        torch.cuda.synchronize()
        assert sc.check() == 0
        res = {}
        for k, v in out.items():
            a = v.cpu().numpy()
            if k == "rgba8":
                a = a.view(np.uint32)
            if k == "normal":
                a = a.reshape(3, -1).T.copy()
            res[k] = a
    res["hit"] = (res["prim"] >= 0).astype(np.uint8) if "prim" in res else None
    return res


# Tolerances.  Engine vs the reference CUDA kernel: every plane bit-exact (hit mask,
# primitive, t, normal, float RGBA; RGBA8 is the float RGBA quantised).  Engine vs the
# oracle: hit mask, primitive, t and normal bit-exact; RGBA8 within 1 LSB (the host powf
# of the oracle's shading differs from the device powf in the last bits).


def assert_bit_exact(a, b, name, rgba_lsb=1):
    assert (a["hit"] == b["hit"]).all(), f"{name}: hit mask differs at {(a['hit'] != b['hit']).sum()} px"
    m = b["hit"] == 1
    assert (a["prim"][m] == b["prim"][m]).all(), f"{name}: primitive ids differ"
    bad_t = ~ulp_equal(a["t"][m], b["t"][m])
    assert not bad_t.any(), f"{name}: t differs at {bad_t.sum()} px"
    bad_n = ~ulp_equal(a["normal"][m], b["normal"][m]).all(1)
    assert not bad_n.any(), f"{name}: normal differs at {bad_n.sum()} px"
    if rgba_lsb is not None and "rgba8" in a and "rgba8" in b:
        d = np.abs(a["rgba8"].view(np.uint8).astype(int) - b["rgba8"].view(np.uint8).astype(int))
        assert d.max() <= rgba_lsb, f"{name}: RGBA8 differs by {d.max()} LSB"


@pytest.mark.parametrize("case", sorted(HOST_CASES))
def test_engine_matches_oracle_on_golden_cases(csg, oracle, torch_cuda, case):
    g = HOST_CASES[case]
    w, h = (int(v) for v in g["size"])
    text = scene_text(case)
    eng = engine_render(csg, text, g["camera"], g["light"], w, h)
    nodes, prims = oracle.parse(text)
    thf = csg.device_tan_half_fov(float(g["camera"][5]))
    ref = oracle.render(nodes, prims, g["camera"], g["light"], w, h, mode="fma", tan_half_fov=thf)
    assert_bit_exact(eng, ref, case)


@pytest.mark.skipif(not GPU_CASES, reason="reference GPU fixtures not generated yet")
@pytest.mark.parametrize("case", sorted(GPU_CASES))
def test_engine_matches_reference_kernel_fixtures(csg, torch_cuda, case):
    g = GPU_CASES[case]
    w, h = (int(v) for v in g["size"])
    eng = engine_render(csg, scene_text(case), g["camera"], g["light"], w, h)
    assert_bit_exact(eng, g, case)
    if "rgba_hit" in g:
        m = g["hit"] == 1
        assert ulp_equal(eng["rgba32f"][m], g["rgba_hit"]).all(), f"{case}: float RGBA differs"


def _live_cases():
    from csgrt import scenes
    import csgrt
    rng = np.random.default_rng(21)
    out = [("wiki-c1", scenes.write_text(scenes.wikipedia_tree()), csgrt.Camera().set_fov(60).floats(),
            np.float32([-1, -1, -1]), 1280, 720)]
    for seed in range(2):
        out.append((f"cheese{seed}", scenes.write_text(scenes.cheese_tree(seed)),
                    csgrt.Camera.look_at_origin(scenes.seeded_direction(rng)).floats(), csgrt.light_dir(), 640, 360))
    for seed in range(6):
        out.append((f"random{seed}", scenes.write_text(scenes.random_tree(seed)),
                    csgrt.Camera.look_at_origin(scenes.seeded_direction(rng), 3.0).floats(), csgrt.light_dir(),
                    480, 270))
    for f in sorted((GOLDEN / "scenes").glob("*.txt")):
        out.append((f.stem, f.read_text(), csgrt.Camera().set_fov(60).floats(), np.float32([-1, -1, -1]), 320, 180))
    return out


def test_engine_matches_reference_kernel_live(csg, torch_cuda, refcuda):
    from oracle import quantize_rgba8
    for name, text, cam, light, w, h in _live_cases():
        eng = engine_render(csg, text, cam, light, w, h)
        nodes44, prims48, _ = csg.parse_tree(text)
        ref = refcuda.render(nodes44, prims48, cam, light, w, h)
        ref["rgba8"] = quantize_rgba8(ref["rgba"])
        assert_bit_exact(eng, ref, name)
        assert ulp_equal(eng["rgba32f"], ref["rgba"]).all(), f"{name}: float RGBA differs"


@pytest.mark.parametrize("config", [2, 3])
def test_full_size_frame_vs_reference_kernel(csg, oracle, torch_cuda, refcuda, config):
    """Configurations 2 (cheese-512, 3840x2160) and 3 (random tree, 1920x1080) at full size:
    every pixel against the reference kernel; a seeded sample against the oracle."""
    from csgrt import scenes
    from oracle import quantize_rgba8
    text = scenes.config_scene_text(config, 0)
    view = scenes.config_views(config, 0)[0]
    eng = engine_render(csg, text, view.camera, view.light, view.w, view.h, planes=("rgba8", "t", "prim", "normal"))
    nodes44, prims48, _ = csg.parse_tree(text)
    ref = refcuda.render(nodes44, prims48, view.camera, view.light, view.w, view.h)
    ref["rgba8"] = quantize_rgba8(ref["rgba"])
    assert_bit_exact(eng, ref, f"config{config}")
    rng = np.random.default_rng(config)
    pix = rng.integers(0, view.w * view.h, 20000)
    nodes, prims = oracle.parse(text)
    thf = csg.device_tan_half_fov(float(view.camera[5]))
    o = oracle.render_list(nodes, prims, view.camera, view.light, view.w, view.h, pix, mode="fma",
                           tan_half_fov=thf, want=("hit", "t", "prim", "normal", "rgba8"))
    sub = {k: eng[k][pix] for k in ("hit", "t", "prim", "normal", "rgba8")}
    assert_bit_exact(sub, o, f"config{config}-oracle-sample")


def test_full_size_cheese_vs_oracle_without_reference(csg, oracle, torch_cuda):
    """Configuration 2 at full size against the oracle on a pixel sample (runs even where
    the reference cubin is absent)."""
    from csgrt import scenes
    text = scenes.config_scene_text(2, 0)
    view = scenes.config_views(2, 0)[0]
    eng = engine_render(csg, text, view.camera, view.light, view.w, view.h, planes=("rgba8", "t", "prim", "normal"))
    rng = np.random.default_rng(99)
    pix = rng.integers(0, view.w * view.h, 30000)
    nodes, prims = oracle.parse(text)
    thf = csg.device_tan_half_fov(float(view.camera[5]))
    o = oracle.render_list(nodes, prims, view.camera, view.light, view.w, view.h, pix, mode="fma",
                           tan_half_fov=thf, want=("hit", "t", "prim", "normal", "rgba8"))
    sub = {k: eng[k][pix] for k in ("hit", "t", "prim", "normal", "rgba8")}
    assert_bit_exact(sub, o, "cheese-full-sample")
    assert sub["hit"].mean() > 0.05


def test_deep_tree_uses_32_entry_stacks(csg, oracle, torch_cuda):
    """A chain of 24 operators (deeper than the 15 levels the small stack classes cover):
    the engine reproduces the reference's 32-entry stacks, including dropped pushes."""
    from csgrt import scenes
    import csgrt
    tree = ("Sphere", 0, 0, 0, "FF0000", 0.9)
    rng = np.random.default_rng(4)
    for i in range(24):
        leaf = ("Sphere", *rng.uniform(-1, 1, 3), "00FF00", 0.3) if i % 3 else ("Cube", *rng.uniform(-1, 1, 3), "0000FF", 0.5)
        tree = (["Union", "Difference", "Intersection"][i % 3] if i % 5 else "Union", tree, leaf)
    text = scenes.write_text(tree)
    with csg.Scene(text) as sc:
        assert sc.info()["stack_class"] == 32
    cam = csgrt.Camera.look_at_origin([0.3, 0.4, 1.0], 3.5).floats()
    light = csgrt.light_dir()
    eng = engine_render(csg, text, cam, light, 128, 96)
    nodes, prims = oracle.parse(text)
    thf = csg.device_tan_half_fov(float(cam[5]))
    ref = oracle.render(nodes, prims, cam, light, 128, 96, mode="fma", tan_half_fov=thf)
    assert_bit_exact(eng, ref, "deep")


def test_planes_agree_and_stream_ordering(csg, torch_cuda):
    """rgba8 equals the quantised rgba32f; rendering on a side stream gives the same frame."""
    import torch
    from csgrt import scenes
    from oracle import quantize_rgba8
    text = scenes.config_scene_text(3, 1)
    view = scenes.config_views(3, 1)[0]
    cam = csg.Camera.from_floats(view.camera)
    w, h = 640, 360
    with csg.Scene(text) as sc:
        a = sc.render_torch(cam, view.light, w, h, planes=("rgba8", "rgba32f"))
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            b = sc.render_torch(cam, view.light, w, h, planes=("rgba8",), stream=s)
        s.synchronize()
        torch.cuda.synchronize()
    q = quantize_rgba8(a["rgba32f"].cpu().numpy())
    assert (a["rgba8"].cpu().numpy().view(np.uint32) == q).all()
    assert torch.equal(a["rgba8"], b["rgba8"])


def test_render_rejects_misaligned_float4_output(csg, torch_cuda):
    import ctypes
    import torch
    from csgrt import scenes
    buf = torch.empty(16 * 16 * 4 + 1, dtype=torch.float32, device="cuda")
    cam = csg.Camera()
    light = (ctypes.c_float * 3)(-1, -1, -1)
    with csg.Scene(scenes.write_text(scenes.wikipedia_tree())) as sc:
        rc = csg.lib().csg_render_f4(sc.h, ctypes.byref(cam.c), light, 16, 16, ctypes.c_void_p(buf.data_ptr() + 4),
                                    None)
        assert rc == csg.CSG_E_ARG
        rc = csg.lib().csg_render_f4(sc.h, ctypes.byref(cam.c), light, 16, 16, ctypes.c_void_p(buf.data_ptr()), None)
        assert rc == csg.CSG_OK
    torch.cuda.synchronize()


def test_rays_without_live_leaves_vs_reference_kernel(csg, torch_cuda, refcuda):
    """Views where most rays meet no primitive (a ray whose live mask is empty after the
    pre-pass is written as the background without a traversal): the cheese scene seen from
    behind the camera's usual side, from far away and at grazing angles, and random trees
    framed so the object fills a corner; every plane against the reference kernel."""
    from csgrt import scenes
    from oracle import quantize_rgba8
    light = np.float32(csg.light_dir())
    rng = np.random.default_rng(77)
    cases = [(scenes.config_scene_text(2, 0), d, dist) for d, dist in
             (((0.0, 0.0, 1.0), 12.0), ((0.3, 0.95, 0.1), 2.2), ((1.0, 0.0, 0.0), 1.75))]
    cases += [(scenes.write_text(scenes.random_tree(31000 + s, 64, 600, 10)), scenes.seeded_direction(rng),
               float(rng.uniform(2.0, 6.0))) for s in range(4)]
    for k, (text, d, dist) in enumerate(cases):
        cam = csg.Camera.look_at_origin(np.array(d, float), dist).floats()
        cam = cam.copy()
        cam[0:3] += np.float32(0.6) * cam[9:12]  # shift the eye sideways: the object off centre
        eng = engine_render(csg, text, cam, light, 160, 120)
        nodes44, prims48, _ = csg.parse_tree(text)
        ref = refcuda.render(nodes44, prims48, cam, light, 160, 120)
        ref["rgba8"] = quantize_rgba8(ref["rgba"])
        assert_bit_exact(eng, ref, f"sparse view {k}")
        assert ulp_equal(eng["rgba32f"], ref["rgba"]).all(), f"sparse view {k}: float RGBA differs"
