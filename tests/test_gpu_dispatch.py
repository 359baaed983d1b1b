"""Cost-ordered block dispatch of large frames (csrc/render.cu, `prepare_dispatch`): the
render kernel records every block's duration, and the next frame of the same scene, on the
same tile grid and stream, starts its tiles longest first.  Only the order in which blocks
start may change, never a pixel: every reordered frame is compared bit for bit, in every
plane, with the scene's first frame (centre-out order, the order the full-size parity tests
check against the reference kernel) and with renders on a stream that does not own the
scene's dispatch state.  Outputs are filled with a sentinel before each frame, so a tile
that no block rendered would show."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PLANES = ("rgba8", "t", "prim", "normal")


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    torch.cuda.set_device(0)
    return torch


def _frame(torch, sc, cam, light, w, h, stream):
    n = w * h
    dev = torch.device("cuda", 0)
    with torch.cuda.stream(stream):
        out = {"rgba8": torch.full((n,), 0x5A5A5A5A, dtype=torch.int32, device=dev),
               "t": torch.full((n,), -7.0, dtype=torch.float32, device=dev),
               "prim": torch.full((n,), -7, dtype=torch.int32, device=dev),
               "normal": torch.full((3, n), -7.0, dtype=torch.float32, device=dev)}
    sc.render_torch(cam, light, w, h, planes=PLANES, stream=stream, out=out)
    stream.synchronize()
    assert sc.check(stream.cuda_stream) == 0
    return {k: v.cpu().numpy().view(np.uint32).copy() for k, v in out.items()}


def _same(a, b, name):
    for k in PLANES:
        d = a[k] != b[k]
        assert not d.any(), f"{name}: plane {k} differs at {int(d.sum())} values"


def _view(config, w=None, h=None):
    from csgrt import scenes
    text = scenes.config_scene_text(config, 0)
    v = scenes.config_views(config, 0)[0]
    return text, v.camera, v.light, w or v.w, h or v.h


@pytest.mark.parametrize("config", [2, 3, 1])
def test_reordered_frames_match_the_first_frame(csg, torch_cuda, config):
    """Four frames of one view at 3840x2160 (64,800 tiles) on one stream: the first in
    centre-out order, the others in the order the previous frame's durations give."""
    torch = torch_cuda
    text, camf, light, w, h = _view(config, 3840, 2160)
    cam = csg.Camera.from_floats(camf)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    with csg.Scene(text) as sc, csg.Scene(text) as other:
        frames = [_frame(torch, sc, cam, light, w, h, s1) for _ in range(4)]
        for i, f in enumerate(frames[1:], 2):
            _same(f, frames[0], f"config{config} frame {i}")
        _same(_frame(torch, other, cam, light, w, h, s2), frames[0], f"config{config} second scene")
        # another stream on the same scene: the plain order, the state left to s1
        _same(_frame(torch, sc, cam, light, w, h, s2), frames[0], f"config{config} non-owner stream")
        _same(_frame(torch, sc, cam, light, w, h, s1), frames[0], f"config{config} owner after non-owner")
        assert frames[0]["prim"].view(np.int32).max() >= 0


def test_camera_size_and_grid_changes(csg, torch_cuda):
    """The order a frame uses comes from the previous frame: a new camera, a new size and a
    frame stored into page-locked host memory (another warp tile, so another tile grid)
    must each render exactly what a fresh scene renders."""
    torch = torch_cuda
    text, camf, light, w, h = _view(2, 3840, 2160)
    cams = [csg.Camera.from_floats(camf)]
    for yaw in (0.05, 0.3):
        c = csg.Camera.from_floats(camf)
        c.rotate(0.02, yaw)
        cams.append(c)
    st = torch.cuda.Stream()
    with csg.Scene(text) as sc:
        for _ in range(2):
            _frame(torch, sc, cams[0], light, w, h, st)
        for i, c in enumerate(cams[1:], 1):
            got = _frame(torch, sc, c, light, w, h, st)
            with csg.Scene(text) as fresh:
                want = _frame(torch, fresh, c, light, w, h, st)
            _same(got, want, f"camera {i}")
        for (ww, hh) in ((4096, 2048), (3840, 2160)):
            a = _frame(torch, sc, cams[0], light, ww, hh, st)
            b = _frame(torch, sc, cams[0], light, ww, hh, st)
            with csg.Scene(text) as fresh:
                want = _frame(torch, fresh, cams[0], light, ww, hh, st)
            _same(a, want, f"{ww}x{hh} first")
            _same(b, want, f"{ww}x{hh} second")
        dev_rgba = _frame(torch, sc, cams[0], light, w, h, st)["rgba8"]
        host = torch.empty(w * h, dtype=torch.int32, pin_memory=True)
        for _ in range(3):
            host.fill_(0x5A5A5A5A)
            sc.render_host(cams[0], light, w, h, host.data_ptr(), stream=st.cuda_stream)
            st.synchronize()
            assert (host.numpy().view(np.uint32) == dev_rgba).all(), "host frame differs"
        assert sc.check(st.cuda_stream) == 0


def test_gate_over_many_frames(csg, torch_cuda):
    """Forty frames with every ray missing (the cheese scene, camera turned away): the cost
    summary closes the gate (plain frames for a while, then a new recording), and every frame,
    whichever form rendered it, equals the first.  Then the cheese frame itself on the same
    grid and stream, whose long blocks keep the dispatch on."""
    torch = torch_cuda
    text, camf, light, w, h = _view(2, 3840, 2160)
    turned = np.array(camf, np.float32).copy()
    turned[6:9] *= -1.0
    sky, cheese = csg.Camera.from_floats(turned), csg.Camera.from_floats(camf)
    st = torch.cuda.Stream()
    with csg.Scene(text) as sc:
        first = _frame(torch, sc, sky, light, w, h, st)
        assert (first["prim"].view(np.int32) < 0).all()
        for i in range(1, 40):
            _same(_frame(torch, sc, sky, light, w, h, st), first, f"sky frame {i}")
        ref = _frame(torch, sc, cheese, light, w, h, st)
        for i in range(1, 6):
            _same(_frame(torch, sc, cheese, light, w, h, st), ref, f"cheese frame {i}")
    with csg.Scene(text) as fresh:
        _same(_frame(torch, fresh, cheese, light, w, h, st), ref, "cheese, fresh scene")

