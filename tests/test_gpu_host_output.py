"""csg_render_host: the RGBA8 frame rendered straight into host memory is byte for byte the
frame csg_render_planes writes into device memory -- into page-locked memory (written by
the kernel itself) and into pageable memory (staged through a device frame) -- and a
device destination is refused."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cases(csg):
    from csgrt import scenes
    yield "config1", scenes.config_scene_text(1, 0), scenes.config_views(1, 0)[0], (1280, 720)
    yield "config3-seed2", scenes.config_scene_text(3, 2), scenes.config_views(3, 2)[0], (333, 177)
    yield "cheese-64", scenes.write_text(scenes.cheese_tree(3, 64)), scenes.config_views(2, 3)[0], (17, 13)


def test_host_frames_equal_device_frames(csg):
    import torch
    torch.cuda.set_device(0)
    st = torch.cuda.current_stream()
    for name, text, view, (w, h) in _cases(csg):
        with csg.Scene(text) as sc:
            cam = csg.Camera.from_floats(view.camera)
            dev = torch.zeros(w * h, dtype=torch.int32, device="cuda")
            sc.render_ptrs(cam, view.light, w, h, rgba8=dev.data_ptr(), stream=st.cuda_stream)
            pinned = torch.zeros(w * h, dtype=torch.int32, pin_memory=True)
            sc.render_host(cam, view.light, w, h, pinned.data_ptr(), stream=st.cuda_stream)
            pageable = np.zeros(w * h, dtype=np.int32)
            sc.render_host(cam, view.light, w, h, pageable.ctypes.data, stream=st.cuda_stream)
            torch.cuda.synchronize()
            assert sc.check(st.cuda_stream) == 0
            ref = dev.cpu().numpy()
            assert np.array_equal(pinned.numpy(), ref), name
            assert np.array_equal(pageable, ref), name
            assert (ref != 0).any()


def test_host_render_refuses_device_destination(csg):
    import torch
    torch.cuda.set_device(0)
    with csg.Scene("Sphere 0 0 0 FF0000 1") as sc:
        dev = torch.zeros(16 * 16, dtype=torch.int32, device="cuda")
        light = (ctypes.c_float * 3)(-1, -1, -1)
        cam = csg.Camera()
        rc = csg.lib().csg_render_host(sc.h, ctypes.byref(cam.c), light, 16, 16, dev.data_ptr(), None)
        assert rc == csg.CSG_E_ARG
