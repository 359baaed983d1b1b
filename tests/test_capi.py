"""The C ABI library loads and exports every function include/*.h declares (no compute
calls: this runs without a GPU), and the host-only entry points behave."""
from __future__ import annotations

import ctypes
import re

import numpy as np
import pytest

from conftest import GOLDEN, ROOT


def declared_functions() -> set[str]:
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(csg_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(csg):
    names = declared_functions()
    assert len(names) >= 20
    lib = csg.lib()
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(csg.EXPORTED) == names  # the binding lists exactly what the header declares


def test_status_strings_and_version(csg):
    assert csg.lib().csg_abi_version() == 1
    for code in range(10):
        assert csg.status_string(code)


def test_camera_matches_reference_bytes(csg):
    data = np.load(GOLDEN / "ref_camera.npz")
    eq = lambda a, b: (np.asarray(a, np.float32).view(np.uint32) == np.asarray(b, np.float32).view(np.uint32)).all()
    assert eq(csg.Camera().floats(), data["default"])
    assert eq(csg.Camera().set_fov(60).floats(), data["fov60"])
    assert eq(csg.Camera().set_position(1, 2, 3).set_rotation(0.3, -1.2).set_fov(45).floats(), data["posrot"])
    assert eq(csg.Camera().set_rotation(2.0, 7.0).floats(), data["clamped"])
    assert eq(csg.Camera().set_fov(75).rotate(0.21, -0.33).move(0.7, -0.4, 0.25).floats(), data["moved"])
    for i in range(16):
        a = data[f"lookat{i}/args"]
        c = csg.Camera().set_position(*map(float, a[:3])).set_rotation(float(a[3]), float(a[4])).set_fov(60)
        assert eq(c.floats(), data[f"lookat{i}"])
    assert eq(csg.light_dir(), data["light_default"])
    assert eq(csg.light_dir(0.4, 1.1), data["light_custom"])


def test_camera_struct_layout(csg):
    assert ctypes.sizeof(csg.csg_camera) == 60
    assert ctypes.sizeof(csg.csg_scene_info) == 48
    assert ctypes.sizeof(csg.csg_server_stats) == 88
    c = csg.Camera.from_floats(np.arange(15, dtype=np.float32))
    assert (c.floats() == np.arange(15, dtype=np.float32)).all()


def test_render_rejects_bad_arguments_without_gpu(csg):
    lib = csg.lib()
    cam = csg.Camera()
    light = (ctypes.c_float * 3)(-1, -1, -1)
    assert lib.csg_render(None, ctypes.byref(cam.c), light, 16, 16, None, None, None, None, None) == csg.CSG_E_ARG
    assert lib.csg_scene_destroy(None) == csg.CSG_E_ARG
    out = ctypes.c_void_p()
    assert lib.csg_scene_create(None, 5, ctypes.byref(out), None, 0) == csg.CSG_E_ARG


def test_server_rejects_bad_configs_without_gpu(csg):
    lib = csg.lib()
    h = ctypes.c_void_p()
    for bad in (dict(slots=17), dict(slots=-1), dict(max_batch_views=5000), dict(warp_tile_w=6), dict(planes=64),
                dict(order=3), dict(order=-1)):
        cfg = csg.csg_server_config()
        for k, v in bad.items():
            setattr(cfg, k, v)
        assert lib.csg_server_create(ctypes.byref(cfg), ctypes.byref(h)) == csg.CSG_E_ARG, bad
    assert lib.csg_server_create(None, None) == csg.CSG_E_ARG
    assert lib.csg_server_submit(None, None, None) == csg.CSG_E_ARG
    assert lib.csg_server_release(None, 1) == csg.CSG_E_ARG


def test_batch_entry_points_reject_null_without_gpu(csg):
    lib = csg.lib()
    assert lib.csg_batch_set_shape(None, 4, 0) == csg.CSG_E_ARG
    assert lib.csg_batch_set_tile(None, 8) == csg.CSG_E_ARG
    info = csg.csg_batch_class_info()
    assert lib.csg_batch_get_class(None, 0, ctypes.byref(info)) == csg.CSG_E_ARG
    assert lib.csg_batch_get_info(None, None) == csg.CSG_E_ARG
    # the structs' layout: eight-byte aligned info, ten four-byte fields per class
    assert ctypes.sizeof(csg.csg_batch_info) == 48
    assert ctypes.sizeof(csg.csg_batch_class_info) == 40


def test_host_render_rejects_null_without_gpu(csg):
    lib = csg.lib()
    cam = csg.Camera()
    light = (ctypes.c_float * 3)(-1, -1, -1)
    buf = (ctypes.c_uint32 * 4)()
    assert lib.csg_render_host(None, ctypes.byref(cam.c), light, 2, 2, ctypes.addressof(buf), None) == csg.CSG_E_ARG


def test_batch_class_setter_rejects_null_without_gpu(csg):
    assert csg.lib().csg_batch_set_class(None, 0, 8, 4, 0) == csg.CSG_E_ARG


def test_camera_and_light_match_reference_on_random_inputs(csg):
    """csg_camera_* and csg_light_dir against the reference's Camera (Camera.h:18-52,
    Camera.cpp:4-36) and DirectionalLight (DirectionalLight.h:13-18) compiled for the
    host: random positions, rotations beyond the +-89 degree clamp, fields of view, and
    chains of rotate/move calls, byte for byte."""
    from oracle import RefHost
    if not RefHost.available():
        pytest.skip("the reference's host build is not present here")
    R = RefHost()
    rng = np.random.default_rng(7)
    eq = lambda a, b: (np.asarray(a, np.float32).view(np.uint32) == np.asarray(b, np.float32).view(np.uint32)).all()
    for i in range(400):
        pos = tuple(float(np.float32(v)) for v in rng.uniform(-50, 50, 3))
        rot = tuple(float(np.float32(v)) for v in rng.uniform(-4, 4, 2))
        fov = float(np.float32(rng.uniform(1, 179)))
        c = csg.Camera().set_position(*pos).set_rotation(*rot).set_fov(fov)
        ref = R.camera(position=pos, rotation=rot, fov_deg=fov)
        assert eq(c.floats(), ref), i
        for _ in range(3):
            dp, dy = (float(np.float32(v)) for v in rng.uniform(-1, 1, 2))
            f, r, u = (float(np.float32(v)) for v in rng.uniform(-2, 2, 3))
            c.rotate(dp, dy).move(f, r, u)
            ref = R.camera_move(R.camera_rotate(ref, dp, dy), f, r, u)
            assert eq(c.floats(), ref), i
        polar, az = (float(np.float32(v)) for v in rng.uniform(-7, 7, 2))
        assert eq(csg.light_dir(polar, az), R.light_dir(polar, az)), i
