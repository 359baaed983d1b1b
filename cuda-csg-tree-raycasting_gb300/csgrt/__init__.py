"""Python bindings (ctypes) of libcsgrt, the GB300 CSG ray-casting engine.

Thin mirror of the C ABI in ``include/csgrt.h`` for tests and benchmarks.  Device
buffers are plain device pointers (``torch.Tensor.data_ptr()`` works); the library is
the only compute path -- :func:`lib` raises if ``libcsgrt.so`` has not been built, and
nothing here falls back to a CPU implementation.

Mirrors of the reference interface:

* :class:`Scene` -- ``CSGTree::Parse`` + ``Raycaster::ChangeSize``'s upload
  (CSGTree.cu:5-179, Raycaster.cu:3-21); raises :class:`CsgError` with the reference's
  parse message on bad input.
* :class:`Camera` -- the reference ``Camera`` (Camera.h / Camera.cpp), same byte layout.
* :func:`light_dir` -- ``DirectionalLight::getLightDir`` (DirectionalLight.h:13-18).
* :meth:`Scene.render` -- ``Raycaster::Raycast`` (Raycaster.cu:23-34).
"""
from __future__ import annotations

import ctypes
import math
import os
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent.parent
LIB_PATH = PKG_DIR / "_build" / "libcsgrt.so"

CSG_OK, CSG_E_PARSE, CSG_E_RANGE, CSG_E_COUNT, CSG_E_CUDA = 0, 1, 2, 3, 4
CSG_E_BUDGET, CSG_E_TIMEOUT, CSG_E_DEPTH, CSG_E_ARG, CSG_E_CAPACITY = 5, 6, 7, 8, 9

# Every function include/csgrt.h declares.
EXPORTED = [
    "csg_abi_version", "csg_status_string",
    "csg_tree_parse", "csg_scene_create", "csg_scene_destroy", "csg_scene_get_info", "csg_scene_export_reference_layout",
    "csg_camera_init", "csg_camera_set_position", "csg_camera_set_rotation", "csg_camera_set_fov",
    "csg_camera_move", "csg_camera_rotate", "csg_light_dir", "csg_light_default",
    "csg_render", "csg_render_f4", "csg_render_planes", "csg_scene_check", "csg_device_tan_half_fov",
    "csg_probe_fp32_peak",
    "csg_batch_create", "csg_batch_destroy", "csg_batch_render", "csg_batch_set_tile", "csg_batch_tune",
    "csg_batch_get_info", "csg_batch_check", "csg_render_views_noalloc",
    "csg_server_create", "csg_server_destroy", "csg_server_add_scene", "csg_server_preload", "csg_server_submit",
    "csg_server_wait", "csg_server_release", "csg_server_replay", "csg_server_stats_get", "csg_server_clock",
    "csg_image_write", "csg_scene_create_ex", "csg_tree_parse_ex", "csg_batch_set_shape", "csg_batch_get_class",
    "csg_render_host", "csg_batch_set_class", "csg_set_iteration_cap", "csg_tree_plan",
]

_vp = ctypes.c_void_p
_f = ctypes.c_float
_i32 = ctypes.c_int32


class CsgError(RuntimeError):
    def __init__(self, code: int, msg: str = ""):
        super().__init__(f"csg status {code}: {msg}")
        self.code = code
        self.msg = msg


class csg_camera(ctypes.Structure):
    _fields_ = [("x", _f), ("y", _f), ("z", _f), ("rot_x", _f), ("rot_y", _f), ("fov", _f),
                ("forward", _f * 3), ("right", _f * 3), ("up", _f * 3)]


class csg_scene_info(ctypes.Structure):
    _fields_ = [("n_nodes", _i32), ("n_prims", _i32), ("op_depth", _i32), ("stack_class", _i32),
                ("device_bytes", ctypes.c_uint64), ("rolled", _i32), ("live_words", _i32), ("live_shift", _i32),
                ("fine_words", _i32), ("short_circuit", _i32)]


class csg_planes(ctypes.Structure):
    _fields_ = [("rgba8", _vp), ("rgba32f", _vp), ("t", _vp), ("prim", _vp), ("normal", _vp)]


class csg_view(ctypes.Structure):
    _fields_ = [("scene", _vp), ("cam", csg_camera), ("light_dir", _f * 3), ("w", _i32), ("h", _i32),
                ("out", csg_planes)]


class csg_batch_info(ctypes.Structure):
    _fields_ = [("n_views", _i32), ("n_items", _i32), ("warp_tile_w", _i32), ("stack_class", _i32),
                ("rolled", _i32), ("grid", _i32), ("device_bytes", ctypes.c_uint64), ("n_classes", _i32),
                ("warps_per_block", _i32), ("local_stacks", _i32)]


class csg_batch_class_info(ctypes.Structure):
    _fields_ = [("n_views", _i32), ("stack_class", _i32), ("rolled", _i32), ("live_words", _i32),
                ("warp_tile_w", _i32), ("warps_per_block", _i32), ("local_stacks", _i32), ("grid", _i32),
                ("n_items", _i32), ("tuned_ms", _f)]


CSG_PLANE_RGBA8, CSG_PLANE_T, CSG_PLANE_PRIM, CSG_PLANE_NORMAL, CSG_PLANE_RGBA32F = 1, 2, 4, 8, 16
CSG_REQ_ALONE = 1


class csg_server_config(ctypes.Structure):
    _fields_ = [("hbm_budget", ctypes.c_uint64), ("slots", _i32), ("max_batch_views", _i32), ("warp_tile_w", _i32),
                ("planes", _i32), ("keep_results", _i32), ("order", _i32)]


class csg_request(ctypes.Structure):
    _fields_ = [("scene", _i32), ("flags", _i32), ("cam", csg_camera), ("light_dir", _f * 3), ("w", _i32),
                ("h", _i32), ("host_rgba8", _vp)]


class csg_result(ctypes.Structure):
    _fields_ = [("status", _i32), ("batch_views", _i32), ("t_arrive", ctypes.c_double),
                ("t_launch", ctypes.c_double), ("t_done", ctypes.c_double), ("planes", csg_planes)]


class csg_server_stats(ctypes.Structure):
    _fields_ = [("budget", ctypes.c_uint64), ("scene_bytes", ctypes.c_uint64), ("output_bytes", ctypes.c_uint64),
                ("peak_bytes", ctypes.c_uint64), ("requests_done", ctypes.c_int64), ("batches", ctypes.c_int64),
                ("evictions", ctypes.c_int64), ("rejected", ctypes.c_int64), ("scenes", _i32),
                ("resident_scenes", _i32), ("slots_busy", _i32), ("pending", _i32), ("capped_rays", ctypes.c_uint64)]


_LIB = None


def lib() -> ctypes.CDLL:
    """Load libcsgrt.so (built by build_lib.py).  Raises if it is missing."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = os.environ.get("CSGRT_LIB", str(LIB_PATH))
    if not os.path.exists(path):
        raise RuntimeError(f"libcsgrt.so not built ({path}); run __graft_entry__.build()")
    L = ctypes.CDLL(path)
    L.csg_abi_version.restype = ctypes.c_int
    L.csg_status_string.argtypes = [ctypes.c_int]
    L.csg_status_string.restype = ctypes.c_char_p
    L.csg_scene_create.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(_vp), ctypes.c_char_p,
                                   ctypes.c_size_t]
    L.csg_scene_destroy.argtypes = [_vp]
    L.csg_scene_create_ex.argtypes = [ctypes.c_char_p, ctypes.c_size_t, _i32, ctypes.POINTER(_vp), ctypes.c_char_p,
                                      ctypes.c_size_t]
    L.csg_tree_parse_ex.argtypes = [ctypes.c_char_p, ctypes.c_size_t, _i32, _vp, _i32, _vp, _i32,
                                    ctypes.POINTER(_i32), ctypes.POINTER(_i32), ctypes.POINTER(_i32),
                                    ctypes.c_char_p, ctypes.c_size_t]
    L.csg_tree_parse.argtypes = [ctypes.c_char_p, ctypes.c_size_t, _vp, _i32, _vp, _i32, ctypes.POINTER(_i32),
                                 ctypes.POINTER(_i32), ctypes.POINTER(_i32), ctypes.c_char_p, ctypes.c_size_t]
    L.csg_scene_get_info.argtypes = [_vp, ctypes.POINTER(csg_scene_info)]
    L.csg_scene_export_reference_layout.argtypes = [_vp, _vp, _i32, _vp, _i32, ctypes.POINTER(_i32),
                                                    ctypes.POINTER(_i32)]
    C = ctypes.POINTER(csg_camera)
    L.csg_camera_init.argtypes = [C]
    L.csg_camera_set_position.argtypes = [C, _f, _f, _f]
    L.csg_camera_set_rotation.argtypes = [C, _f, _f]
    L.csg_camera_set_fov.argtypes = [C, _f]
    L.csg_camera_move.argtypes = [C, _f, _f, _f]
    L.csg_camera_rotate.argtypes = [C, _f, _f]
    for n in ("csg_camera_init", "csg_camera_set_position", "csg_camera_set_rotation", "csg_camera_set_fov",
              "csg_camera_move", "csg_camera_rotate", "csg_light_dir", "csg_light_default"):
        getattr(L, n).restype = None
    L.csg_light_dir.argtypes = [_f, _f, ctypes.POINTER(_f)]
    L.csg_light_default.argtypes = [ctypes.POINTER(_f)]
    L.csg_render.argtypes = [_vp, C, ctypes.POINTER(_f), _i32, _i32, _vp, _vp, _vp, _vp, _vp]
    L.csg_render_f4.argtypes = [_vp, C, ctypes.POINTER(_f), _i32, _i32, _vp, _vp]
    L.csg_render_planes.argtypes = [_vp, C, ctypes.POINTER(_f), _i32, _i32, ctypes.POINTER(csg_planes), _vp]
    L.csg_render_host.argtypes = [_vp, C, ctypes.POINTER(_f), _i32, _i32, _vp, _vp]
    L.csg_set_iteration_cap.argtypes = [ctypes.c_uint32]
    L.csg_tree_plan.argtypes = [ctypes.c_char_p, ctypes.c_size_t, _i32, ctypes.POINTER(csg_scene_info),
                                ctypes.c_char_p, ctypes.c_size_t]
    L.csg_scene_check.argtypes = [_vp, _vp, ctypes.POINTER(ctypes.c_uint64)]
    L.csg_device_tan_half_fov.argtypes = [_f, ctypes.POINTER(_f)]
    L.csg_probe_fp32_peak.argtypes = [ctypes.POINTER(_f), ctypes.POINTER(_f)]
    L.csg_batch_create.argtypes = [ctypes.POINTER(csg_view), _i32, ctypes.POINTER(_vp)]
    L.csg_batch_destroy.argtypes = [_vp]
    L.csg_batch_render.argtypes = [_vp, _vp]
    L.csg_batch_set_tile.argtypes = [_vp, _i32]
    L.csg_batch_tune.argtypes = [_vp, _vp, ctypes.POINTER(_i32), ctypes.POINTER(_f)]
    L.csg_batch_get_info.argtypes = [_vp, ctypes.POINTER(csg_batch_info)]
    L.csg_batch_set_shape.argtypes = [_vp, _i32, _i32]
    L.csg_batch_get_class.argtypes = [_vp, _i32, ctypes.POINTER(csg_batch_class_info)]
    L.csg_batch_set_class.argtypes = [_vp, _i32, _i32, _i32, _i32]
    L.csg_batch_check.argtypes = [_vp, _vp, ctypes.POINTER(ctypes.c_uint64)]
    L.csg_render_views_noalloc.argtypes = [ctypes.POINTER(csg_view), _i32, _i32, _vp]
    L.csg_server_create.argtypes = [ctypes.POINTER(csg_server_config), ctypes.POINTER(_vp)]
    L.csg_server_destroy.argtypes = [_vp]
    L.csg_server_add_scene.argtypes = [_vp, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(_i32), ctypes.c_char_p,
                                       ctypes.c_size_t]
    L.csg_server_preload.argtypes = [_vp, _i32]
    L.csg_server_submit.argtypes = [_vp, ctypes.POINTER(csg_request), ctypes.POINTER(ctypes.c_int64)]
    L.csg_server_wait.argtypes = [_vp, ctypes.c_int64, ctypes.c_double, ctypes.POINTER(csg_result)]
    L.csg_server_release.argtypes = [_vp, ctypes.c_int64]
    L.csg_server_replay.argtypes = [_vp, ctypes.POINTER(csg_request), ctypes.POINTER(ctypes.c_double), _i32,
                                    ctypes.POINTER(csg_result), ctypes.POINTER(ctypes.c_int64),
                                    ctypes.POINTER(ctypes.c_double)]
    L.csg_server_stats_get.argtypes = [_vp, ctypes.POINTER(csg_server_stats)]
    L.csg_server_clock.argtypes = [_vp]
    L.csg_image_write.argtypes = [ctypes.c_char_p, _vp, _i32, _i32, _i32]
    L.csg_server_clock.restype = ctypes.c_double
    _LIB = L
    return L


def device_tan_half_fov(fov: float) -> float:
    out = _f()
    check(lib().csg_device_tan_half_fov(fov, ctypes.byref(out)))
    return out.value


def probe_fp32_peak() -> float:
    """Measured FP32 FMA rate of the current GPU in TFLOP/s."""
    tf, ms = _f(), _f()
    check(lib().csg_probe_fp32_peak(ctypes.byref(tf), ctypes.byref(ms)))
    return tf.value


def write_image(path, rgba8, w: int, h: int, fmt: str = "png"):
    """Writes an RGBA8 frame (host array of w*h uint32/int32, row 0 on top) as PNG or PPM."""
    import numpy as np
    a = np.ascontiguousarray(np.asarray(rgba8).reshape(-1).view(np.uint32))
    if a.size != w * h:
        raise ValueError("frame size does not match w*h")
    code = {"ppm": 0, "png": 1}[fmt]
    check(lib().csg_image_write(str(path).encode(), a.ctypes.data, w, h, code))


def status_string(code: int) -> str:
    return lib().csg_status_string(code).decode()


def check(code: int, msg: str = ""):
    if code != CSG_OK:
        raise CsgError(code, msg or status_string(code))


CSG_SCENE_EXACT_BOXES = 1
CSG_SCENE_FINE_MASK = 2


def parse_tree(text: str | bytes, exact_boxes: bool = False):
    """CSGTree::Parse on the host: (nodes, prims, op_depth) with nodes and prims as raw
    bytes in the reference's 44-byte CSGNode / 48-byte Primitive layouts (boxes of the
    exact-box mode with exact_boxes)."""
    data = text.encode() if isinstance(text, str) else bytes(text)
    flags = CSG_SCENE_EXACT_BOXES if exact_boxes else 0
    nn, npr, dep = _i32(), _i32(), _i32()
    err = ctypes.create_string_buffer(512)
    rc = lib().csg_tree_parse_ex(data, len(data), flags, None, 0, None, 0, ctypes.byref(nn), ctypes.byref(npr),
                                 ctypes.byref(dep), err, 512)
    if rc != CSG_OK:
        raise CsgError(rc, err.value.decode(errors="replace"))
    nodes = np.zeros(nn.value * 44, np.uint8)
    prims = np.zeros(npr.value * 48, np.uint8)
    check(lib().csg_tree_parse_ex(data, len(data), flags, nodes.ctypes.data, nn.value, prims.ctypes.data,
                                  npr.value, ctypes.byref(nn), ctypes.byref(npr), ctypes.byref(dep), err, 512))
    return nodes, prims, dep.value


def plan_tree(text: str | bytes, exact_boxes: bool = False, fine_mask: bool = False) -> dict:
    """csg_tree_plan: what a Scene built from `text` would hold (sizes, kernel variant, live
    masks), computed on the host alone."""
    data = text.encode() if isinstance(text, str) else bytes(text)
    inf = csg_scene_info()
    err = ctypes.create_string_buffer(512)
    flags = (CSG_SCENE_EXACT_BOXES if exact_boxes else 0) | (CSG_SCENE_FINE_MASK if fine_mask else 0)
    rc = lib().csg_tree_plan(data, len(data), flags, ctypes.byref(inf), err, 512)
    if rc != CSG_OK:
        raise CsgError(rc, err.value.decode(errors="replace"))
    return {k: getattr(inf, k) for k, _ in csg_scene_info._fields_}


# ------------------------------------------------------------------------------------
class Camera:
    """The reference Camera (Camera.h:3-53): position, pitch/yaw, fov, cached basis."""

    def __init__(self):
        self.c = csg_camera()
        lib().csg_camera_init(ctypes.byref(self.c))

    @classmethod
    def from_floats(cls, v) -> "Camera":
        cam = cls()
        arr = np.ascontiguousarray(v, np.float32)
        ctypes.memmove(ctypes.byref(cam.c), arr.ctypes.data, 60)
        return cam

    def floats(self) -> np.ndarray:
        return np.frombuffer(bytes(self.c), np.float32).copy()

    def set_position(self, x, y, z):
        lib().csg_camera_set_position(ctypes.byref(self.c), x, y, z)
        return self

    def set_rotation(self, pitch, yaw):
        lib().csg_camera_set_rotation(ctypes.byref(self.c), pitch, yaw)
        return self

    def set_fov(self, degrees):
        lib().csg_camera_set_fov(ctypes.byref(self.c), degrees)
        return self

    def move(self, fwd, right, up):
        lib().csg_camera_move(ctypes.byref(self.c), fwd, right, up)
        return self

    def rotate(self, dpitch, dyaw):
        lib().csg_camera_rotate(ctypes.byref(self.c), dpitch, dyaw)
        return self

    @classmethod
    def look_at_origin(cls, direction, distance=4.0, fov_deg=60.0) -> "Camera":
        """Camera at distance * unit(direction), looking at the origin: pitch = asin(-p.y),
        yaw = atan2(p.x, p.z) (forward = (-sin yaw cos pitch, sin pitch, -cos yaw cos pitch))."""
        d = np.asarray(direction, np.float64)
        d = d / np.linalg.norm(d)
        cam = cls()
        p = distance * d
        cam.set_position(float(np.float32(p[0])), float(np.float32(p[1])), float(np.float32(p[2])))
        cam.set_rotation(float(np.float32(math.asin(-d[1]))), float(np.float32(math.atan2(d[0], d[2]))))
        cam.set_fov(fov_deg)
        return cam


def light_dir(polar=None, azimuth=None) -> np.ndarray:
    out = (_f * 3)()
    if polar is None:
        lib().csg_light_default(out)
    else:
        lib().csg_light_dir(polar, azimuth, out)
    return np.array(list(out), np.float32)


# ------------------------------------------------------------------------------------
class Scene:
    """A parsed, device-resident CSG scene (opaque handle)."""

    def __init__(self, text: str | bytes, exact_boxes: bool = False, fine_mask: bool = False):
        data = text.encode() if isinstance(text, str) else bytes(text)
        h = _vp()
        err = ctypes.create_string_buffer(512)
        flags = (CSG_SCENE_EXACT_BOXES if exact_boxes else 0) | (CSG_SCENE_FINE_MASK if fine_mask else 0)
        rc = lib().csg_scene_create_ex(data, len(data), flags, ctypes.byref(h), err, 512)
        if rc != CSG_OK:
            raise CsgError(rc, err.value.decode(errors="replace"))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().csg_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def info(self) -> dict:
        inf = csg_scene_info()
        check(lib().csg_scene_get_info(self.h, ctypes.byref(inf)))
        return {k: getattr(inf, k) for k, _ in csg_scene_info._fields_}

    def export_reference_layout(self):
        """(nodes, prims) as raw bytes in the reference's CSGNode / Primitive layouts."""
        nn, npr = _i32(), _i32()
        check(lib().csg_scene_export_reference_layout(self.h, None, 0, None, 0, ctypes.byref(nn),
                                                      ctypes.byref(npr)))
        nodes = np.zeros(nn.value * 44, np.uint8)
        prims = np.zeros(npr.value * 48, np.uint8)
        check(lib().csg_scene_export_reference_layout(self.h, nodes.ctypes.data, nn.value, prims.ctypes.data,
                                                      npr.value, ctypes.byref(nn), ctypes.byref(npr)))
        return nodes, prims

    def render_ptrs(self, cam: Camera, light, w: int, h: int, rgba8=0, rgba32f=0, t=0, prim=0, normal=0,
                    stream=0):
        light = (_f * 3)(*[float(v) for v in light])
        pl = csg_planes(rgba8 or None, rgba32f or None, t or None, prim or None, normal or None)
        check(lib().csg_render_planes(self.h, ctypes.byref(cam.c), light, w, h, ctypes.byref(pl),
                                      stream or None))

    def render_host(self, cam: Camera, light, w: int, h: int, host_rgba8: int, stream=0):
        """RGBA8 frame into host memory at address `host_rgba8` (csg_render_host): written by
        the kernel itself when page-locked, staged through the device otherwise."""
        light = (_f * 3)(*[float(v) for v in light])
        check(lib().csg_render_host(self.h, ctypes.byref(cam.c), light, w, h, host_rgba8, stream or None))

    def render_torch(self, cam: Camera, light, w: int, h: int, planes=("rgba8",), stream=None, out=None):
        """Render into torch CUDA tensors; returns a dict of the requested planes."""
        import torch
        dev = torch.device("cuda", torch.cuda.current_device())
        n = w * h
        out = dict(out or {})
        spec = {"rgba8": (n,), "rgba32f": (n, 4), "t": (n,), "prim": (n,), "normal": (3, n)}
        dts = {"rgba8": torch.int32, "rgba32f": torch.float32, "t": torch.float32, "prim": torch.int32,
               "normal": torch.float32}
        for k in planes:
            if k not in out:
                out[k] = torch.empty(spec[k], dtype=dts[k], device=dev)
        st = stream if stream is not None else torch.cuda.current_stream()
        self.render_ptrs(cam, light, w, h, **{k: out[k].data_ptr() for k in planes}, stream=st.cuda_stream)
        return out

    def check(self, stream=0) -> int:
        n = ctypes.c_uint64()
        rc = lib().csg_scene_check(self.h, stream or None, ctypes.byref(n))
        if rc not in (CSG_OK, CSG_E_TIMEOUT):
            check(rc)
        return int(n.value)


# ------------------------------------------------------------------------------------
def view_array(views):
    """A csg_view array for (scene, camera, light, w, h, planes) tuples (planes: plane name ->
    device pointer, as for Batch)."""
    arr = (csg_view * len(views))()
    for i, (scene, cam, light, w, h, planes) in enumerate(views):
        v = arr[i]
        v.scene = scene.h
        ctypes.memmove(ctypes.byref(v.cam), ctypes.byref(cam.c), 60)
        for k in range(3):
            v.light_dir[k] = float(light[k])
        v.w, v.h = int(w), int(h)
        v.out = csg_planes(planes.get("rgba8") or None, planes.get("rgba32f") or None, planes.get("t") or None,
                           planes.get("prim") or None, planes.get("normal") or None)
    return arr


def render_views_noalloc(views, warp_tile_w=8, stream=None):
    """csg_render_views_noalloc: the views rendered by one view-table launch whose scratch is
    the library's fixed device array (asynchronous on `stream`)."""
    check(lib().csg_render_views_noalloc(view_array(views), len(views), int(warp_tile_w), stream))


class Batch:
    """Many views of many scenes rendered by one persistent, graph-replayed launch.

    `views` is a list of (scene, camera, light, w, h, planes) where planes maps plane names
    ("rgba8", "rgba32f", "t", "prim", "normal") to device pointers.  The scenes and the
    planes must outlive the batch."""

    def __init__(self, views):
        arr = view_array(views)
        h = _vp()
        check(lib().csg_batch_create(arr, len(views), ctypes.byref(h)))
        self.h = h
        self._keep = views

    def close(self):
        if getattr(self, "h", None):
            lib().csg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def render(self, stream=0):
        check(lib().csg_batch_render(self.h, stream or None))

    def set_tile(self, warp_tile_w: int):
        check(lib().csg_batch_set_tile(self.h, warp_tile_w))

    def set_shape(self, warps_per_block: int = 4, local_stacks: bool = False):
        """Block shape of every class's launch: (4, False), (4, True), (2, False) or (8, False)."""
        check(lib().csg_batch_set_shape(self.h, warps_per_block, int(bool(local_stacks))))

    def set_class(self, k: int, warp_tile_w: int, warps_per_block: int = 4, local_stacks: bool = False):
        """Class k's warp tile width and block shape."""
        check(lib().csg_batch_set_class(self.h, k, warp_tile_w, warps_per_block, int(bool(local_stacks))))

    def copy_config(self, other: "Batch"):
        """Gives every class the configuration of the same class of `other` (a batch over the
        same scenes, e.g. one that was tuned)."""
        mine, theirs = self.classes(), other.classes()
        if [(c["stack_class"], c["rolled"], c["live_words"], c["n_views"]) for c in mine] != \
                [(c["stack_class"], c["rolled"], c["live_words"], c["n_views"]) for c in theirs]:
            raise ValueError("batches have different tree-size classes")
        for k, c in enumerate(theirs):
            self.set_class(k, c["warp_tile_w"], c["warps_per_block"], bool(c["local_stacks"]))

    def classes(self) -> list:
        """Per tree-size class (heaviest first): its kernel variant and configuration."""
        out = []
        for k in range(self.info()["n_classes"]):
            c = csg_batch_class_info()
            check(lib().csg_batch_get_class(self.h, k, ctypes.byref(c)))
            out.append({n: getattr(c, n) for n, _ in csg_batch_class_info._fields_})
        return out

    def tune(self, stream=0):
        tw, ms = _i32(), _f()
        check(lib().csg_batch_tune(self.h, stream or None, ctypes.byref(tw), ctypes.byref(ms)))
        return tw.value, ms.value

    def info(self) -> dict:
        inf = csg_batch_info()
        check(lib().csg_batch_get_info(self.h, ctypes.byref(inf)))
        return {k: getattr(inf, k) for k, _ in csg_batch_info._fields_}

    def check(self, stream=0) -> int:
        n = ctypes.c_uint64()
        rc = lib().csg_batch_check(self.h, stream or None, ctypes.byref(n))
        if rc not in (CSG_OK, CSG_E_TIMEOUT):
            check(rc)
        return int(n.value)


# ------------------------------------------------------------------------------------
class Server:
    """Render server with continuous batching (csg_server_* of the C ABI).

    Scenes are added once (parsed now, resident on first use, evicted least recently used
    under `hbm_budget`); requests are submitted with `submit` (returns a ticket) and
    collected with `wait`; `replay` runs an open-loop arrival trace inside the library."""

    def __init__(self, hbm_budget=0, slots=0, max_batch_views=0, warp_tile_w=0, planes=0, keep_results=False,
                 longest_first=False, order=None):
        """order: 0 arrival order, 1 each batch's views longest first, 2 size-aware
        (earliest deadline first, priority streams); default 1 if longest_first else 0."""
        if order is None:
            order = 1 if longest_first else 0
        cfg = csg_server_config(int(hbm_budget), int(slots), int(max_batch_views), int(warp_tile_w), int(planes),
                                1 if keep_results else 0, int(order))
        h = _vp()
        check(lib().csg_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().csg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def add_scene(self, text) -> int:
        data = text.encode() if isinstance(text, str) else bytes(text)
        sid = _i32()
        err = ctypes.create_string_buffer(512)
        rc = lib().csg_server_add_scene(self.h, data, len(data), ctypes.byref(sid), err, len(err))
        check(rc, err.value.decode(errors="replace") if rc != CSG_OK else "")
        return sid.value

    def preload(self, sid: int):
        check(lib().csg_server_preload(self.h, sid))

    @staticmethod
    def request(scene: int, cam: "Camera", light, w: int, h: int, alone=False, host_rgba8=0) -> csg_request:
        r = csg_request()
        r.scene = scene
        r.flags = CSG_REQ_ALONE if alone else 0
        ctypes.memmove(ctypes.byref(r.cam), ctypes.byref(cam.c), 60)
        for k in range(3):
            r.light_dir[k] = float(light[k])
        r.w, r.h = int(w), int(h)
        r.host_rgba8 = host_rgba8 or None
        return r

    def submit(self, req: csg_request) -> int:
        t = ctypes.c_int64()
        check(lib().csg_server_submit(self.h, ctypes.byref(req), ctypes.byref(t)))
        return t.value

    def wait(self, ticket: int, timeout_s: float = -1.0) -> csg_result:
        r = csg_result()
        check(lib().csg_server_wait(self.h, ticket, timeout_s, ctypes.byref(r)))
        return r

    def release(self, ticket: int):
        check(lib().csg_server_release(self.h, ticket))

    def replay(self, reqs, arrival_s, keep=False):
        """Returns (results array, tickets or None, wall seconds)."""
        n = len(reqs)
        arr = (csg_request * n)(*reqs)
        at = (ctypes.c_double * n)(*[float(a) for a in arrival_s])
        res = (csg_result * n)()
        tk = (ctypes.c_int64 * n)() if keep else None
        wall = ctypes.c_double()
        check(lib().csg_server_replay(self.h, arr, at, n, res, tk, ctypes.byref(wall)))
        return res, (list(tk) if keep else None), wall.value

    def stats(self) -> dict:
        st = csg_server_stats()
        check(lib().csg_server_stats_get(self.h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in csg_server_stats._fields_}

    def clock(self) -> float:
        return lib().csg_server_clock(self.h)
