"""CPU oracle for the CSG ray-casting path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
may import this package, and only to check results against it (or, for the baseline,
as the timed CPU restatement of the reference).  The product never imports it.

* :class:`Oracle` wraps ``oracle/_build/liboracle.so`` (``csg_oracle.c``), a plain-C
  restatement of the reference's parser, camera, traversal, intersections and shading.
* :class:`RefHost` wraps ``oracle/_ref/libref_host.so``, the reference's own code
  compiled for the host (only where the reference sources are present).
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

NODE_DTYPE = np.dtype([("type", "<i4"), ("prim", "<i4"), ("left", "<i4"), ("right", "<i4"),
                       ("parent", "<i4"), ("box", "<f4", (6,))])
PRIM_DTYPE = np.dtype([("id", "<i4"), ("pos", "<f4", (3,)), ("rgb", "<f4", (3,)),
                       ("p", "<f4", (5,))])
COUNTS_DTYPE = np.dtype([("iters", "<u4"), ("aabb", "<u4"), ("sphere", "<u4"), ("cyl", "<u4"),
                         ("cube", "<u4"), ("max_actions", "<u4"), ("flops_trace", "<u4"),
                         ("flops", "<u4")])
assert NODE_DTYPE.itemsize == 44 and PRIM_DTYPE.itemsize == 48

_vp = ctypes.c_void_p
_f = ctypes.c_float
_i = ctypes.c_int


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_vp)


class ParseError(Exception):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code
        self.msg = msg


class Oracle:
    """ctypes wrapper of the C oracle."""

    def __init__(self, lib_path: str | None = None):
        path = lib_path or str(HERE / "_build" / "liboracle.so")
        if not os.path.exists(path):
            from . import build_oracle
            build_oracle.build()
        self.lib = L = ctypes.CDLL(path)
        L.orc_parse.argtypes = [ctypes.c_char_p, ctypes.c_size_t, _vp, _i, _vp, _i,
                                ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.c_char_p, ctypes.c_size_t]
        L.orc_parse.restype = _i
        for name in ("orc_render_ieee", "orc_render_fma", "orc_render_f64"):
            fn = getattr(L, name)
            fn.argtypes = [_vp, _i, _vp, _i, _vp, _f, _vp, _i, _i, _i, _i, _i,
                           _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]
            fn.restype = _i
        for name in ("orc_render_list_ieee", "orc_render_list_fma", "orc_render_list_f64"):
            fn = getattr(L, name)
            fn.argtypes = [_vp, _i, _vp, _i, _vp, _f, _vp, _i, _i, _vp, ctypes.c_int64, _i,
                           _vp, _vp, _vp, _vp, _vp, _vp]
            fn.restype = _i
        L.orc_tan_half_fov.argtypes = [_f]
        L.orc_set_short_circuit.argtypes = [_i]
        L.orc_set_short_circuit.restype = None
        L.orc_set_live_pruning.argtypes = [_i]
        L.orc_set_live_pruning.restype = None
        L.orc_set_live_region.argtypes = [_i]
        L.orc_set_live_region.restype = None
        L.orc_set_union_shortcut.argtypes = [_i]
        L.orc_set_union_shortcut.restype = None
        L.orc_set_leaf_shortcut.argtypes = [_i]
        L.orc_set_leaf_shortcut.restype = None
        L.orc_boxes_exact.argtypes = [_vp, _i, _vp]
        L.orc_boxes_exact.restype = None
        L.orc_tan_half_fov.restype = _f
        for name, args in (("orc_camera_default", [_vp]),
                           ("orc_camera_set_position", [_vp, _f, _f, _f]),
                           ("orc_camera_set_rotation", [_vp, _f, _f]),
                           ("orc_camera_set_fov", [_vp, _f]),
                           ("orc_camera_move", [_vp, _f, _f, _f]),
                           ("orc_camera_rotate", [_vp, _f, _f]),
                           ("orc_light_dir", [_f, _f, _vp]),
                           ("orc_light_default", [_vp])):
            getattr(L, name).argtypes = args
            getattr(L, name).restype = None

    # -- scene -------------------------------------------------------------------------
    def parse(self, text: str | bytes, max_nodes: int | None = None, exact_boxes: bool = False):
        data = text.encode() if isinstance(text, str) else text
        ntok = max(1, len(data.split()))
        max_nodes = max_nodes or ntok + 1
        nodes = np.zeros(max_nodes, NODE_DTYPE)
        prims = np.zeros(max_nodes, PRIM_DTYPE)
        nn, npr = _i(), _i()
        err = ctypes.create_string_buffer(512)
        rc = self.lib.orc_parse(data, len(data), _ptr(nodes), max_nodes, _ptr(prims), max_nodes,
                                ctypes.byref(nn), ctypes.byref(npr), err, 512)
        if rc != 0:
            raise ParseError(rc, err.value.decode(errors="replace"))
        nodes, prims = nodes[: nn.value].copy(), prims[: npr.value].copy()
        if exact_boxes:
            self.lib.orc_boxes_exact(_ptr(nodes), len(nodes), _ptr(prims))
        return nodes, prims

    # -- camera / light ----------------------------------------------------------------
    def camera(self, position=None, rotation=None, fov_deg=None) -> np.ndarray:
        cam = np.zeros(15, np.float32)
        self.lib.orc_camera_default(_ptr(cam))
        if position is not None:
            self.lib.orc_camera_set_position(_ptr(cam), *map(float, position))
        if rotation is not None:
            self.lib.orc_camera_set_rotation(_ptr(cam), float(rotation[0]), float(rotation[1]))
        if fov_deg is not None:
            self.lib.orc_camera_set_fov(_ptr(cam), float(fov_deg))
        return cam

    def camera_move(self, cam, f, r, u):
        cam = np.array(cam, np.float32)
        self.lib.orc_camera_move(_ptr(cam), f, r, u)
        return cam

    def camera_rotate(self, cam, dp, dy):
        cam = np.array(cam, np.float32)
        self.lib.orc_camera_rotate(_ptr(cam), dp, dy)
        return cam

    def light_dir(self, polar=None, azimuth=None) -> np.ndarray:
        out = np.zeros(3, np.float32)
        if polar is None:
            self.lib.orc_light_default(_ptr(out))
        else:
            self.lib.orc_light_dir(polar, azimuth, _ptr(out))
        return out

    def set_short_circuit(self, on: bool):
        """The engine's operator short-circuit in the traversal (off: the reference's own)."""
        self.lib.orc_set_short_circuit(1 if on else 0)

    def set_live_pruning(self, mode: int):
        """The engine's live-leaf pruning in the traversal: 0 off (the reference's own),
        1 one restore record per ray, 2 the rule without its loop restore, 3 the rule on
        trees of any depth (2 and 3 are unsound), 4 one restore record per region of
        `set_live_region` groups, 5 and 6 modes 1 and 4 restoring only groups that were
        live at tmin = 0."""
        self.lib.orc_set_live_pruning(int(mode))

    def set_union_shortcut(self, max_leaves: int):
        """With live-leaf pruning: an all-Union operator subtree of at most max_leaves
        leaves with one live leaf is evaluated as that leaf (0: off)."""
        self.lib.orc_set_union_shortcut(int(max_leaves))

    def set_leaf_shortcut(self, max_leaves: int):
        """With live-leaf pruning: any operator subtree of at most max_leaves leaves with
        one live leaf evaluates to that leaf's result when the path down to it passes only
        Unions and Differences entered on their left, else to a Miss (0: off)."""
        self.lib.orc_set_leaf_shortcut(int(max_leaves))

    def set_live_region(self, groups: int):
        """Groups per restore record of pruning modes 4 and 6 (default 128: four mask words)."""
        self.lib.orc_set_live_region(int(groups))

    def tan_half_fov(self, fov: float) -> float:
        return float(np.float32(self.lib.orc_tan_half_fov(fov)))

    # -- render ------------------------------------------------------------------------
    def render(self, nodes, prims, cam, light, w, h, mode="ieee", tan_half_fov=None,
               rows=None, nthreads=0, want=("hit", "t", "prim", "normal", "pos", "rgba", "rgba8"),
               counts=False):
        cam = np.ascontiguousarray(cam, np.float32)
        light = np.ascontiguousarray(light, np.float32)
        thf = self.tan_half_fov(float(cam[5])) if tan_half_fov is None else float(tan_half_fov)
        n = w * h
        out = {}
        shapes = {"hit": ((n,), np.uint8), "t": ((n,), np.float32), "prim": ((n,), np.int32),
                  "normal": ((n, 3), np.float32), "pos": ((n, 3), np.float32),
                  "rgba": ((n, 4), np.float32), "rgba8": ((n,), np.uint32)}
        for k in want:
            shp, dt = shapes[k]
            out[k] = np.zeros(shp, dt)
        if counts:
            out["counts"] = np.zeros(n, COUNTS_DTYPE)
        y0, y1 = rows if rows is not None else (0, h)
        fn = {"ieee": self.lib.orc_render_ieee, "fma": self.lib.orc_render_fma, "f64": self.lib.orc_render_f64}[mode]
        capped = fn(_ptr(nodes), len(nodes), _ptr(prims), len(prims), _ptr(cam), thf, _ptr(light),
                    w, h, y0, y1, nthreads,
                    _ptr(out.get("hit")), _ptr(out.get("t")), _ptr(out.get("prim")),
                    _ptr(out.get("normal")), _ptr(out.get("pos")), _ptr(out.get("rgba")),
                    _ptr(out.get("rgba8")), _ptr(out.get("counts")))
        out["capped"] = capped
        return out

    def render_list(self, nodes, prims, cam, light, w, h, pix, mode="ieee", nthreads=0, tan_half_fov=None,
                    want=("rgba8", "t", "prim"), counts=False):
        """Render the listed pixel indices (y*w + x) of a w x h frame."""
        cam = np.ascontiguousarray(cam, np.float32)
        light = np.ascontiguousarray(light, np.float32)
        thf = self.tan_half_fov(float(cam[5])) if tan_half_fov is None else float(tan_half_fov)
        pix = np.ascontiguousarray(pix, np.int64)
        n = len(pix)
        shapes = {"hit": ((n,), np.uint8), "t": ((n,), np.float32), "prim": ((n,), np.int32),
                  "normal": ((n, 3), np.float32), "rgba8": ((n,), np.uint32)}
        out = {k: np.zeros(*shapes[k]) for k in want}
        if counts:
            out["counts"] = np.zeros(n, COUNTS_DTYPE)
        fn = {"ieee": self.lib.orc_render_list_ieee, "fma": self.lib.orc_render_list_fma,
              "f64": self.lib.orc_render_list_f64}[mode]
        out["capped"] = fn(_ptr(nodes), len(nodes), _ptr(prims), len(prims), _ptr(cam), thf, _ptr(light), w, h,
                           _ptr(pix), n, nthreads, _ptr(out.get("hit")), _ptr(out.get("t")),
                           _ptr(out.get("prim")), _ptr(out.get("normal")), _ptr(out.get("rgba8")),
                           _ptr(out.get("counts")))
        return out


class RefHost:
    """ctypes wrapper of the reference's own code compiled for the host."""

    PATH = HERE / "_ref" / "libref_host.so"

    @classmethod
    def available(cls) -> bool:
        return cls.PATH.exists()

    def __init__(self):
        self.lib = L = ctypes.CDLL(str(self.PATH))
        L.ref_parse.argtypes = [ctypes.c_char_p, ctypes.c_size_t, _vp, _i, _vp, _i,
                                ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.c_char_p, ctypes.c_size_t]
        L.ref_parse.restype = _i
        L.ref_camera.argtypes = [_i, _f, _f, _f, _i, _f, _f, _i, _f, _vp]
        L.ref_camera_move.argtypes = [_vp, _f, _f, _f]
        L.ref_camera_rotate.argtypes = [_vp, _f, _f]
        L.ref_light_dir.argtypes = [_i, _f, _f, _vp]
        L.ref_render.argtypes = [_vp, _i, _vp, _i, _vp, _vp, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i]

    def parse(self, text: str | bytes):
        data = text.encode() if isinstance(text, str) else text
        cap = max(1, len(data.split())) + 1
        nodes = np.zeros(cap, NODE_DTYPE)
        prims = np.zeros(cap, PRIM_DTYPE)
        nn, npr = _i(), _i()
        err = ctypes.create_string_buffer(512)
        rc = self.lib.ref_parse(data, len(data), _ptr(nodes), cap, _ptr(prims), cap,
                                ctypes.byref(nn), ctypes.byref(npr), err, 512)
        if rc != 0:
            raise ParseError(rc, err.value.decode(errors="replace"))
        return nodes[: nn.value].copy(), prims[: npr.value].copy()

    def camera(self, position=None, rotation=None, fov_deg=None) -> np.ndarray:
        cam = np.zeros(15, np.float32)
        p = position or (0, 0, 0)
        r = rotation or (0, 0)
        self.lib.ref_camera(int(position is not None), *map(float, p), int(rotation is not None),
                            float(r[0]), float(r[1]), int(fov_deg is not None),
                            float(fov_deg or 0), _ptr(cam))
        return cam

    def camera_move(self, cam, f, r, u):
        cam = np.array(cam, np.float32)
        self.lib.ref_camera_move(_ptr(cam), f, r, u)
        return cam

    def camera_rotate(self, cam, dp, dy):
        cam = np.array(cam, np.float32)
        self.lib.ref_camera_rotate(_ptr(cam), dp, dy)
        return cam

    def light_dir(self, polar=None, azimuth=None) -> np.ndarray:
        out = np.zeros(3, np.float32)
        self.lib.ref_light_dir(int(polar is not None), float(polar or 0), float(azimuth or 0), _ptr(out))
        return out

    def render(self, nodes, prims, cam, light, w, h, nthreads=0):
        n = w * h
        out = {"hit": np.zeros(n, np.uint8), "t": np.zeros(n, np.float32),
               "pos": np.zeros((n, 3), np.float32), "normal": np.zeros((n, 3), np.float32),
               "prim": np.zeros(n, np.int32), "rgba": np.zeros((n, 4), np.float32)}
        cam = np.ascontiguousarray(cam, np.float32)
        light = np.ascontiguousarray(light, np.float32)
        self.lib.ref_render(_ptr(nodes), len(nodes), _ptr(prims), len(prims), _ptr(cam), _ptr(light),
                            w, h, _ptr(out["hit"]), _ptr(out["t"]), _ptr(out["pos"]),
                            _ptr(out["normal"]), _ptr(out["prim"]), _ptr(out["rgba"]), nthreads)
        return out


RAYHIT_DTYPE = np.dtype([("hit", "u1"), ("pad", "u1", (3,)), ("t", "<f4"), ("pos", "<f4", (3,)),
                         ("normal", "<f4", (3,)), ("prim", "<i4")])
assert RAYHIT_DTYPE.itemsize == 36


class RefCuda:
    """The reference's own CUDA kernels (cubin built by build_ref.py), launched through
    oracle/ref_cuda_runner.c on GPU 0 exactly as Raycaster::Raycast launches them."""

    CUBIN = HERE / "_ref" / "ref_kernels.cubin"
    LIB = HERE / "_build" / "librefcu.so"

    @classmethod
    def available(cls) -> bool:
        return cls.CUBIN.exists()

    def __init__(self):
        if not self.LIB.exists():
            from . import build_oracle
            build_oracle.build_refcu()
        self.lib = L = ctypes.CDLL(str(self.LIB))
        L.refcu_error.restype = ctypes.c_char_p
        L.refcu_init.argtypes = [ctypes.c_char_p]
        L.refcu_render.argtypes = [_vp, _i, _vp, _i, _vp, _vp, _i, _i, _vp, _vp, _i,
                                   ctypes.POINTER(_f), ctypes.POINTER(_f), ctypes.POINTER(_f)]
        rc = L.refcu_init(str(self.CUBIN).encode())
        if rc != 0:
            raise RuntimeError(f"reference cubin load failed: {L.refcu_error().decode()}")

    def render(self, nodes44: np.ndarray, prims48: np.ndarray, cam, light, w, h, reps=0, want_hits=True,
               want_rgba=True):
        """nodes44/prims48: raw bytes in the reference layouts.  Returns planes like
        RefHost.render plus timings (ms) when reps > 0."""
        n = w * h
        hits = np.zeros(n, RAYHIT_DTYPE) if want_hits else None
        rgba = np.zeros((n, 4), np.float32) if want_rgba else None
        cam = np.ascontiguousarray(cam, np.float32)
        light = np.ascontiguousarray(light, np.float32)
        a, b, f = _f(), _f(), _f()
        nodes44 = np.ascontiguousarray(nodes44)
        prims48 = np.ascontiguousarray(prims48)
        rc = self.lib.refcu_render(_ptr(nodes44), nodes44.nbytes // 44, _ptr(prims48), prims48.nbytes // 48,
                                   _ptr(cam), _ptr(light), w, h, _ptr(hits), _ptr(rgba), reps,
                                   ctypes.byref(a), ctypes.byref(b), ctypes.byref(f))
        if rc != 0:
            raise RuntimeError(f"reference kernel failed: {self.lib.refcu_error().decode()}")
        out = {"ms_ray": a.value, "ms_light": b.value, "ms_frame": f.value}
        if hits is not None:
            m = hits["hit"] != 0
            out["hit"] = m.astype(np.uint8)
            out["t"] = hits["t"].copy()
            out["prim"] = np.where(m, hits["prim"], -1).astype(np.int32)
            out["normal"] = np.where(m[:, None], hits["normal"], 0).astype(np.float32)
            out["pos"] = np.where(m[:, None], hits["pos"], 0).astype(np.float32)
        if rgba is not None:
            out["rgba"] = rgba
        return out


def quantize_rgba8(rgba: np.ndarray) -> np.ndarray:
    """q = lrintf(clamp(c, 0, 1) * 255) per channel, packed R | G<<8 | B<<16 | A<<24."""
    c = np.clip(rgba.astype(np.float32), 0, 1) * np.float32(255)
    q = np.rint(c).astype(np.uint32)
    return q[:, 0] | (q[:, 1] << 8) | (q[:, 2] << 16) | (q[:, 3] << 24)
