"""Generates the committed golden fixtures under tests/golden/ from the reference itself.

    python tests/golden/make_golden.py scenes   # copy the reference's Test/*.txt scene files
    python tests/golden/make_golden.py host     # reference code compiled for the host
    python tests/golden/make_golden.py gpu OUT  # reference CUDA kernel (needs a GPU + cubin)

* ``scenes/*.txt`` -- the reference's own test scenes (Test/*.txt), inputs only.
* ``ref_parse.npz`` -- CSGTree::Parse output (44-byte nodes, 48-byte primitives) for every
  scene, from oracle/_ref/libref_host.so.
* ``ref_errors.json`` -- malformed scene texts and the reference parser's exception text.
* ``ref_camera.npz`` -- Camera / DirectionalLight bytes for a list of constructions.
* ``ref_host.npz`` -- per-pixel render planes from the reference's RaycastKernel +
  LightningKernel compiled for the host (pins the oracle's "ieee" mode).
* ``ref_gpu.npz`` -- the same planes from the reference's kernels compiled by nvcc for
  sm_103a and run on a GB300 (pins the oracle's "fma" mode and the engine), with the
  device's tan(fov/2) for each case.

The first four need the reference sources (this container only); ``gpu`` runs where the
reference cubin was built and shipped.
"""
from __future__ import annotations

import json
import math
import os
import shutil
import sys
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent
ROOT = GOLDEN.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "cuda-csg-tree-raycasting_gb300"))

# The reference checkout: CSG_REFERENCE_ROOT, as oracle/build_ref.py reads it.
REF_ROOT = Path(os.environ.get("CSG_REFERENCE_ROOT", "/root/reference"))
REF_TEST_DIR = REF_ROOT / "Test"
FIX_W, FIX_H = 64, 48

# Malformed inputs covering every error path of CSGTree::Parse (CSGTree.cu:24, 68, 91,
# 104-108, 126, 140, 147) and of std::stof / stod / stoi.
ERROR_CASES = [
    "",
    "   \n\t ",
    "Union",
    "Union Sphere 0 0 0 FF0000 1",
    "Sphere 0 0 0 FF0000 1 Sphere 1 0 0 00FF00 1",
    "Spere 0 0 0 FF0000 1",
    "Union Sphere 0 0 0 FF000 1 Sphere 1 0 0 00FF00 1",
    "Union Sphere 0 0 0 GG0000 1 Sphere 1 0 0 00FF00 1",
    "Union Sphere 0 0 0 -F0000 1 Sphere 1 0 0 00FF00 1",
    "Union Sphere a 0 0 FF0000 1 Sphere 1 0 0 00FF00 1",
    "Union Sphere 0 0 0 FF0000 1e50 Sphere 1 0 0 00FF00 1",
    "Union Cylinder 0 0 0 FF0000 1 2 361 0 0 Sphere 1 0 0 00FF00 1",
    "Union Cylinder 0 0 0 FF0000 1 2 0 -1 0 Sphere 1 0 0 00FF00 1",
    "Union Cylinder 0 0 0 FF0000 1 2 0 0 400 Sphere 1 0 0 00FF00 1",
    "Union Cylinder 0 0 0 FF0000 1 2 0 0 x Sphere 1 0 0 00FF00 1",
    "Union Cube 0 0 0 FF0000 2 Union Sphere 1 0 0 00FF00 1",
    "Difference Cube 0 0 0 FF0000 2 Sphere 0 0 0 0000FF 1 Sphere 0 0 0 0000FF 1",
    "Intersection Cube 0 0 0 ff00ff 2 Sphere 0.5 0.5 0.5 0a0B0c 1.2",
    "Cube 1.5abc 0 0 FF0000 2",
]


def scene_files():
    return sorted((GOLDEN / "scenes").glob("*.txt"))


def cases():
    """(name, scene text, camera builder, light, w, h) for every fixture case."""
    import csgrt
    from csgrt import scenes

    out = []
    light_default = csgrt.light_dir()
    for f in scene_files():
        text = f.read_text()
        out.append((f"{f.stem}/front", text, lambda: csgrt.Camera().set_fov(60), np.float32([-1, -1, -1]),
                    FIX_W, FIX_H))
        out.append((f"{f.stem}/moved", text,
                    lambda: csgrt.Camera().set_fov(75).rotate(0.21, -0.33).move(0.7, -0.4, 0.25),
                    light_default, FIX_W + 16, FIX_H))
    rng = np.random.default_rng(7)
    for seed in range(2):
        d = scenes.seeded_direction(rng)
        out.append((f"cheese{seed}/lookat", scenes.write_text(scenes.cheese_tree(seed)),
                    (lambda d=d: csgrt.Camera.look_at_origin(d)), light_default, 96, 54))
    for seed in range(8):
        d = scenes.seeded_direction(rng)
        out.append((f"random{seed}/lookat", scenes.write_text(scenes.random_tree(seed, 2, 512, 12)),
                    (lambda d=d: csgrt.Camera.look_at_origin(d, 3.0)), light_default, 96, 54))
    return out


def planes_from(out: dict, n: int) -> dict:
    hit = out["hit"].astype(np.uint8)
    m = hit == 1
    res = {"hit": hit, "prim": np.where(m, out["prim"], -1).astype(np.int32),
           "t": np.where(m, out["t"], np.inf).astype(np.float32),
           "normal": np.where(m[:, None], out["normal"], 0).astype(np.float32)}
    from oracle import quantize_rgba8
    res["rgba8"] = quantize_rgba8(out["rgba"]) if "rgba" in out else out["rgba8"]
    return res


def make_scenes():
    dst = GOLDEN / "scenes"
    dst.mkdir(exist_ok=True)
    for f in sorted(REF_TEST_DIR.glob("*.txt")):
        shutil.copyfile(f, dst / f.name)


def make_host():
    from oracle import RefHost

    R = RefHost()
    parse = {}
    for f in scene_files():
        nodes, prims = R.parse(f.read_bytes())
        parse[f"{f.stem}/nodes"] = nodes.view(np.uint8)
        # zero the parameter slots the reference leaves uninitialised
        p = prims.copy()
        for i in range(len(nodes)):
            if nodes["prim"][i] >= 0 and nodes["type"][i] != 4:
                p["p"][nodes["prim"][i], 1:] = 0
        parse[f"{f.stem}/prims"] = p.view(np.uint8)
    np.savez_compressed(GOLDEN / "ref_parse.npz", **parse)

    errors = []
    from oracle import ParseError
    for text in ERROR_CASES:
        try:
            nodes, prims = R.parse(text)
            errors.append({"text": text, "ok": True, "nodes": int(len(nodes))})
        except ParseError as e:
            errors.append({"text": text, "ok": False, "message": e.msg})
    (GOLDEN / "ref_errors.json").write_text(json.dumps(errors, indent=1) + "\n")

    cams = {}
    cams["default"] = R.camera()
    cams["fov60"] = R.camera(fov_deg=60)
    cams["posrot"] = R.camera(position=(1, 2, 3), rotation=(0.3, -1.2), fov_deg=45)
    cams["clamped"] = R.camera(rotation=(2.0, 7.0))
    c = R.camera(fov_deg=75)
    c = R.camera_rotate(c, 0.21, -0.33)
    cams["moved"] = R.camera_move(c, 0.7, -0.4, 0.25)
    rng = np.random.default_rng(11)
    for i in range(16):
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        pitch = float(np.float32(math.asin(-d[1])))
        yaw = float(np.float32(math.atan2(d[0], d[2])))
        p = tuple(float(np.float32(v)) for v in 4 * d)
        cams[f"lookat{i}"] = R.camera(position=p, rotation=(pitch, yaw), fov_deg=60)
        cams[f"lookat{i}/args"] = np.float32([p[0], p[1], p[2], pitch, yaw])
    cams["light_default"] = R.light_dir()
    cams["light_custom"] = R.light_dir(0.4, 1.1)
    np.savez_compressed(GOLDEN / "ref_camera.npz", **cams)

    arrays = {}
    for name, text, cam_fn, light, w, h in cases():
        nodes, prims = R.parse(text)
        cam = cam_fn().floats()
        out = R.render(nodes, prims, cam, light, w, h, nthreads=8)
        for k, v in planes_from(out, w * h).items():
            arrays[f"{name}/{k}"] = v
        arrays[f"{name}/camera"] = cam
        arrays[f"{name}/light"] = np.float32(light)
        arrays[f"{name}/size"] = np.int32([w, h])
    np.savez_compressed(GOLDEN / "ref_host.npz", **arrays)


def make_gpu(out_path: str):
    import csgrt
    from oracle import RefCuda

    G = RefCuda()
    arrays = {}
    for name, text, cam_fn, light, w, h in cases():
        nodes44, prims48, _ = csgrt.parse_tree(text)
        cam = cam_fn().floats()
        out = G.render(nodes44, prims48, cam, light, w, h)
        for k, v in planes_from(out, w * h).items():
            arrays[f"{name}/{k}"] = v
        arrays[f"{name}/rgba_hit"] = out["rgba"][out["hit"] == 1].astype(np.float32)
        arrays[f"{name}/camera"] = cam
        arrays[f"{name}/light"] = np.float32(light)
        arrays[f"{name}/size"] = np.int32([w, h])
        arrays[f"{name}/thf"] = np.float32([csgrt.device_tan_half_fov(float(cam[5]))])
    np.savez_compressed(out_path, **arrays)


if __name__ == "__main__":
    what = sys.argv[1]
    if what == "scenes":
        make_scenes()
    elif what == "host":
        make_host()
    elif what == "gpu":
        make_gpu(sys.argv[2])
    else:
        raise SystemExit(__doc__)
