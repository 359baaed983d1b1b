"""A compiled C++ caller of the C ABI (tests/capi_cpp/main.cpp): the reference's
RenderManager integration built with g++ against include/csgrt.h and
libcsgrt.so.  Where the reference's sources are present (CSG_REFERENCE_ROOT, as
oracle/build_ref.py reads it) the program is built with the reference's own Camera.h,
Camera.cpp and DirectionalLight.h and passes those objects across the boundary; elsewhere
a stand-in with the same layout takes their place.

CPU: the layout static_asserts compile, the reference's Camera methods and csg_camera_*
build the same bytes, a parse error carries the reference's message, and the host-only
parse of the README tree equals the reference parser's records (tests/golden).
GPU: csg_render_f4 into a cudaMalloc'd float4 buffer, as RenderManager::CalculateRays
renders into its PBO, equals the reference's own kernels (RefCuda) bit for bit."""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

SRC = ROOT / "tests" / "capi_cpp" / "main.cpp"
CAMERA_REL = Path("CSGRayCasting/Graphics/RenderManager/Camera")
LIGHT_REL = Path("CSGRayCasting/Graphics/RenderManager")


def reference_root() -> Path | None:
    root = Path(os.environ.get("CSG_REFERENCE_ROOT", "/root/reference"))
    return root if (root / CAMERA_REL / "Camera.h").is_file() else None


def build(out_dir: Path, with_reference: bool) -> Path:
    import build_lib
    lib = Path(build_lib.LIB)
    if not lib.exists():
        pytest.skip("libcsgrt.so is not built")
    cuda = build_lib.cuda_home()
    exe = out_dir / ("capi_cpp_ref" if with_reference else "capi_cpp")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-ffp-contract=off", f"-I{ROOT / 'include'}",
           f"-I{cuda / 'include'}"]
    srcs = [str(SRC)]
    if with_reference:
        ref = reference_root()
        cmd += ["-DCSG_REFERENCE_HEADERS", f"-I{ref / CAMERA_REL}", f"-I{ref / LIGHT_REL}"]
        srcs.append(str(ref / CAMERA_REL / "Camera.cpp"))
    cmd += [*srcs, "-o", str(exe), f"-L{lib.parent}", "-lcsgrt", f"-Wl,-rpath,{lib.parent}",
            f"-L{cuda / 'lib64'}", "-lcudart", f"-Wl,-rpath,{cuda / 'lib64'}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def run(exe: Path, *args) -> str:
    r = subprocess.run([str(exe), *map(str, args)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    return r.stdout


@pytest.fixture(scope="module")
def programs(tmp_path_factory, csg):
    if not shutil.which("g++"):
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("capi_cpp")
    out = {"stand-in": build(d, False)}
    if reference_root():
        out["reference"] = build(d, True)
    return out


def test_cpp_caller_layout_and_camera(programs):
    for kind, exe in programs.items():
        assert run(exe, "layout").strip().endswith("same bytes"), kind


def test_cpp_caller_parses_like_the_reference(programs, tmp_path):
    data = np.load(GOLDEN / "ref_parse.npz")
    for case in ("testWikipedia", "testCubeCutEdges", "testCheese256"):
        out = tmp_path / f"{case}.bin"
        run(programs["stand-in"], "parse", GOLDEN / "scenes" / f"{case}.txt", out)
        nodes, prims = data[f"{case}/nodes"], data[f"{case}/prims"]
        raw = out.read_bytes()
        assert raw == nodes.tobytes() + prims.tobytes(), case


@pytest.mark.gpu
def test_cpp_caller_renders_like_the_reference_kernel(programs, tmp_path, csg):
    from oracle import RefCuda
    if not RefCuda.available():
        pytest.skip("reference cubin not built")
    w, h, fov = 1280, 720, 60.0
    scene = GOLDEN / "scenes" / "testWikipedia.txt"
    out = tmp_path / "frame.f4"
    run(programs["stand-in"], "render", scene, w, h, fov, out)
    got = np.fromfile(out, np.float32).reshape(w * h, 4)
    nodes44, prims48, _ = csg.parse_tree(scene.read_text())
    cam = csg.Camera().set_fov(fov).floats()
    ref = RefCuda().render(nodes44, prims48, cam, csg.light_dir(), w, h, want_hits=False)
    assert np.array_equal(got.view(np.uint32), ref["rgba"].view(np.uint32))
