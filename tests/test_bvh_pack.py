"""The pre-pass BVH the scene packer builds (csrc/scene.cpp, pack_scene), checked on the
CPU by a small C++ program compiled against the packer (tests/bvh_pack/check.cpp): every
leaf reached once, nested boxes, and per-slot bounding spheres that hold their boxes (the
warp-wide cone test of the pre-pass rejects a box only through that sphere, so a sphere
that left part of its box out could drop a live leaf).  Scenes: random trees of 2-4,096
leaves, the cheese scene, a drilled block, the reference's test scenes where present, and
random trees whose text carries nan, inf and huge values."""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np

from conftest import ROOT

SRC = ROOT / "tests" / "bvh_pack" / "check.cpp"
CSRC = ROOT / "cuda-csg-tree-raycasting_gb300" / "csrc"


def test_bvh_pack_invariants(tmp_path):
    import build_lib
    from csgrt import scenes
    exe = tmp_path / "bvh_check"
    cuda = build_lib.cuda_home()
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", f"-I{CSRC}", f"-I{cuda / 'include'}", str(SRC),
           str(CSRC / "scene.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    files = []
    texts = [scenes.write_text(scenes.random_tree(7000 + s, 2, 4096, 12)) for s in range(40)]
    texts += [scenes.write_text(scenes.cheese_tree(0)), scenes.write_text(scenes.drilled_block(0, 30))]
    rng = np.random.default_rng(11)
    specials = ["nan", "inf", "-inf", "1e38", "-1e38"]
    for s in range(20):
        toks = scenes.write_text(scenes.random_tree(9100 + s, 8, 300, 10)).split()
        slots = [i for i, t in enumerate(toks) if t not in scenes.OPERATORS + scenes.PRIMITIVES and len(t) != 6]
        for _ in range(int(rng.integers(1, 4))):
            toks[slots[int(rng.integers(len(slots)))]] = specials[int(rng.integers(len(specials)))]
        texts.append(" ".join(toks))
    for k, t in enumerate(texts):
        p = tmp_path / f"s{k}.txt"
        p.write_text(t)
        files.append(str(p))
    ref_tests = Path(__import__("os").environ.get("CSG_REFERENCE_ROOT", "/root/reference")) / "Test"
    if ref_tests.is_dir():
        files += sorted(str(p) for p in ref_tests.glob("*.txt"))
    r = subprocess.run([str(exe), *files], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr
    checked = int(r.stdout.split("scenes ")[1].split()[0])
    assert checked >= 55, r.stdout  # the 42 generated trees and most of the mutated ones
