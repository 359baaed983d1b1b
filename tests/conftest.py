"""Shared test setup: import paths, the `gpu` marker, and common fixtures."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (str(ROOT), str(ROOT / "cuda-csg-tree-raycasting_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def pytest_collection_modifyitems(config, items):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA GPU on this machine")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def csg():
    import csgrt
    csgrt.lib()
    return csgrt


def load_cases(npz_path: Path) -> dict:
    """{case name: {field: array}} from a golden npz keyed 'case/field'."""
    data = np.load(npz_path)
    cases: dict = {}
    for key in data.files:
        case, field = key.rsplit("/", 1)
        cases.setdefault(case, {})[field] = data[key]
    return cases


def scene_text(case: str) -> str:
    """Scene text for a golden case name (scene file stem, or a generated config)."""
    from csgrt import scenes
    stem = case.split("/")[0]
    f = GOLDEN / "scenes" / f"{stem}.txt"
    if f.exists():
        return f.read_text()
    if stem.startswith("cheese"):
        return scenes.write_text(scenes.cheese_tree(int(stem[len("cheese"):])))
    if stem.startswith("random"):
        return scenes.write_text(scenes.random_tree(int(stem[len("random"):]), 2, 512, 12))
    raise KeyError(case)


def ulp_equal(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    return np.asarray(a, np.float32).view(np.uint32) == np.asarray(b, np.float32).view(np.uint32)
