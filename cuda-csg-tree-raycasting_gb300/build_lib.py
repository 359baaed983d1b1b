"""Build recipe for libcsgrt.so, the CSG ray-casting engine (C ABI in include/csgrt.h).

CUDA translation units are compiled by nvcc for sm_103a only; host translation units
by g++ with -ffp-contract=off (the camera and parser arithmetic must be the reference's
separately rounded sequence on aarch64 as well as x86-64).  Everything is compiled in
parallel into ``_build/`` beside this file and linked into one shared library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
CSRC = HERE / "csrc"
OUT = HERE / "_build"
LIB = OUT / "libcsgrt.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["render.cu", "render_rec.cu", "noalloc.cu", "views_shapes_w2.cu", "views_shapes_w8.cu", "views_shapes_local.cu",
              "bench_kernels.cu"]
CPP_SOURCES = ["scene.cpp", "capi.cpp", "batch_host.cpp", "server.cpp", "image.cpp"]


def cuda_home() -> Path:
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def _sources(names):
    return [CSRC / n for n in names if (CSRC / n).exists()]


def build(verbose: bool = False, extra_nvcc: list[str] | None = None, out_dir: Path | None = None,
          defines: list[str] | None = None) -> str:
    """Builds libcsgrt.so into `out_dir` (default _build/); `extra_nvcc` adds flags to the
    CUDA translation units (e.g. -D tuning knobs of trace.cuh / render.cu), `defines`
    (NAME=VALUE) to every translation unit (knobs shared by host and device code, such as
    CSG_LIVE_WORDS_MAX)."""
    dflags = [f"-D{d}" for d in (defines or [])]
    OUT = Path(out_dir) if out_dir else globals()["OUT"]
    LIB = OUT / "libcsgrt.so"
    OUT.mkdir(parents=True, exist_ok=True)
    cuda = cuda_home()
    inc = [f"-I{ROOT / 'include'}", f"-I{CSRC}", f"-I{cuda / 'include'}"]
    jobs = []
    objs = []
    for src in _sources(CU_SOURCES):
        obj = OUT / (src.stem + ".cu.o")
        cmd = ["nvcc", *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-v", *inc, *dflags, *(extra_nvcc or []),
               "-c", str(src), "-o", str(obj)]
        jobs.append((src.name, cmd))
        objs.append(obj)
    for src in _sources(CPP_SOURCES):
        obj = OUT / (src.stem + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
               "-Wno-unused-parameter", *inc, *dflags, "-c", str(src), "-o", str(obj)]
        jobs.append((src.name, cmd))
        objs.append(obj)
    procs = [(name, cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
             for name, cmd in jobs]
    logs = []
    failed = []
    for name, cmd, p in procs:
        out = p.communicate()[0]
        logs.append(f"== {name}\n{out}")
        if p.returncode != 0:
            failed.append(f"{name}:\n{' '.join(cmd)}\n{out}")
    (OUT / "build.log").write_text("\n".join(logs))
    if failed:
        raise RuntimeError("libcsgrt build failed:\n" + "\n".join(failed))
    link = ["g++", "-shared", "-o", str(LIB), *map(str, objs), f"-L{cuda / 'lib64'}", "-lcudart",
            f"-Wl,-rpath,{cuda / 'lib64'}"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"libcsgrt link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("\n".join(logs))
    return str(LIB)


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
