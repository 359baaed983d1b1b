"""Build recipe for the C oracle (test infrastructure only): oracle/_build/liboracle.so.

Compiled with ``-ffp-contract=off`` so every separately written product and sum is
rounded on its own on x86-64 and aarch64 alike; the fused operations of the "fma" mode
are explicit ``fmaf`` calls.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "liboracle.so"


def build(extra_flags: list[str] | None = None, out: Path | None = None) -> str:
    OUT.mkdir(parents=True, exist_ok=True)
    out = out or LIB
    cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-math-errno", "-Wall", "-Wno-unused-function", *(extra_flags or []),
           str(HERE / "csg_oracle.c"), "-o", str(out), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return str(out)


def build_refcu(out: Path | None = None) -> str:
    """oracle/_build/librefcu.so: the driver-API runner of the reference's cubin."""
    import shutil
    OUT.mkdir(parents=True, exist_ok=True)
    out = out or (OUT / "librefcu.so")
    nvcc = shutil.which("nvcc")
    cuda = Path(nvcc).resolve().parent.parent if nvcc else Path("/usr/local/cuda")
    cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-Wall", f"-I{cuda / 'include'}",
           str(HERE / "ref_cuda_runner.c"), "-o", str(out), f"-L{cuda / 'lib64' / 'stubs'}", "-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference runner build failed:\n{r.stdout}\n{r.stderr}")
    return str(out)


if __name__ == "__main__":
    print(build())
    print(build_refcu())
