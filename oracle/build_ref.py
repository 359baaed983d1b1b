"""Build recipe for the reference's own code, used only as a test oracle.

Reads the reference sources where they lie (default ``/root/reference``, override with
``CSG_REFERENCE_ROOT``) and writes every output under ``oracle/_ref/`` (git-ignored):

* ``oracle/_ref/src/RaycastingKernels.cu`` -- a build copy of
  ``CSGRayCasting/Graphics/RayCasting/Kernels/RaycastingKernels.cu`` with one neutral
  patch: ``return true;`` appended to ``cylinderHit`` (the function falls off the end of
  a ``bool`` function at RaycastingKernels.cu:335-336, which under optimisation makes
  every cylinder scene loop forever; ``hitPrimitive`` never reads the return value,
  RaycastingKernels.cu:113-133, so outputs are unchanged).  This copy never leaves the
  machine it was made on (the repository's ignore lists exclude it).
* ``oracle/_ref/libref_host.so`` -- the reference kernels, parser and camera compiled as
  host C++ with OpenMP (``oracle/ref_host_shim.cpp``).  Pins the C restatement.
* ``oracle/_ref/ref_kernels.cubin`` -- the reference's ``RaycastKernel`` and
  ``LightningKernel`` compiled by nvcc for sm_103a with the reference's default flags
  (``--fmad=true``, IEEE div/sqrt, no ftz).  Device code only; it is launched on a GPU
  through ``oracle/ref_cuda_runner.c``.

Nothing in the product links or loads anything built here.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
SRC = OUT / "src"

KERNELS_REL = "CSGRayCasting/Graphics/RayCasting/Kernels"
TREE_REL = "CSGRayCasting/Graphics/RayCasting/CSGTree"
CAMERA_REL = "CSGRayCasting/Graphics/RenderManager/Camera"

# Itanium-mangled names of the two reference kernels, as nvcc emits them for
# RaycastingKernels.cuh:39 and :42 (checked against ptxas -v output when building).
RAYCAST_KERNEL = "_Z13RaycastKernel6Camera11CudaCSGTreeP6RayHitff"
LIGHTNING_KERNEL = "_Z15LightningKernel6CameraP6RayHitP9PrimitiveP6float46float3ff"


def reference_root() -> Path | None:
    root = Path(os.environ.get("CSG_REFERENCE_ROOT", "/root/reference"))
    return root if (root / KERNELS_REL / "RaycastingKernels.cu").is_file() else None


def cuda_home() -> Path:
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def _patched_kernels(root: Path) -> Path:
    """Write the build copy of RaycastingKernels.cu with the cylinderHit return patch."""
    src = (root / KERNELS_REL / "RaycastingKernels.cu").read_text()
    lines = src.split("\n")
    # Locate the end of cylinderHit: the line that sets primitiveType to Cylinder,
    # followed by the closing brace of the function.
    idx = None
    for i, line in enumerate(lines):
        if "hitInfo.primitiveType = CSGTree::NodeType::Cylinder;" in line:
            idx = i
    if idx is None or lines[idx + 1].strip() != "}":
        raise RuntimeError("cylinderHit end not found where expected; refusing to patch")
    lines.insert(idx + 1, "\treturn true; // build-copy patch: falls off the end otherwise")
    SRC.mkdir(parents=True, exist_ok=True)
    dst = SRC / "RaycastingKernels.cu"
    dst.write_text("\n".join(lines))
    return dst


def build(verbose: bool = False) -> dict:
    """Build libref_host.so and ref_kernels.cubin.  Returns {name: path or None}."""
    root = reference_root()
    if root is None:
        return {"host": None, "cubin": None}
    OUT.mkdir(parents=True, exist_ok=True)
    _patched_kernels(root)
    cuda = cuda_home()
    incs = [f"-I{SRC}", f"-I{root / KERNELS_REL}", f"-I{root / TREE_REL}", f"-I{root / CAMERA_REL}"]

    host_so = OUT / "libref_host.so"
    host_cmd = ["g++", "-O3", "-fopenmp", "-std=c++17", "-fPIC", "-shared", "-w",
                # no FMA contraction on any host: the x86-64 baseline has no FMA and an
                # aarch64 build must compute the same IEEE sequence
                "-ffp-contract=off",
                f"-I{cuda / 'include'}", *incs, str(HERE / "ref_host_shim.cpp"),
                str(root / CAMERA_REL / "Camera.cpp"),
                "-o", str(host_so)]
    cubin = OUT / "ref_kernels.cubin"
    cubin_cmd = ["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a",
                 "-std=c++17", "--expt-relaxed-constexpr", "-w", "-Xptxas", "-v",
                 *incs, str(SRC / "RaycastingKernels.cu"), "-o", str(cubin)]
    procs = []
    for cmd in (host_cmd, cubin_cmd):
        procs.append(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
    outs = [p.communicate()[0] for p in procs]
    res = {}
    for name, p, out, path in zip(("host", "cubin"), procs, outs, (host_so, cubin)):
        if p.returncode != 0:
            raise RuntimeError(f"reference {name} build failed:\n{out}")
        if verbose:
            print(out)
        res[name] = str(path)
    names = set(re.findall(r"entry function '([^']+)'", outs[1]))
    missing = {RAYCAST_KERNEL, LIGHTNING_KERNEL} - names
    if missing:
        raise RuntimeError(f"reference cubin lacks expected entries {missing}; found {names}")
    (OUT / "ref_kernels.ptxas.txt").write_text(outs[1])
    return res


if __name__ == "__main__":
    r = build(verbose="-v" in sys.argv)
    print(r)
