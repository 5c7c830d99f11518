"""Build the closest-point engine's shared library for sm_103a.

Compiles every CUDA translation unit of ``csrc/`` in parallel with nvcc
(``-gencode arch=compute_103a,code=sm_103a -lineinfo -O3``) and the host-only
C++ ones (``*.cpp``: the glTF reader) with the host compiler, and links
``gpurt_cpq/libgpurt_cpq.so`` in-tree.  No CMake, no torch extension machinery:
the library has a plain C ABI (``include/cpq.h``) and links only the CUDA
runtime.  Run as ``python gpu-rt_gb300/build_ext.py`` or call :func:`build`.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent
CSRC = PKG_ROOT / "csrc"
OUT_DIR = PKG_ROOT / "gpurt_cpq"
LIB_NAME = "libgpurt_cpq.so"
BUILD_DIR = PKG_ROOT / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden",
              "--expt-relaxed-constexpr", "-Werror", "all-warnings"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-Wall", "-Wextra", "-Werror"]
# per-file additions: the path tracer rounds every FP32 expression as written
# (no multiply-add contraction), as the shader's operations do
FILE_FLAGS = {"shade.cu": ["-fmad=false"]}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _needs_rebuild(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile csrc/*.cu and link the shared library; returns its path."""
    nvcc = _nvcc()
    BUILD_DIR.mkdir(exist_ok=True)
    sources = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    headers = (sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) +
               [PKG_ROOT.parent / "include" / "cpq.h"])
    cxx = os.environ.get("CXX") or shutil.which("g++") or "c++"
    objs = []
    jobs = []
    for src in sources:
        obj = BUILD_DIR / (src.stem + ("_host" if src.suffix == ".cpp" else "") + ".o")
        objs.append(obj)
        if force or _needs_rebuild(obj, [src] + headers):
            inc = ["-I", str(PKG_ROOT.parent / "include")]
            if src.suffix == ".cpp":
                cmd = [cxx, *CXX_FLAGS, *inc, "-c", str(src), "-o", str(obj)]
            else:
                cmd = [nvcc, *ARCH, *NVCC_FLAGS, *FILE_FLAGS.get(src.name, []), *inc, "-c", str(src), "-o", str(obj)]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    lib = OUT_DIR / LIB_NAME
    if force or jobs or _needs_rebuild(lib, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lcudart"]
        run(cmd)
    return lib


if __name__ == "__main__":
    p = build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(p)
