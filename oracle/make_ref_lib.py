"""ORACLE recipe: the reference's own math headers compiled as C++.

Compiles oracle/ref_lib_wrap.cpp against src/lib/mathlib.h of a checkout of
the reference (REFERENCE_ROOT, default /root/reference; the headers are read
where they lie, nothing is copied) into oracle/_ref/libref_lib.so, git-ignored.
It exposes BBox::enclose, BBox::surface_area (src/lib/bbox.h:35-59) and
Line::closest (src/lib/line.h:28-32) to the tests, which pin the
restatement's boxes, SAH costs and edge projection to them.  Without a
checkout it builds nothing.

The reference's log.h opens log.txt in the working directory when the library
loads; load() therefore loads it from a temporary directory.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys
import tempfile
from ctypes import c_int64, c_void_p
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
LIB = OUT / "libref_lib.so"


def build(ref_root: Path | None = None) -> Path | None:
    """Compile; returns the library, or None without a checkout."""
    try:
        from .make_ref_shade import reference_root
    except ImportError:
        from make_ref_shade import reference_root  # run as a script from oracle/
    root = Path(ref_root) if ref_root else reference_root()
    inc = root / "src" / "lib"
    if not (inc / "mathlib.h").exists():
        return None
    OUT.mkdir(exist_ok=True)
    wrap = HERE / "ref_lib_wrap.cpp"
    deps = [wrap] + sorted(inc.glob("*.h"))
    if LIB.exists() and all(LIB.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return LIB
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
                    "-I", str(inc), "-o", str(LIB), str(wrap)], check=True, cwd=tempfile.gettempdir())
    return LIB


_lib = None


def load():
    """The compiled library with its signatures, or None without a checkout."""
    global _lib
    if _lib is None:
        path = build()
        if path is None:
            _lib = False
        else:
            cwd = os.getcwd()
            with tempfile.TemporaryDirectory() as tmp:
                os.chdir(tmp)  # the reference's log.h opens log.txt here
                try:
                    L = ctypes.CDLL(str(path))
                finally:
                    os.chdir(cwd)
            P = c_void_p
            for name, args in [("ref_bbox_triangles", [c_int64, P, P]), ("ref_bbox_merge", [c_int64, P, P, P]),
                               ("ref_bbox_area", [c_int64, P, P]), ("ref_line_closest", [c_int64, P, P, P, P])]:
                getattr(L, name).argtypes = args
                getattr(L, name).restype = None
            _lib = L
    return _lib or None


if __name__ == "__main__":
    lib = build(Path(sys.argv[1]) if len(sys.argv) > 1 else None)
    print(lib if lib else "no reference checkout: nothing built")
