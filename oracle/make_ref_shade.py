"""ORACLE recipe: compile the reference's own shading functions as C++.

Reads src/shaders/rt/rtcommon.glsl, restir.glsl and rt.rgen (the
ray-generation shader: camera, integrators, ReSTIR, accumulation), and
src/shaders/tonemap.frag (into oracle/_ref/tonemap_ref.h), from a
checkout of the reference (REFERENCE_ROOT, default /root/reference), applies
the textual rewrites below so they compile as C++ against
oracle/glsl_shim.h, writes the result to oracle/_ref/rtcommon_ref.h and
builds oracle/_ref/libref_shade.so from oracle/ref_shade_wrap.cpp, linked
against the oracle's liboracle.so (its sin / cos / pow / exp and scene
tracer stand behind the shim).  Everything it writes stays in oracle/_ref/
(git-ignored); without a checkout it builds nothing.

Rewrites (syntax only; no function body is changed):
  - #version / #extension / #include lines are dropped (the three files are
    concatenated in include order);
  - uniform blocks (`layout(...) uniform Name {...} inst;`, the push
    constants and the uniform buffer) become C++ structs with one global
    instance; storage-buffer blocks over one unsized array become a global
    pointer (an array of such blocks, a global array of structs holding
    one); other `layout(...) uniform T name;` declarations (images,
    samplers, the acceleration structure) and the ray payload become plain
    globals, as do a stage's `layout(...) in/out` variables; `void main()`
    becomes `void rt_main()`;
  - `inout T x` and `out T x` parameters become `T& x`;
  - floating literals get an `f` suffix (GLSL float literals are FP32);
  - `vec2(randf(seed), randf(seed))` becomes brace initialisation, which
    evaluates its arguments left to right as GLSL does (C++ leaves the
    order of function arguments unspecified).
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
LIB = OUT / "libref_shade.so"


def rewrite(src: str) -> str:
    lines = [ln for ln in src.splitlines() if not re.match(r"\s*#\s*(version|extension|include)\b", ln)]
    s = "\n".join(lines)
    lay = r"layout\s*\([^)]*\)\s*"
    s = re.sub(lay + r"uniform\s+(\w+)\s*\{", r"struct \1 {", s)
    s = re.sub(lay + r"(?:readonly\s+|writeonly\s+)?buffer\s+(\w+)\s*\{\s*(\w+)\s+(\w+)\s*\[\s*\]\s*;\s*\}\s*(\w+)\s*"
               r"\[\s*\]\s*;", r"struct \1 { \2* \3; }; \1* \4;", s)
    s = re.sub(lay + r"(?:readonly\s+|writeonly\s+)?buffer\s+(\w+)\s*\{\s*(\w+)\s+(\w+)\s*\[\s*\]\s*;\s*\}\s*;",
               r"\2* \3;", s)
    s = re.sub(lay + r"uniform\s+(\w+)\s+(\w+)\s*\[\s*\]\s*;", r"\1* \2;", s)
    s = re.sub(lay + r"uniform\s+(\w+)\s+(\w+)\s*;", r"\1 \2;", s)
    s = re.sub(lay + r"rayPayloadEXT\s+", "", s)
    s = re.sub(lay + r"(?:in|out)\s+(\w+)\s+(\w+)\s*;", r"\1 \2;", s)  # stage inputs and outputs
    s = re.sub(r"\bvoid\s+main\s*\(\s*\)", "void rt_main()", s)
    s = re.sub(r"\b(inout|out)\s+(\w+)\s+(\w+)", r"\2& \3", s)
    s = re.sub(r"(?<![\w.])(\d+\.\d*(?:[eE][-+]?\d+)?|\d+[eE][-+]?\d+)(?![\w.])", r"\1f", s)
    s = s.replace("vec2(randf(seed), randf(seed))", "vec2{randf(seed), randf(seed)}")
    return s


def reference_root() -> Path:
    """The reference checkout the oracle's recipes and reference-reading
    tests use: REFERENCE_ROOT, default /root/reference (may be absent)."""
    return Path(os.environ.get("REFERENCE_ROOT", "/root/reference"))


def build(ref_root: Path | None = None) -> Path | None:
    """Generate and compile; returns the library, or None without a checkout."""
    root = Path(ref_root) if ref_root else reference_root()
    rt = root / "src" / "shaders" / "rt"
    if not (rt / "rtcommon.glsl").exists():
        return None
    OUT.mkdir(exist_ok=True)
    body = "\n".join(rewrite((rt / f).read_text()) for f in ("rtcommon.glsl", "restir.glsl", "rt.rgen"))
    hdr = OUT / "rtcommon_ref.h"
    text = ("// generated by oracle/make_ref_shade.py from the reference's shaders; not committed\n#pragma once\n"
            "#undef M_PI\n" + body)  # the shader's own 3.141592, not the C library's
    if not hdr.exists() or hdr.read_text() != text:
        hdr.write_text(text)
    try:
        from . import oracle as O  # imported as oracle.make_ref_shade
    except ImportError:
        import oracle as O  # run as a script from oracle/

    orc = O.build()
    tm = OUT / "tonemap_ref.h"
    tm_text = ("// generated by oracle/make_ref_shade.py from the reference's tonemap.frag; not committed\n"
               "#pragma once\n" + rewrite((root / "src" / "shaders" / "tonemap.frag").read_text()))
    if not tm.exists() or tm.read_text() != tm_text:
        tm.write_text(tm_text)
    wrap = HERE / "ref_shade_wrap.cpp"
    deps = [hdr, tm, wrap, HERE / "glsl_shim.h", HERE / "shade_oracle.h", orc]
    if LIB.exists() and all(LIB.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return LIB
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
                    "-Wno-return-type", "-I", str(HERE), "-I", str(OUT), "-o", str(LIB), str(wrap),
                    "-L", str(HERE), "-loracle", "-Wl,-rpath,$ORIGIN/.."], check=True)
    return LIB


if __name__ == "__main__":
    lib = build(Path(sys.argv[1]) if len(sys.argv) > 1 else None)
    print(lib if lib else "no reference checkout: nothing built")
