"""Source-level guards on the product boundary.

The oracle (oracle/) is test infrastructure: the product package and its
CUDA/C++ sources must neither import it nor link it, so that no product path
can route through the CPU checker.  And nothing committed may use a scratch
path (_work/).
"""
from __future__ import annotations

import re
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "gpu-rt_gb300"


def _product_sources():
    return [p for p in PKG.rglob("*") if p.suffix in {".py", ".cu", ".cuh", ".cpp", ".h"} and p.is_file()]


def test_product_never_reaches_the_oracle():
    pat = re.compile(r"(^\s*(from|import)\s+oracle\b)|liboracle|cpq_oracle|shade_oracle|orc_[a-z]", re.M)
    hits = [f"{p.relative_to(ROOT)}: {m.group(0)}" for p in _product_sources()
            for m in [pat.search(p.read_text(errors="replace"))] if m]
    assert not hits, hits
    assert _product_sources(), "no product sources found"


def test_nothing_committed_uses_scratch_paths():
    try:
        files = subprocess.run(["git", "ls-files"], cwd=ROOT, capture_output=True, text=True,
                               check=True).stdout.split()
    except (OSError, subprocess.CalledProcessError):
        # folders the repository ignores (.gitignore entries ending in "/") are not committed:
        # an entry with an inner "/" is a path from the root, others match any folder name
        import fnmatch

        dirs = [ln.strip().strip("/") for ln in (ROOT / ".gitignore").read_text().splitlines()
                if ln.strip().endswith("/") and not ln.startswith("#")]

        def ignored(rel: Path) -> bool:
            parts = rel.parts[:-1]
            for d in dirs:
                if "/" in d:
                    if "/".join(parts).startswith(d):
                        return True
                elif any(fnmatch.fnmatch(q, d) for q in parts):
                    return True
            return ".git" in parts

        files = [str(p.relative_to(ROOT)) for p in ROOT.rglob("*") if p.is_file() and not ignored(p.relative_to(ROOT))]
    pat = re.compile(r"(?<![A-Za-z0-9])_work/")
    hits = []
    for f in files:
        if f in {".gitignore", ".gpurunignore", "tests/test_boundaries.py"} or f.endswith(".md"):
            continue
        p = ROOT / f
        if p.suffix in {".so", ".npz", ".png", ".bin"} or not p.is_file():
            continue
        if pat.search(p.read_text(errors="replace")):
            hits.append(f)
    assert not hits, hits
