"""Shared test setup: import paths, the `gpu` marker, library fixtures."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "gpu-rt_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def cpq():
    import gpurt_cpq
    return gpurt_cpq


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def reference_root():
    """The reference checkout (one lookup, in the oracle's recipe); tests that
    read its files skip where it is absent, as on a GPU machine."""
    from oracle.make_ref_shade import reference_root as lookup

    root = lookup()
    if not (root / "src").is_dir():
        pytest.skip("no checkout of the reference")
    return root
