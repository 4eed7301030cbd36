"""Test configuration: paths, the `gpu` marker, fixtures.

`-m "not gpu"` runs anywhere (the CPU oracle against the golden fixtures, the
host logic, the C-ABI exports). `-m gpu` needs a CUDA device and calls the
kernels through the C-ABI; on a machine with a GPU a missing or broken
extension fails those tests rather than skipping them.
"""

from __future__ import annotations

import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "ultrasound-engine_gb300"
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(PKG / "python"))
GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def _have_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAVE_GPU = _have_gpu()


def pytest_collection_modifyitems(config, items):
    if HAVE_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA device on this machine")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def oracle():
    """The CPU oracle (built on demand; it is a few seconds of gcc)."""
    so = ROOT / "oracle" / "liboracle.so"
    if not so.exists():
        sys.path.insert(0, str(PKG))
        import build
        build.build_oracle()
    from oracle import oracle as O
    return O.Lib("oracle")


@pytest.fixture(scope="session")
def golden():
    cache = {}

    def load(name: str):
        if name not in cache:
            cache[name] = dict(np.load(GOLDEN / f"golden_{name}.npz"))
        return cache[name]

    return load
