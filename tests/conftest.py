"""Shared fixtures.  `-m gpu` tests need a GPU and the built libpms.so;
everything else runs on the CPU."""
from __future__ import annotations

import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libpms.so")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


def golden_cases():
    return sorted(os.path.basename(p)[len("surface_"):-4] for p in glob.glob(os.path.join(GOLDEN, "surface_*.npz")))


def load_golden(name: str) -> dict:
    z = np.load(os.path.join(GOLDEN, f"surface_{name}.npz"))
    d = {k: z[k] for k in z.files}
    d["config"] = str(d["config"])
    return d


@pytest.fixture(scope="session")
def pms_lib():
    """libpms, built if needed (no GPU required to load it)."""
    from postmps_gb300 import build, pms
    build.build()
    return pms


@pytest.fixture
def tmp_config(tmp_path):
    def make(text: str) -> str:
        p = tmp_path / "config.txt"
        p.write_text(text)
        return str(p)
    return make
