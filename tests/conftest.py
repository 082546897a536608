"""Shared pytest setup: import paths, the ``gpu`` marker and golden fixtures."""

from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG_ROOT = ROOT / "vibespatial-raster_gb300"
for p in (str(ROOT), str(PKG_ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = ROOT / "tests" / "golden" / "focal_golden.npz"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libvsr")


@pytest.fixture(scope="session")
def golden():
    arrays = np.load(GOLDEN)
    manifest = json.loads(GOLDEN.with_suffix(".json").read_text())
    return arrays, manifest


@pytest.fixture(scope="session")
def vsr():
    """The product package with its CUDA library loaded (GPU tests only)."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu-marked test run without a CUDA device")
    import vsr_gb300

    vsr_gb300.load_library()
    return vsr_gb300
