"""The C-ABI library builds, loads and exports every symbol include/vsr.h declares.

CPU only: dlopen + symbol binding; no CUDA call is made.
"""

from __future__ import annotations

import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib():
    from vsr_gb300 import _build, _lib

    _build.build()
    return _lib.load()


def _declared_symbols() -> set[str]:
    text = "\n".join(p.read_text() for p in sorted((ROOT / "include").glob("*.h")))
    return set(re.findall(r"VSR_API\s+[\w\s\*]+?\b(vsr_\w+)\s*\(", text))


def test_header_declares_the_bound_symbols():
    from vsr_gb300 import _lib

    declared = _declared_symbols()
    assert declared, "no VSR_API declarations found"
    assert declared == set(_lib.SIGNATURES), (declared ^ set(_lib.SIGNATURES))


def test_library_exports_every_declared_symbol(lib):
    for name in _declared_symbols():
        assert hasattr(lib, name), name


def test_version_and_error_string(lib):
    assert lib.vsr_version() >= 100
    assert isinstance(lib.vsr_last_error(), bytes)


def test_invalid_arguments_are_rejected_without_a_gpu(lib):
    """Argument checks run before any CUDA call and set a message."""
    from vsr_gb300 import _lib

    st = lib.vsr_horn_fused(None, _lib.VSR_F32, 4, 4, 4, 1.0, 1.0, 0.0, 0, 0, 1, None, _lib.VSR_F32, 4,
                            None, 4, 1.0, 0.5, 0.5, None)
    assert st == _lib.VSR_ERR_INVALID_ARG
    assert b"dem" in lib.vsr_last_error()
    st = lib.vsr_horn_fused(1 << 20, _lib.VSR_F32, 4, 4, 2, 1.0, 1.0, 0.0, 0, 0, 1 << 20, None,
                            _lib.VSR_F32, 4, None, 4, 1.0, 0.5, 0.5, None)
    assert st == _lib.VSR_ERR_INVALID_ARG  # pitch < width
    st = lib.vsr_horn_fused(1 << 20, 99, 4, 4, 4, 1.0, 1.0, 0.0, 0, 0, 1 << 20, None, _lib.VSR_F32, 4,
                            None, 4, 1.0, 0.5, 0.5, None)
    assert st == _lib.VSR_ERR_INVALID_ARG  # dtype
    st = lib.vsr_horn_fused(1 << 20, _lib.VSR_F32, 4, 4, 4, 0.0, 1.0, 0.0, 0, 0, 1 << 20, None,
                            _lib.VSR_F32, 4, None, 4, 1.0, 0.5, 0.5, None)
    assert st == _lib.VSR_ERR_INVALID_ARG  # cell size
    # empty rasters are a no-op
    assert lib.vsr_horn_fused(None, _lib.VSR_F32, 0, 7, 7, 1.0, 1.0, 0.0, 0, 0, None, None, _lib.VSR_F32, 7,
                              None, 7, 1.0, 0.5, 0.5, None) == _lib.VSR_OK
