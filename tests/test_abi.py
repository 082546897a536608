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


def test_gaussian_workspace_sizes(lib):
    """The Gaussian's workspace query (host-only): the FP32 kernels need a few KB;
    the tensor-core line passes (8/16-bit rasters; AUTO from k = 35) need their
    two chunk planes -- 2 x 2 KB per 8 padded rows of each 64-column block -- plus
    an aligned copy of one band."""
    from vsr_gb300 import _lib

    plain = lib.vsr_gaussian_workspace_size(65, _lib.VSR_PREC_FP32)
    assert 0 < plain < 64 * 1024
    H = W = 10980
    # k = 65: windows of 64 + 64 positions (Kp = 128), 8-position chunks of 2 KB
    np_chunks = ((H + 63) // 64 * 64 - 64 + 128) // 8
    planes = 2 * ((W + 63) // 64) * np_chunks * 2048
    tc = lib.vsr_gaussian_workspace_bytes(H, W, _lib.VSR_U16, 8.0, 65, _lib.VSR_PREC_AUTO)
    assert planes < tc < planes + H * W * 2 + 64 * 1024
    assert lib.vsr_gaussian_workspace_bytes(H, W, _lib.VSR_U16, 8.0, 65, _lib.VSR_PREC_SPLIT_BF16) == tc
    # FP32 kernels: float rasters, explicit FP32, and AUTO below k = 35
    for dt, k, prec in [(_lib.VSR_F32, 65, _lib.VSR_PREC_AUTO), (_lib.VSR_U16, 65, _lib.VSR_PREC_FP32),
                        (_lib.VSR_U16, 33, _lib.VSR_PREC_AUTO)]:
        assert lib.vsr_gaussian_workspace_bytes(H, W, dt, 8.0, k, prec) < 64 * 1024
    # the default size from sigma (2 ceil(3 sigma) + 1 = 49) and invalid sigma
    assert lib.vsr_gaussian_workspace_bytes(100, 100, _lib.VSR_U16, 8.0, 0, _lib.VSR_PREC_AUTO) > 64 * 1024
    assert lib.vsr_gaussian_workspace_bytes(100, 100, _lib.VSR_U16, 0.0, 0, _lib.VSR_PREC_AUTO) == 0


def _header_prototypes() -> dict[str, tuple[str, list[str]]]:
    """name -> (return type, parameter types) of every VSR_API prototype."""
    text = "\n".join(p.read_text() for p in sorted((ROOT / "include").glob("*.h")))
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    protos = {}
    for ret, name, params in re.findall(r"VSR_API\s+([\w\s\*]+?)\s*\b(vsr_\w+)\s*\(([^)]*)\)\s*;", text):
        ps = [] if params.strip() in ("", "void") else [p.strip() for p in params.split(",")]
        # drop the parameter name, keep the type
        types = [re.sub(r"\s+", " ", re.sub(r"\b\w+$", "", q)).strip() for q in ps]
        protos[name] = (" ".join(ret.split()), types)
    return protos


def _ctype_kind(t) -> str:
    import ctypes

    if t is None:
        return "void"
    if t in (ctypes.c_void_p, ctypes.c_char_p) or (isinstance(t, type) and issubclass(t, ctypes._Pointer)):
        return "ptr"
    # c_size_t and c_uint64 are the same ctypes type on LP64 targets
    return {ctypes.c_int: "int", ctypes.c_int64: "int64_t", ctypes.c_double: "double", ctypes.c_uint32: "uint32_t",
            ctypes.c_size_t: "u64"}[t]


def _c_kind(t: str) -> str:
    if "*" in t:
        return "ptr"
    t = t.replace("const ", "").strip()
    return "u64" if t in ("size_t", "uint64_t") else t


def test_ctypes_signatures_match_the_header():
    """Argument count and kind (pointer, int, int64_t, double, uint32_t, size_t / uint64_t)
    of every binding in ``_lib.SIGNATURES`` against its prototype in vsr.h."""
    from vsr_gb300 import _lib

    protos = _header_prototypes()
    assert set(protos) == set(_lib.SIGNATURES)
    for name, (ret, params) in protos.items():
        restype, argtypes = _lib.SIGNATURES[name]
        assert [_c_kind(p) for p in params] == [_ctype_kind(a) for a in argtypes], name
        assert _c_kind(ret) == _ctype_kind(restype), name


def test_noalloc_scratch_covers_every_supported_kernel(lib):
    """vsr_convolve_noalloc's static scratch (358,912 bytes) holds the workspace
    vsr_convolve asks for at every precision for every kernel up to 80 x 80
    (host-only size queries), and the split-BF16 41 x 41 case fills it exactly."""
    from vsr_gb300 import _lib

    limit = 358912
    for kh in range(1, 81):
        for kw in range(1, 81):
            for prec in (_lib.VSR_PREC_AUTO, _lib.VSR_PREC_FP32, _lib.VSR_PREC_SPLIT_BF16):
                assert lib.vsr_convolve_workspace_size(kh, kw, prec) <= limit, (kh, kw, prec)
    assert lib.vsr_convolve_workspace_size(41, 41, _lib.VSR_PREC_SPLIT_BF16) == limit
