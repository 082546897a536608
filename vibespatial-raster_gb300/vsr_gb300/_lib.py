"""ctypes binding of libvsr.so (the sm_103a C ABI declared in include/vsr.h).

The library is loaded once per process.  There is no fallback: if the shared
library is missing or CUDA is unavailable, every operation raises.
"""

from __future__ import annotations

import ctypes
import threading
from pathlib import Path

import numpy as np

from vsr_gb300._build import LIB_PATH

VSR_OK = 0
VSR_ERR_INVALID_ARG = 1
VSR_ERR_UNSUPPORTED = 2
VSR_ERR_CUDA = 3
VSR_ERR_WORKSPACE = 4
VSR_ERR_DEVICE = 5

VSR_U8, VSR_I16, VSR_U16, VSR_I32, VSR_F32, VSR_F64 = 1, 2, 3, 4, 5, 6
VSR_NODATA_NONE, VSR_NODATA_VALUE, VSR_NODATA_NAN = 0, 1, 2
VSR_HORN_CENTER_ONLY = 1
VSR_HORN_SA_NAN_UNMASKED = 2
VSR_PREC_AUTO, VSR_PREC_FP32, VSR_PREC_SPLIT = 0, 1, 2
VSR_PREC_SPLIT_BF16 = VSR_PREC_SPLIT  # earlier name of the same code
VSR_OP_HORN, VSR_OP_BATCH = 1, 2
VSR_DEVERR_TMA_TIMEOUT, VSR_DEVERR_MMA_TIMEOUT, VSR_DEVERR_QUEUE, VSR_DEVERR_PLAN = 1, 2, 4, 8
VSR_STAT = {"min": 0, "max": 1, "mean": 2, "std": 3, "range": 4, "variety": 5}

DTYPE_CODES = {
    np.dtype(np.uint8): VSR_U8,
    np.dtype(np.int16): VSR_I16,
    np.dtype(np.uint16): VSR_U16,
    np.dtype(np.int32): VSR_I32,
    np.dtype(np.float32): VSR_F32,
    np.dtype(np.float64): VSR_F64,
}

_c = ctypes
_i64 = _c.c_int64
_vp = _c.c_void_p
_dbl = _c.c_double
_int = _c.c_int
_u32 = _c.c_uint32
_sz = _c.c_size_t

# name -> (restype, argtypes); every symbol include/vsr.h declares.
SIGNATURES: dict[str, tuple] = {
    "vsr_version": (_int, []),
    "vsr_last_error": (_c.c_char_p, []),
    "vsr_device_info": (_int, [_c.POINTER(_int), _c.POINTER(_int), _c.POINTER(_int)]),
    "vsr_poll_device_error": (_int, [_vp, _c.POINTER(_u32)]),
    "vsr_wait_selftest": (_int, [_c.c_uint64, _vp, _vp]),
    "vsr_tuning_count": (_int, [_int]),
    "vsr_tuning_set": (_int, [_int, _int]),
    "vsr_tuning_get": (_int, [_int]),
    "vsr_horn_fused": (
        _int,
        [_vp, _int, _i64, _i64, _i64, _dbl, _dbl, _dbl, _int, _u32, _vp, _vp, _int, _i64, _vp, _i64,
         _dbl, _dbl, _dbl, _vp],
    ),
    "vsr_horn_fused_bands": (
        _int,
        [_vp, _int, _int, _i64, _i64, _i64, _i64, _dbl, _dbl, _dbl, _int, _u32, _vp, _vp, _int, _i64, _i64, _vp,
         _i64, _i64, _dbl, _dbl, _dbl, _vp],
    ),
    "vsr_terrain_derivatives_bands": (
        _int,
        [_vp, _int, _int, _i64, _i64, _i64, _i64, _dbl, _dbl, _dbl, _int, _dbl, _vp, _vp, _vp, _int, _i64, _i64,
         _vp],
    ),
    "vsr_convolve_bands": (
        _int,
        [_vp, _int, _int, _i64, _i64, _i64, _i64, _c.POINTER(_dbl), _int, _int, _dbl, _int, _vp, _int, _i64, _i64,
         _int, _vp, _sz, _vp],
    ),
    "vsr_terrain_derivatives": (
        _int,
        [_vp, _int, _i64, _i64, _i64, _dbl, _dbl, _dbl, _int, _dbl, _vp, _vp, _vp, _int, _i64, _vp],
    ),
    "vsr_convolve_workspace_size": (_sz, [_int, _int, _int]),
    "vsr_convolve": (
        _int,
        [_vp, _int, _i64, _i64, _i64, _c.POINTER(_dbl), _int, _int, _dbl, _int, _vp, _int, _i64, _int,
         _vp, _sz, _vp],
    ),
    "vsr_convolve_noalloc": (
        _int,
        [_vp, _int, _i64, _i64, _i64, _c.POINTER(_dbl), _int, _int, _dbl, _int, _vp, _int, _i64, _int, _vp],
    ),
    "vsr_gaussian_workspace_size": (_sz, [_int, _int]),
    "vsr_gaussian_workspace_bytes": (_sz, [_i64, _i64, _int, _dbl, _int, _int]),
    "vsr_gaussian_bands_workspace_bytes": (_sz, [_int, _i64, _i64, _int, _dbl, _int, _int]),
    "vsr_gaussian": (
        _int,
        [_vp, _int, _i64, _i64, _i64, _dbl, _int, _dbl, _int, _vp, _int, _i64, _int, _vp, _sz, _vp],
    ),
    "vsr_tiff_assemble": (
        _int,
        [_vp, _vp, _int, _int, _int, _int, _int, _int, _int, _i64, _i64, _vp, _i64, _i64, _vp],
    ),
    "vsr_batch_plan_size": (_sz, [_int]),
    "vsr_batch_plan": (_int, [_vp, _int, _dbl, _int, _vp, _sz, _c.POINTER(_c.c_int64), _vp]),
    "vsr_batch_run": (_int, [_vp, _int, _vp]),
    "vsr_gaussian_bands": (
        _int,
        [_vp, _int, _int, _i64, _i64, _i64, _i64, _dbl, _int, _dbl, _int, _vp, _int, _i64, _i64, _int, _vp, _sz, _vp],
    ),
    "vsr_focal_mean_bands": (
        _int,
        [_vp, _int, _int, _i64, _i64, _i64, _i64, _int, _int, _dbl, _int, _vp, _int, _i64, _i64, _vp],
    ),
    "vsr_focal_mean": (
        _int,
        [_vp, _int, _i64, _i64, _i64, _int, _int, _dbl, _int, _vp, _int, _i64, _vp],
    ),
    "vsr_focal_stat": (
        _int,
        [_vp, _int, _i64, _i64, _i64, _int, _int, _int, _dbl, _int, _vp, _int, _i64, _vp],
    ),
    "vsr_focal_stat_bands": (
        _int,
        [_vp, _int, _int, _i64, _i64, _i64, _i64, _int, _int, _int, _dbl, _int, _vp, _int, _i64, _i64, _vp],
    ),
}

_lock = threading.Lock()
_lib: ctypes.CDLL | None = None


class VsrError(RuntimeError):
    """A libvsr call failed (CUDA error or device-side error)."""


def load(path: str | Path | None = None) -> ctypes.CDLL:
    """Load libvsr.so and bind every exported symbol.  Raises if absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise RuntimeError(
                f"libvsr.so not found at {p}; build it first "
                "(python -c 'import __graft_entry__ as g; g.build()')"
            )
        lib = ctypes.CDLL(str(p))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)  # AttributeError if a declared symbol is missing
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def last_error() -> str:
    lib = load()
    msg = lib.vsr_last_error()
    return msg.decode() if msg else ""


def check(status: int, what: str) -> None:
    """Map a libvsr status to the reference-style Python exception."""
    if status == VSR_OK:
        return
    msg = f"{what}: {last_error()}"
    if status in (VSR_ERR_INVALID_ARG, VSR_ERR_WORKSPACE):
        raise ValueError(msg)
    if status == VSR_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise VsrError(msg)


def dtype_code(dt) -> int:
    code = DTYPE_CODES.get(np.dtype(dt))
    if code is None:
        raise ValueError(f"unsupported raster dtype {np.dtype(dt)}")
    return code
