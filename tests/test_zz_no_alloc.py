"""vsr_convolve_noalloc: the convolution entry point that allocates nothing.

Some callers cannot allocate device memory and cannot hand the library a
workspace: a serving process whose device memory budget was fixed when it
started, or a host that reaches the library through a plugin boundary
(ctypes, cgo, JNI) with no access to the process's device allocator.  This
entry point keeps its scratch in a static device array inside libvsr, shared
by every call.  The test calls it through the C ABI on several kernels in a
row -- the largest first, so that a smaller call reading stale scratch from a
larger one would show -- and checks each result against the workspace-taking
vsr_convolve (given its own workspace) on the same input, within the
convolution tests' tolerance (1e-5 relative; the two run the same kernels, so
they should agree exactly).  The cases cover every path the scratch serves:
split-BF16 41 x 41 (which fills the whole array), AUTO 31 x 31 on a
well-conditioned kernel (the tensor-core path), FP32 80 x 80 (the largest
kernel) and FP32 5 x 5.  The file is named to be collected last.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-5


def _noalloc(lib):
    fn = lib.vsr_convolve_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                   ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                   ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p]
    return fn


def _with_workspace(lib, src, H, W, wc, k, prec, stream):
    """vsr_convolve with a workspace of its own (a separate device buffer)."""
    import torch

    from vsr_gb300 import _lib

    n = lib.vsr_convolve_workspace_size(k, k, prec)
    ws = torch.empty(n + 256, dtype=torch.uint8, device="cuda")
    wsp = (ws.data_ptr() + 255) // 256 * 256
    out = torch.empty((H, W), dtype=torch.float64, device="cuda")
    st = lib.vsr_convolve(src.data_ptr(), _lib.VSR_F32, H, W, W, wc.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                          k, k, -9999.0, _lib.VSR_NODATA_VALUE, out.data_ptr(), _lib.VSR_F64, W, prec, wsp, n, stream)
    _lib.check(st, "vsr_convolve")
    return out, ws


def test_noalloc_matches_workspace_convolution_in_a_row(vsr):
    import torch

    from vsr_gb300 import _lib

    lib = _lib.load()
    fn = _noalloc(lib)
    rng = np.random.default_rng(77)
    H, W = 301, 517
    d = (rng.random((H, W)) * 10 + np.linspace(0, 100, H * W).reshape(H, W)).astype(np.float32)
    d[rng.random((H, W)) < 0.02] = -9999.0
    src = torch.from_numpy(d).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    cases = [(41, _lib.VSR_PREC_SPLIT_BF16), (31, _lib.VSR_PREC_AUTO), (80, _lib.VSR_PREC_FP32),
             (5, _lib.VSR_PREC_FP32), (31, _lib.VSR_PREC_AUTO)]
    for k, prec in cases:
        w = rng.random((k, k))
        w /= w.sum()
        wc = np.ascontiguousarray(w)
        out = torch.empty((H, W), dtype=torch.float64, device="cuda")
        st = fn(src.data_ptr(), _lib.VSR_F32, H, W, W, wc.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), k, k,
                -9999.0, _lib.VSR_NODATA_VALUE, out.data_ptr(), _lib.VSR_F64, W, prec, stream)
        _lib.check(st, "vsr_convolve_noalloc")
        ref, _ws = _with_workspace(lib, src, H, W, wc, k, prec, stream)
        torch.cuda.synchronize()
        a = out.cpu().numpy()
        b = ref.cpu().numpy()
        np.testing.assert_array_equal(np.isnan(a), np.isnan(b))
        m = ~np.isnan(b)
        assert np.all(np.abs(a[m] - b[m]) <= REL * np.maximum(np.abs(b[m]), 1.0)), (k, prec)


def test_noalloc_rejects_kernels_beyond_its_scratch(vsr):
    import torch

    from vsr_gb300 import _lib

    lib = _lib.load()
    fn = _noalloc(lib)
    src = torch.zeros((8, 8), dtype=torch.float32, device="cuda")
    out = torch.empty((8, 8), dtype=torch.float64, device="cuda")
    w = np.ones((81, 81))
    st = fn(src.data_ptr(), _lib.VSR_F32, 8, 8, 8, w.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 81, 81,
            0.0, _lib.VSR_NODATA_NONE, out.data_ptr(), _lib.VSR_F64, 8, _lib.VSR_PREC_FP32,
            torch.cuda.current_stream().cuda_stream)
    assert st == _lib.VSR_ERR_UNSUPPORTED
    assert b"80x80" in lib.vsr_last_error()
