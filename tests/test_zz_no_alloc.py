"""vsr_convolve_noalloc: the convolution entry point that allocates nothing.

It serves callers that cannot allocate device memory (a serving process
with a device budget fixed at start-up, a host reaching the library through a
plugin boundary without the process allocator, work issued during a CUDA
graph capture that forbids allocation).  Its scratch is a static device array
inside libvsr, so this test calls it through the C ABI, twice in a row with
different weights, and checks each result against the workspace-taking
vsr_convolve on the same input, within the convolution tests' tolerance
(1e-5 relative; the two share one kernel, so they should agree exactly).
The file is named to be collected last.
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


def test_noalloc_matches_workspace_convolution_twice(vsr):
    import torch

    from vsr_gb300 import _lib, algebra

    lib = _lib.load()
    fn = _noalloc(lib)
    rng = np.random.default_rng(77)
    H, W = 301, 517
    d = (rng.random((H, W)) * 10 + np.linspace(0, 100, H * W).reshape(H, W)).astype(np.float32)
    d[rng.random((H, W)) < 0.02] = -9999.0
    src = torch.from_numpy(d).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    raster = vsr.from_device(src, nodata=-9999.0)
    for k in (31, 5):  # two calls in a row: the second must not see the first's scratch
        w = rng.random((k, k))
        w /= w.sum()
        wc = np.ascontiguousarray(w)
        out = torch.empty((H, W), dtype=torch.float64, device="cuda")
        st = fn(src.data_ptr(), _lib.VSR_F32, H, W, W, wc.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), k, k,
                -9999.0, _lib.VSR_NODATA_VALUE, out.data_ptr(), _lib.VSR_F64, W, _lib.VSR_PREC_FP32, stream)
        _lib.check(st, "vsr_convolve_noalloc")
        ref = algebra.convolve_bands(raster, w, precision="fp32")[0]
        torch.cuda.synchronize()
        a = out.cpu().numpy()
        b = ref.cpu().numpy()
        np.testing.assert_array_equal(np.isnan(a), np.isnan(b))
        m = ~np.isnan(b)
        assert np.all(np.abs(a[m] - b[m]) <= REL * np.maximum(np.abs(b[m]), 1.0)), k


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
