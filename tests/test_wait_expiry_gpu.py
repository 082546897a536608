"""The bounded mbarrier wait that every TMA / tensor-core kernel uses gives
up cleanly: a wait on a barrier that nothing completes runs out after its
(short) limit, raises VSR_DEVERR_TMA_TIMEOUT in the device error word, leaves
nothing in flight, and the next launch on the same context works."""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def test_wait_expiry_reports_and_context_survives(vsr):
    import torch

    from vsr_gb300 import _lib

    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    code = ctypes.c_uint32(0)
    _lib.check(lib.vsr_poll_device_error(stream, ctypes.byref(code)), "poll")  # clear earlier bits
    res = torch.zeros(2, dtype=torch.int32, device="cuda")
    limit_ns = 2_000_000  # 2 ms
    _lib.check(lib.vsr_wait_selftest(limit_ns, res.data_ptr(), stream), "vsr_wait_selftest")
    _lib.check(lib.vsr_poll_device_error(stream, ctypes.byref(code)), "poll")
    assert code.value == _lib.VSR_DEVERR_TMA_TIMEOUT
    gave_up, waited = res.cpu().numpy().view(np.uint32)
    assert gave_up == 1
    assert limit_ns <= waited < 200 * limit_ns
    # the error word was cleared by the poll, and the context still runs kernels
    _lib.check(lib.vsr_poll_device_error(stream, ctypes.byref(code)), "poll")
    assert code.value == 0
    dem = (np.arange(40 * 64, dtype=np.float32).reshape(40, 64) % 97) * 3.0
    out = vsr.raster_slope(vsr.from_numpy(dem)).to_numpy()
    ref = oracle.slope_aspect(dem, (1.0, 0, 0, 0, -1.0, 0), None, compute_aspect=False)[0]
    np.testing.assert_allclose(out, ref, atol=1e-4, rtol=0)
    _lib.check(lib.vsr_poll_device_error(stream, ctypes.byref(code)), "poll")
    assert code.value == 0


def test_wait_limit_is_checked(vsr):
    import torch

    from vsr_gb300 import _lib

    lib = _lib.load()
    res = torch.zeros(2, dtype=torch.int32, device="cuda")
    assert lib.vsr_wait_selftest(10, res.data_ptr(), None) == _lib.VSR_ERR_INVALID_ARG
    assert lib.vsr_wait_selftest(3_000_000_000, res.data_ptr(), None) == _lib.VSR_ERR_INVALID_ARG
    assert lib.vsr_wait_selftest(10_000, None, None) == _lib.VSR_ERR_INVALID_ARG
