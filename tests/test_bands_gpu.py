"""Band stacks in one launch (vsr_*_bands): every band of the stack equals
the same raster run on its own, bit for bit, on both the TMA / tensor-core
kernels and the generic ones.  (Per-band parity with the oracle is covered
by each operation's own tests; this checks the band indexing.)"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

AFF = (10.0, 0, 0, 0, -10.0, 0)


def _dem_stack(rng, bands, shape, dtype=np.float32):
    y, x = np.mgrid[0 : shape[0], 0 : shape[1]]
    out = []
    for b in range(bands):
        z = 500 + 40 * b + 30 * np.sin(x / (7.0 + b)) + 20 * np.cos(y / 5.0) + rng.normal(0, 2, shape)
        out.append(z)
    return np.stack(out).astype(dtype)


@pytest.mark.parametrize("shape,dtype", [((70, 256), np.float32), ((61, 133), np.float32), ((50, 90), np.uint16)])
def test_terrain_bands_one_launch(vsr, shape, dtype):
    rng = np.random.default_rng(1)
    stack = _dem_stack(rng, 3, shape, dtype)
    nd = -9999.0 if dtype == np.float32 else 0
    stack[1, 7, 9] = nd
    stack[2, -1, -1] = nd
    r = vsr.from_numpy(stack, nodata=nd, affine=AFF)
    out = vsr.raster_terrain(r)
    for b in range(3):
        one = vsr.raster_terrain(vsr.from_numpy(stack[b], nodata=nd, affine=AFF))
        for k in ("slope", "aspect", "hillshade"):
            np.testing.assert_array_equal(out[k].to_numpy()[b], one[k].to_numpy(), err_msg=f"{k} band {b}")
    rs, _ = oracle.slope_aspect(stack[2], AFF, nd)
    s2 = out["slope"].to_numpy()[2].astype(np.float64)
    fin = ~np.isnan(rs)
    assert np.abs(s2[fin] - rs[fin]).max() <= 1e-4


def test_terrain_bands_strided_outputs(vsr):
    """Output band strides other than H * W (a padded output buffer)."""
    import torch

    from vsr_gb300 import _lib

    rng = np.random.default_rng(2)
    stack = _dem_stack(rng, 2, (40, 64))
    src = torch.from_numpy(stack).cuda()
    H, W = 40, 64
    big = torch.full((2, H + 3, W), -1.0, dtype=torch.float32, device="cuda")
    lib = _lib.load()
    st = lib.vsr_horn_fused_bands(src.data_ptr(), _lib.VSR_F32, 2, H * W, H, W, W, 10.0, 10.0, 0.0,
                                  _lib.VSR_NODATA_NONE, 0, big.data_ptr(), None, _lib.VSR_F32, (H + 3) * W, W,
                                  None, 0, 0, 1.0, 0.7, 5.5, None)
    _lib.check(st, "vsr_horn_fused_bands")
    got = big.cpu().numpy()
    for b in range(2):
        one = vsr.raster_slope(vsr.from_numpy(stack[b], affine=AFF)).to_numpy()
        np.testing.assert_array_equal(got[b, :H], one)
        assert (got[b, H:] == -1.0).all()
    bad = lib.vsr_horn_fused_bands(src.data_ptr(), _lib.VSR_F32, 2, H * W - 1, H, W, W, 10.0, 10.0, 0.0,
                                   _lib.VSR_NODATA_NONE, 0, big.data_ptr(), None, _lib.VSR_F32, (H + 3) * W, W,
                                   None, 0, 0, 1.0, 0.7, 5.5, None)
    assert bad == _lib.VSR_ERR_INVALID_ARG


@pytest.mark.parametrize("precision,k", [("split_bf16", 31), ("fp32", 31), ("fp32", 5)])
def test_convolve_bands_one_launch(vsr, precision, k):
    from vsr_gb300 import algebra

    rng = np.random.default_rng(k)
    stack = (rng.random((3, 150, 200)) * 10 + np.arange(3)[:, None, None] * 50).astype(np.float32)
    stack[1, 20:24, 30:33] = -9999.0
    w = rng.random((k, k))
    w /= w.sum()
    r = vsr.from_numpy(stack, nodata=-9999.0)
    out = algebra.convolve_bands(r, w, precision=precision).cpu().numpy()
    for b in range(3):
        one = vsr.raster_convolve(vsr.from_numpy(stack[b], nodata=-9999.0), w, precision=precision).to_numpy()
        np.testing.assert_array_equal(out[b], one, err_msg=f"band {b}")


def test_terrain_derivative_bands_one_launch(vsr):
    rng = np.random.default_rng(4)
    stack = _dem_stack(rng, 3, (33, 47), np.float32)
    stack[0, 3, 3] = -9999.0
    r = vsr.from_numpy(stack, nodata=-9999.0, affine=AFF)
    out = vsr.raster_terrain_derivatives(r)
    for b in range(3):
        one = vsr.raster_terrain_derivatives(vsr.from_numpy(stack[b], nodata=-9999.0, affine=AFF))
        for k in ("tri", "tpi", "curvature"):
            np.testing.assert_array_equal(out[k].to_numpy()[b], one[k].to_numpy())


def test_bands_argument_checks(vsr):
    from vsr_gb300 import _lib

    lib = _lib.load()
    w = np.ones((3, 3))
    wp = w.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    # bands out of range and strides smaller than a band are rejected before any launch
    assert lib.vsr_convolve_bands(8, _lib.VSR_F32, 0, 100, 10, 10, 10, wp, 3, 3, 0.0, 0, 8, _lib.VSR_F32, 100, 10,
                                  _lib.VSR_PREC_FP32, None, 0, None) == _lib.VSR_ERR_INVALID_ARG
    assert lib.vsr_convolve_bands(8, _lib.VSR_F32, 2, 99, 10, 10, 10, wp, 3, 3, 0.0, 0, 8, _lib.VSR_F32, 100, 10,
                                  _lib.VSR_PREC_FP32, None, 0, None) == _lib.VSR_ERR_INVALID_ARG
    assert lib.vsr_terrain_derivatives_bands(8, _lib.VSR_F32, 2, 100, 10, 10, 10, 1.0, 1.0, 0.0, 0, -9999.0, 8, None,
                                             None, _lib.VSR_F64, 99, 10, None) == _lib.VSR_ERR_INVALID_ARG


@pytest.mark.parametrize("dtype,shape", [(np.uint16, (150, 200)), (np.uint8, (97, 131))])
def test_tensor_core_gaussian_bands_one_launch_and_groups(vsr, dtype, shape):
    """The tensor-core Gaussian over a 3-band stack: one launch pair (room for
    every band's row sums), groups of two and one band (smaller workspaces),
    and each band on its own all agree bit for bit; the stack matches the
    oracle.  The uint8 case has rows that are not 8-byte aligned (the bands
    are then copied one at a time to an aligned pitch)."""
    import torch

    from vsr_gb300 import _lib, algebra

    rng = np.random.default_rng(5)
    hi = 250 if dtype == np.uint8 else 9000
    stack = rng.integers(1, hi, (3,) + shape).astype(dtype)
    stack[1, 40:44, 50:55] = 0
    B, H, W = stack.shape
    r = vsr.from_numpy(stack, nodata=0)
    full = algebra.gaussian_bands(r, 6.0, 49, precision="split", out_dtype=np.float32).cpu().numpy()
    lib = _lib.load()
    code = _lib.dtype_code(stack.dtype)
    src = torch.from_numpy(stack).cuda()
    one = lib.vsr_gaussian_bands_workspace_bytes(1, H, W, code, 6.0, 49, _lib.VSR_PREC_SPLIT)
    three = lib.vsr_gaussian_bands_workspace_bytes(3, H, W, code, 6.0, 49, _lib.VSR_PREC_SPLIT)
    assert three > one
    for nbytes in (one, (one + three) // 2):  # groups of 1, then of 2 + 1
        ws = torch.empty(nbytes + 256, dtype=torch.uint8, device="cuda")
        dst = torch.full((B, H, W), -1.0, dtype=torch.float32, device="cuda")
        p = (ws.data_ptr() + 255) // 256 * 256
        st = lib.vsr_gaussian_bands(src.data_ptr(), code, B, H * W, H, W, W, 6.0, 49, 0.0, _lib.VSR_NODATA_VALUE,
                                    dst.data_ptr(), _lib.VSR_F32, H * W, W, _lib.VSR_PREC_SPLIT, p, nbytes, None)
        _lib.check(st, "vsr_gaussian_bands")
        np.testing.assert_array_equal(dst.cpu().numpy(), full)
    w = oracle.gaussian_weights(6.0, 49)
    for b in range(B):
        single = algebra.gaussian_bands(vsr.from_numpy(stack[b], nodata=0), 6.0, 49, precision="split",
                                        out_dtype=np.float32).cpu().numpy()[0]
        np.testing.assert_array_equal(full[b], single)
        ref = oracle.convolve_normalized(stack[b], w, 0)
        m = ref != 0
        np.testing.assert_array_equal(full[b] == 0, ~m)
        assert (np.abs(full[b][m] - ref[m]) / np.abs(ref[m])).max() <= 2e-6
