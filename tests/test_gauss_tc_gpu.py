"""GPU parity of the split-precision tensor-core Gaussian (two line passes) vs the oracle.

The reference Gaussian (algebra.py:2120-2154) is the normalised correlation
with weights outer(g, g) / sum; the oracle evaluates it densely in float64.
The tensor-core passes split the weights and the row pass's float32 sums into
F16 hi/lo pairs; the row pass multiplies both weight parts with the exact
byte planes of the integer values (v = 256 h + l), the column pass drops only
its lo*lo products: the bound asserted here is 2e-6 relative --
|out - ref| <= 2e-6 * max(|ref|, scale), ``scale`` the mean |value| of the
input -- with nodata placement exact.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

REL_TC = 2e-6


def _max_rel(out, ref, data, nodata):
    out = np.asarray(out, np.float64)
    ref = np.asarray(ref, np.float64)
    if nodata is not None:
        np.testing.assert_array_equal(out == nodata, ref == nodata)
        m = ref != nodata
    else:
        m = np.ones(ref.shape, bool)
    scale = float(np.mean(np.abs(np.asarray(data, np.float64)))) or 1.0
    return float(np.max(np.abs(out[m] - ref[m]) / np.maximum(np.abs(ref[m]), scale), initial=0.0))


def _raster(dtype, shape, nodata, seed):
    rng = np.random.default_rng(seed)
    if dtype == np.uint16:
        d = np.clip(rng.gamma(2.0, 800.0, shape), 0, 10000).astype(np.uint16)
    elif dtype == np.uint8:
        d = rng.integers(0, 255, shape).astype(np.uint8)
    else:
        d = rng.integers(-30000, 30000, shape).astype(np.int16)
    if nodata is not None:
        d[rng.random(shape) < 0.03] = nodata
    return d


@pytest.mark.parametrize("dtype,nodata,shape,k", [
    (np.uint16, 0, (300, 260), 65),       # the multiband workload's kernel, ragged tiles both ways
    (np.uint16, 0, (1100, 200), 35),      # smallest automatic size, tall
    (np.uint16, None, (200, 333), 79),    # largest kernel, no nodata
    (np.uint8, 255, (257, 190), 49),
    (np.int16, -9999, (190, 257), 65),    # negative values, nodata inside the value range
    (np.uint16, 0, (70, 66), 15),         # kernel larger than a quarter of the raster
    (np.uint16, 0, (65, 129), 65),        # row-pass tile past the last 64-column block; 1 row past a line block
    (np.uint8, 0, (97, 60), 3),           # narrower than one row-pass tile; smallest kernel (window lead 8)
    (np.uint16, 0, (97, 131), 41),        # odd width: rows copied to an aligned pitch first
    (np.int16, -32768, (140, 700), 79),   # several row-pass tiles per line, signed high bytes
])
def test_split_bf16_gaussian_vs_oracle(vsr, dtype, nodata, shape, k):
    d = _raster(dtype, shape, nodata, k + shape[0])
    sigma = k / 8.0
    ref = oracle.convolve_normalized(d, oracle.gaussian_weights(sigma, k), nodata)
    r = vsr.from_numpy(d, nodata=nodata)
    out = vsr.raster_gaussian_filter(r, sigma, kernel_size=k, precision="split_bf16").to_numpy()
    err = _max_rel(out, ref, d, nodata)
    assert err <= REL_TC, f"max rel err {err:.3e}"


def test_split_bf16_gaussian_float32_output_and_bands(vsr):
    """All bands of a stack in one call (the passes reuse one workspace band
    after band), float32 output equal to the float64 output rounded."""
    from vsr_gb300 import algebra

    stack = np.stack([_raster(np.uint16, (150, 170), 0, s) for s in range(3)])
    r = vsr.from_numpy(stack, nodata=0)
    o64 = algebra.gaussian_bands(r, 8.0, 65, precision="split_bf16").cpu().numpy()
    o32 = algebra.gaussian_bands(r, 8.0, 65, precision="split_bf16", out_dtype=np.float32).cpu().numpy()
    np.testing.assert_array_equal(o32, o64.astype(np.float32))
    for b in range(3):
        ref = oracle.convolve_normalized(stack[b], oracle.gaussian_weights(8.0, 65), 0)
        assert _max_rel(o64[b], ref, stack[b], 0) <= REL_TC


def test_auto_takes_tensor_cores_for_integer_rasters(vsr):
    """precision="auto" on a uint16 raster with k >= 35 gives the split-BF16
    result bit for bit; k = 33 stays on the FP32 kernels."""
    d = _raster(np.uint16, (130, 140), 0, 7)
    r = vsr.from_numpy(d, nodata=0)
    auto = vsr.raster_gaussian_filter(r, 8.0, kernel_size=65).to_numpy()
    tc = vsr.raster_gaussian_filter(r, 8.0, kernel_size=65, precision="split_bf16").to_numpy()
    np.testing.assert_array_equal(auto, tc)
    a33 = vsr.raster_gaussian_filter(r, 4.0, kernel_size=33).to_numpy()
    f33 = vsr.raster_gaussian_filter(r, 4.0, kernel_size=33, precision="fp32").to_numpy()
    np.testing.assert_array_equal(a33, f33)


def test_split_bf16_gaussian_rejects_float_rasters(vsr):
    r = vsr.from_numpy(np.ones((40, 40), np.float32))
    with pytest.raises(Exception, match="tensor-core Gaussian"):
        vsr.raster_gaussian_filter(r, 8.0, kernel_size=65, precision="split_bf16")
