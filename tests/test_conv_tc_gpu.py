"""Split-BF16 tcgen05 convolution vs the float64 oracle.

Tolerances: the tensor-core path targets 2e-6 relative error against float64
on the trend-plus-noise workload (values 0-100, positive weights); with
nodata present the general convolution bound (1e-5 relative, of
max(|ref|, mean |input|)) applies.  Nodata and NaN placement must be exact.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _trend(shape, seed):
    rng = np.random.default_rng(seed)
    h, w = shape
    return (rng.random(shape) + np.arange(h * w).reshape(shape) * (100.0 / (h * w))).astype(np.float32)


def _rel_err(out, ref, data):
    scale = float(np.nanmean(np.abs(data)))
    m = ~np.isnan(ref)
    return np.abs(out[m] - ref[m]) / np.maximum(np.abs(ref[m]), scale)


def test_small_split_bf16_matches_oracle(vsr):
    d = _trend((150, 208), 1)
    w = np.random.default_rng(2).random((15, 15))
    w /= w.sum()
    out = vsr.raster_convolve(vsr.from_numpy(d), w, precision="split_bf16").to_numpy()
    ref = oracle.convolve_normalized(d, w, None)
    err = _rel_err(out, ref, d)
    assert err.max() <= 2e-6, err.max()


@pytest.mark.parametrize("k", [15, 31, 41])
def test_split_bf16_accuracy_vs_fp64(vsr, k):
    d = _trend((1031, 1212), k)
    w = np.random.default_rng(k).random((k, k))
    w /= w.sum()
    out = vsr.raster_convolve(vsr.from_numpy(d), w, precision="split_bf16").to_numpy()
    ref = oracle.convolve_normalized(d, w, None)
    err = _rel_err(out, ref, d)
    assert err.max() <= 2e-6, (k, err.max(), np.percentile(err, 99))


def test_split_bf16_gaussian_41(vsr, golden):
    arrays, _ = golden
    w = arrays["gaussian/s5.0_k41"]
    d = _trend((700, 516), 5)
    out = vsr.raster_convolve(vsr.from_numpy(d), w, precision="split_bf16").to_numpy()
    ref = oracle.convolve_normalized(d, w, None)
    assert _rel_err(out, ref, d).max() <= 2e-6


@pytest.mark.parametrize("nodata", [-9999.0, float("nan"), 0.0])
def test_split_bf16_nodata(vsr, nodata):
    rng = np.random.default_rng(7)
    d = _trend((300, 404), 9)
    d[rng.random(d.shape) < 0.02] = nodata
    d[:3, :5] = nodata
    w = rng.random((17, 15))
    w /= w.sum()
    out = vsr.raster_convolve(vsr.from_numpy(d, nodata=nodata), w, precision="split_bf16").to_numpy()
    ref = oracle.convolve_normalized(d, w, nodata)
    np.testing.assert_array_equal(np.isnan(out), np.isnan(ref))
    if not np.isnan(nodata):
        np.testing.assert_array_equal(out == nodata, ref == nodata)
    assert _rel_err(out, ref, d).max() <= 1e-5


def test_auto_selects_tensor_cores_for_large_kernels(vsr):
    d = _trend((256, 260), 3)
    w = np.random.default_rng(3).random((31, 31))
    w /= w.sum()
    r = vsr.from_numpy(d)
    a = vsr.raster_convolve(r, w).to_numpy()  # auto
    b = vsr.raster_convolve(r, w, precision="split_bf16").to_numpy()
    np.testing.assert_array_equal(a, b)
    c = vsr.raster_convolve(r, w, precision="fp32").to_numpy()
    assert np.abs(a - c).max() <= 1e-5 * 100


def test_split_bf16_rejects_unaligned_rows(vsr):
    d = _trend((64, 37), 4)  # 37 floats per row: not 16-byte aligned
    w = np.ones((15, 15)) / 225.0
    with pytest.raises(NotImplementedError, match="split-BF16"):
        vsr.raster_convolve(vsr.from_numpy(d), w, precision="split_bf16")
    # auto falls back to the FP32 kernel
    out = vsr.raster_convolve(vsr.from_numpy(d), w).to_numpy()
    np.testing.assert_allclose(out, oracle.convolve_normalized(d, w, None), rtol=1e-5)
