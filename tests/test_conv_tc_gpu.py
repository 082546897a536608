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


def test_split_bf16_unaligned_rows_and_float64_output(vsr):
    d = _trend((131, 37), 4)  # 37 floats per row: rows not 16-byte aligned
    w = np.random.default_rng(4).random((15, 19))
    w /= w.sum()
    ref = oracle.convolve_normalized(d, w, None)
    out = vsr.raster_convolve(vsr.from_numpy(d), w, precision="split_bf16").to_numpy()
    assert _rel_err(out, ref, d).max() <= 2e-6
    out64 = vsr.raster_convolve(vsr.from_numpy(d), w, precision="split_bf16", out_dtype=np.float64).to_numpy()
    assert out64.dtype == np.float64
    assert _rel_err(out64, ref, d).max() <= 2e-6


def test_split_bf16_nan_and_inf_poison_without_nodata(vsr):
    d = _trend((260, 300), 11)
    d[40, 50] = np.nan
    d[200, 7] = np.inf
    d[5, 290] = -np.inf
    w = np.random.default_rng(11).random((21, 17))
    w /= w.sum()
    out = vsr.raster_convolve(vsr.from_numpy(d), w, precision="split_bf16").to_numpy()
    ref = oracle.convolve_normalized(d, w, None)
    # NaN windows, and the signed infinities of windows holding +-inf, exactly
    np.testing.assert_array_equal(np.isnan(out), np.isnan(ref))
    np.testing.assert_array_equal(np.isposinf(out), np.isposinf(ref))
    np.testing.assert_array_equal(np.isneginf(out), np.isneginf(ref))
    assert np.isposinf(ref).any() and np.isneginf(ref).any()
    f = np.isfinite(ref)
    assert _rel_err(out[f], ref[f], d[np.isfinite(d)]).max() <= 2e-6


def test_split_bf16_mixed_sign_weights(vsr):
    from scipy.ndimage import correlate

    d = _trend((300, 333), 12)
    w = np.random.default_rng(12).random((25, 25))
    w[:, 13:] -= 0.9  # window sums > 0 inside, <= 0 where the border cuts off the positive half
    r = vsr.from_numpy(d, nodata=-9999.0)
    out = vsr.raster_convolve(r, w, precision="split_bf16").to_numpy()
    ref = oracle.convolve_normalized(d, w, -9999.0)
    # windows whose weight sum is <= 0 take the nodata value, as in the reference
    np.testing.assert_array_equal(out == -9999.0, ref == -9999.0)
    assert (ref == -9999.0).any() and (ref != -9999.0).any()
    m = ref != -9999.0
    # The split weights w' = bf16(w) + bf16(w - bf16(w)) keep 16 significant
    # bits (|w' - w| <= 2^-17 |w|) and num and den share them, so the result
    # is the w'-weighted mean: it moves from the w-weighted one by at most
    # 2^-17 sum |w| |d - out| / |sum w|, which a near-cancelling weight sum
    # amplifies (the plain FP32 kernel stays far below; AUTO keeps kernels
    # with sum |w| > 4 |sum w| on it).
    aw = np.abs(w)
    den = correlate(np.ones(d.shape), w, mode="constant", cval=0.0)
    bound = (correlate(np.abs(d).astype(np.float64), aw, mode="constant", cval=0.0)
             + correlate(np.ones(d.shape), aw, mode="constant", cval=0.0) * np.abs(ref)) / np.abs(den)
    assert (np.abs(out[m] - ref[m]) <= 2.0 ** -16 * bound[m]).all()
    fp32 = vsr.raster_convolve(r, w, precision="fp32").to_numpy()
    assert (np.abs(fp32[m] - ref[m]) <= 2.0 ** -20 * bound[m]).all()
    np.testing.assert_array_equal(vsr.raster_convolve(r, w).to_numpy(), fp32)
