"""GPU parity of normalised convolution, Gaussian and focal mean vs the oracle.

Tolerances: convolution and Gaussian within 1e-5 relative of the float64
oracle (the path's stated bound) -- measured as |out - ref| <= 1e-5 * max(|ref|,
scale) with ``scale`` the mean |value| of the input, so that outputs that
cancel to ~0 are judged against the data's magnitude; nodata / NaN placement
exact.  Focal mean: integer rasters exactly rounded (sums are exact), float
rasters within 1e-12 relative (compensated float32 sums).
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

REL = 1e-5


def _assert_close(out, ref, data, nodata, rel=REL):
    out = np.asarray(out, np.float64)
    ref = np.asarray(ref, np.float64)
    np.testing.assert_array_equal(np.isnan(out), np.isnan(ref))
    m = ~np.isnan(ref)
    if nodata is not None and not np.isnan(nodata):
        np.testing.assert_array_equal(out[m] == nodata, ref[m] == nodata)
    scale = float(np.nanmean(np.abs(np.asarray(data, np.float64)))) or 1.0
    err = np.abs(out[m] - ref[m])
    bound = rel * np.maximum(np.abs(ref[m]), scale)
    assert (err <= bound).all(), f"max rel err {np.max(err / np.maximum(np.abs(ref[m]), scale)):.3e}"


@pytest.mark.parametrize("shape,k,nodata", [
    ((37, 53), (3, 3), None), ((64, 128), (5, 5), -9999.0), ((129, 257), (15, 15), None),
    ((100, 300), (31, 31), -9999.0), ((70, 90), (7, 3), float("nan")), ((33, 40), (2, 4), None),
    ((1, 50), (3, 3), None), ((50, 1), (5, 5), -1.0), ((200, 150), (41, 41), None), ((65, 70), (65, 65), 0.0),
])
def test_convolve_vs_oracle(vsr, shape, k, nodata):
    rng = np.random.default_rng(sum(shape) + k[0])
    d = (rng.random(shape) + np.linspace(0, 100, shape[0] * shape[1]).reshape(shape)).astype(np.float32)
    if nodata is not None:
        d[rng.random(shape) < 0.03] = nodata
    w = rng.random(k)
    w /= w.sum()
    r = vsr.from_numpy(d, nodata=nodata)
    out = vsr.raster_convolve(r, w, precision="fp32")
    assert out.dtype == np.float64
    assert out.nodata == nodata or (nodata != nodata and out.nodata != out.nodata)
    _assert_close(out.to_numpy(), oracle.convolve_normalized(d, w, nodata), d, nodata)


def test_convolve_signed_and_zero_sum_kernels(vsr):
    rng = np.random.default_rng(4)
    d = rng.uniform(-10, 10, (40, 60)).astype(np.float32)
    for w in (np.array([[1.0, 0.0, -1.0]]), rng.uniform(-1, 1, (5, 5)), np.ones((1, 1))):
        out = vsr.raster_convolve(vsr.from_numpy(d), w, precision="fp32").to_numpy()
        ref = oracle.convolve_normalized(d, w, None)
        # signed kernels cancel: errors measured against the data's magnitude
        np.testing.assert_allclose(out, ref, rtol=1e-4, atol=1e-4 * np.abs(d).mean())


def test_convolve_known_answers(vsr):
    """Reference tests/test_raster_algebra.py:372-418, through the GPU path."""
    d = np.arange(30, dtype=np.float32).reshape(5, 6)
    np.testing.assert_array_equal(vsr.raster_convolve(vsr.from_numpy(d), np.ones((1, 1))).to_numpy(), d)
    ones = vsr.from_numpy(np.ones((8, 8), np.float32))
    np.testing.assert_allclose(vsr.raster_convolve(ones, np.ones((3, 3)) / 9.0).to_numpy(), 1.0, rtol=1e-6)
    with pytest.raises(ValueError, match="kernel must be 2D"):
        vsr.raster_convolve(ones, np.ones(3))
    imp = np.zeros((11, 11), np.float32)
    imp[5, 5] = 100.0
    g = vsr.raster_gaussian_filter(vsr.from_numpy(imp), 1.0).to_numpy()
    assert g[5, 5] < 100.0 and g[5, 6] > 0.0 and g[4, 5] > 0.0
    with pytest.raises(ValueError, match="sigma must be positive"):
        vsr.raster_gaussian_filter(ones, 0.0)
    assert any(e.detail.startswith("gpu_convolve") for e in vsr.raster_convolve(ones, np.ones((3, 3))).diagnostics)


@pytest.mark.parametrize("sigma,ks,nodata", [(1.0, 5, None), (1.0, 5, float("nan")), (1.0, None, -9999.0),
                                             (2.5, 8, None), (5.0, 41, -9999.0), (3.0, None, 0.0),
                                             (8.0, 65, -9999.0)])
def test_gaussian_vs_oracle(vsr, golden, sigma, ks, nodata):
    arrays, manifest = golden
    rng = np.random.default_rng(int(sigma * 10))
    shape = (150, 210)
    d = (rng.random(shape) * 5 + np.linspace(0, 100, shape[0] * shape[1]).reshape(shape)).astype(np.float32)
    if nodata is not None:
        d[rng.random(shape) < 0.02] = nodata
    # the reference's own weights for this (sigma, kernel_size)
    key = f"gaussian/s{sigma}_k{ks}"
    w = arrays[key] if key in arrays.files else oracle.gaussian_weights(sigma, ks)
    ref = oracle.convolve_normalized(d, w, nodata)
    out = vsr.raster_gaussian_filter(vsr.from_numpy(d, nodata=nodata), sigma, kernel_size=ks, precision="fp32")
    _assert_close(out.to_numpy(), ref, d, nodata)


def test_gaussian_multiband_equals_per_band(vsr):
    rng = np.random.default_rng(1)
    stack = rng.random((3, 40, 70)).astype(np.float32)
    out = vsr.raster_gaussian_filter(vsr.from_numpy(stack), 1.0, kernel_size=5).to_numpy()
    for b in range(3):
        ob = vsr.raster_gaussian_filter(vsr.from_numpy(stack[b]), 1.0, kernel_size=5).to_numpy()
        np.testing.assert_array_equal(out[b], ob)


def test_focal_mean_golden(vsr, golden):
    arrays, manifest = golden
    for case in manifest["focal_mean"]:
        name = case["name"]
        data = arrays[f"focal_mean/{name}/input"]
        ref = arrays[f"focal_mean/{name}/output"]
        out = vsr.raster_focal_mean(vsr.from_numpy(data, nodata=case["nodata"]), tuple(case["radius"])).to_numpy()
        assert out.dtype == np.float64
        np.testing.assert_allclose(out, ref, rtol=1e-12, atol=1e-12, err_msg=name)


@pytest.mark.parametrize("dtype,nodata,radius", [(np.uint16, 0, 3), (np.float32, -9999.0, (1, 2)),
                                                 (np.float32, float("nan"), 2), (np.int16, -32768, 1),
                                                 (np.float64, None, 3), (np.uint8, 255, (2, 0))])
def test_focal_mean_vs_oracle(vsr, dtype, nodata, radius):
    rng = np.random.default_rng(5)
    shape = (97, 301)
    if np.issubdtype(dtype, np.integer):
        d = rng.integers(0, 250 if dtype == np.uint8 else 10000, shape).astype(dtype)
    else:
        d = rng.uniform(-100, 4000, shape).astype(dtype)
    if nodata is not None:
        d[rng.random(shape) < 0.05] = nodata
    ry, rx = (radius, radius) if isinstance(radius, int) else radius
    out = vsr.raster_focal_mean(vsr.from_numpy(d, nodata=nodata), radius).to_numpy()
    ref = oracle.focal_mean(d, ry, rx, nodata)
    if np.issubdtype(dtype, np.integer):
        np.testing.assert_array_equal(out, ref)  # exact sums, one float64 division
    else:
        np.testing.assert_allclose(out, ref, rtol=1e-12, atol=1e-9)


def test_focal_mean_known_answer(vsr):
    """Reference tests/test_focal_stats.py:113-127: 1..25 5x5, centre mean 13."""
    d = np.arange(1, 26, dtype=np.float64).reshape(5, 5)
    out = vsr.raster_focal_mean(vsr.from_numpy(d), 1).to_numpy()
    assert out[2, 2] == 13.0
    assert any(e.detail.startswith("gpu_focal_mean") for e in vsr.raster_focal_mean(vsr.from_numpy(d), 1).diagnostics)


@pytest.mark.parametrize("dtype,r", [(np.uint16, 3), (np.int16, 7), (np.uint8, 5), (np.uint16, 1),
                                     (np.int16, 4), (np.uint8, 2), (np.uint16, 4), (np.int16, 2)])
def test_focal_mean_integer_sliding_window(vsr, dtype, r):
    """Square windows on 8/16-bit rasters (the packed sliding-window kernels):
    several 256-row strips and column blocks with ragged edges; an odd row
    pitch (the shared-memory kernel, no paired loads) and pitches that are
    multiples of 4 (the register-resident kernel for radii up to 4: 120-column
    warp strips, 480-column blocks, ragged at 964 = 2 x 480 + 4); exact
    float64 means and correctly rounded float32 means."""
    rng = np.random.default_rng(r)
    lo, hi = {np.uint16: (0, 65535), np.int16: (-32767, 32767), np.uint8: (0, 254)}[dtype]
    nd = {np.uint16: 0, np.int16: -32768, np.uint8: 255}[dtype]
    for shape in [(600, 389), (300, 1024), (530, 964), (9, 4)]:
        d = rng.integers(lo, hi, shape, endpoint=True).astype(dtype)
        d[rng.random(shape) < 0.03] = nd
        d[:20, :30] = nd  # a window with no valid value
        ref = oracle.focal_mean(d, r, r, nd)
        r_ = vsr.from_numpy(d, nodata=nd)
        np.testing.assert_array_equal(vsr.raster_focal_mean(r_, r).to_numpy(), ref)
        out32 = vsr.raster_focal_mean(r_, r, out_dtype=np.float32).to_numpy()
        np.testing.assert_array_equal(out32, ref.astype(np.float32))


def test_focal_mean_multiband_uint16_equals_per_band(vsr):
    from vsr_gb300 import algebra

    rng = np.random.default_rng(11)
    stack = rng.integers(0, 10000, (3, 270, 300)).astype(np.uint16)
    stack[rng.random(stack.shape) < 0.03] = 0
    r = vsr.from_numpy(stack, nodata=0)
    allb = algebra.focal_mean_bands(r, 3, 3, out_dtype=np.float32).cpu().numpy()
    for i in range(3):
        np.testing.assert_array_equal(allb[i], oracle.focal_mean(stack[i], 3, 3, 0).astype(np.float32))


@pytest.mark.parametrize("k", [35, 49, 79])
def test_strip_gaussian_kernel_sizes(vsr, k):
    """The strip kernel's ring depth and output-row groups depend on k: the
    smallest strip size, a mid size and the largest Gaussian (run-time tap
    loops), on 1100 rows (two full 512-row segments and a 76-row one whose
    last output group holds 12 rows) and two 128-column strips."""
    rng = np.random.default_rng(k)
    shape = (1100, 200)
    d = rng.integers(1, 10000, shape).astype(np.uint16)
    d[rng.random(shape) < 0.03] = 0
    sigma = k / 8.0
    w = oracle.gaussian_weights(sigma, k)
    assert w.shape == (k, k)
    ref = oracle.convolve_normalized(d, w, 0)
    out = vsr.raster_gaussian_filter(vsr.from_numpy(d, nodata=0), sigma, kernel_size=k, precision="fp32").to_numpy()
    _assert_close(out, ref, d, 0)


@pytest.mark.parametrize("dtype,nodata", [(np.float32, -9999.0), (np.uint16, 0), (np.float32, float("nan"))])
def test_large_gaussian_strip_segments(vsr, dtype, nodata):
    """sigma 8, 65 x 65 on a raster taller than one 512-row segment and wider
    than one 128-column strip (the ring and segment seams), float32 output."""
    from vsr_gb300 import algebra

    rng = np.random.default_rng(65)
    shape = (1100, 300)
    if dtype == np.uint16:
        d = rng.integers(0, 10000, shape).astype(dtype)
    else:
        d = (rng.random(shape) * 5 + np.linspace(0, 100, shape[0] * shape[1]).reshape(shape)).astype(dtype)
    d[rng.random(shape) < 0.02] = nodata
    w = oracle.gaussian_weights(8.0, 65)
    ref = oracle.convolve_normalized(d, w, nodata)
    r = vsr.from_numpy(d, nodata=nodata)
    out = vsr.raster_gaussian_filter(r, 8.0, kernel_size=65, precision="fp32").to_numpy()
    _assert_close(out, ref, d, nodata)
    out32 = algebra.gaussian_bands(r, 8.0, 65, precision="fp32", out_dtype=np.float32).cpu().numpy()[0]
    _assert_close(out32.astype(np.float64), ref, d, nodata)
