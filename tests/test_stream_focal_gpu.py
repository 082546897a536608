"""Streamed host-to-host focal passes (row strips with a halo of the window's
rows, copies overlapped on several streams) against the resident calls on
the whole raster: exact for the integer focal statistics (exact sums and
comparisons), within 1e-6 relative for the convolution and the Gaussian
(the kernels' per-tile sums start at other rows), NaN and nodata placement
exact.  Small strips force many strips, ragged last strips and halos that
reach the raster's own edges."""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _close(a, b, rel=1e-6):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    np.testing.assert_array_equal(np.isnan(a), np.isnan(b))
    m = ~np.isnan(b)
    scale = max(float(np.abs(b[m]).mean()) if m.any() else 1.0, 1e-30)
    assert (np.abs(a[m] - b[m]) <= rel * np.maximum(np.abs(b[m]), scale)).all()


@pytest.mark.parametrize("precision,k", [("fp32", 7), ("split", 31)])
def test_convolve_host_equals_resident(vsr, precision, k):
    from vsr_gb300 import stream

    rng = np.random.default_rng(k)
    d = (rng.random((301, 180)) * 10 + np.arange(301)[:, None] * 0.2).astype(np.float32)
    d[rng.random(d.shape) < 0.02] = -9999.0
    w = rng.random((k, k))
    w /= w.sum()
    r = vsr.from_numpy(d, nodata=-9999.0)
    got = stream.raster_convolve_host(r, w, precision=precision, strip_rows=37, n_streams=3)
    want = vsr.raster_convolve(r, w, precision=precision).to_numpy()
    assert got.nodata == -9999.0 and got.dtype == np.float64
    g = got.to_numpy()
    np.testing.assert_array_equal(g == -9999.0, want == -9999.0)
    _close(g, want)


def test_gaussian_host_equals_resident(vsr):
    from vsr_gb300 import stream

    rng = np.random.default_rng(2)
    u = rng.integers(1, 9000, (2, 260, 150)).astype(np.uint16)
    u[0, 100:105, 20:30] = 0
    r = vsr.from_numpy(u, nodata=0)
    for prec in ("split", "fp32"):
        got = stream.raster_gaussian_filter_host(r, 6.0, kernel_size=41, precision=prec, strip_rows=50).to_numpy()
        want = vsr.raster_gaussian_filter(r, 6.0, kernel_size=41, precision=prec).to_numpy()
        assert got.shape == u.shape
        np.testing.assert_array_equal(got == 0, want == 0)
        _close(got, want)


@pytest.mark.parametrize("stat", ["min", "max", "mean", "std", "range", "variety"])
def test_focal_host_equals_resident(vsr, stat):
    from vsr_gb300 import stream

    rng = np.random.default_rng(3)
    d = rng.integers(0, 40, (203, 97)).astype(np.int16)
    d[rng.random(d.shape) < 0.05] = -1
    r = vsr.from_numpy(d, nodata=-1)
    got = stream.raster_focal_host(r, stat, (3, 2), strip_rows=29).to_numpy()
    want = getattr(vsr, f"raster_focal_{stat}")(r, (3, 2)).to_numpy()
    if stat == "std":
        np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-13)
    else:
        np.testing.assert_array_equal(got, want)
