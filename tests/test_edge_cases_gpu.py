"""Degenerate shapes through every public operation: empty rasters (0 rows
or 0 columns), a single pixel, a single row and a single column, against
the oracle where it is defined; the result keeps the input's shape."""

from __future__ import annotations

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

AFF = (10.0, 0.0, 0.0, 0.0, -10.0, 0.0)


def _ops(vsr):
    w = np.full((3, 3), 1.0 / 9.0)
    return {
        "slope": lambda r: vsr.raster_slope(r),
        "aspect": lambda r: vsr.raster_aspect(r),
        "hillshade": lambda r: vsr.raster_hillshade(r),
        "convolve": lambda r: vsr.raster_convolve(r, w),
        "gaussian": lambda r: vsr.raster_gaussian_filter(r, 1.0),
        "mean": lambda r: vsr.raster_focal_mean(r, 1),
        "min": lambda r: vsr.raster_focal_min(r, 1),
        "std": lambda r: vsr.raster_focal_std(r, 1),
        "variety": lambda r: vsr.raster_focal_variety(r, 1),
        "tri": lambda r: vsr.raster_tri(r),
    }


@pytest.mark.parametrize("shape", [(0, 5), (5, 0), (0, 0)])
def test_empty_rasters(vsr, shape):
    r = vsr.from_numpy(np.zeros(shape, np.float32), nodata=-9999.0, affine=AFF)
    for name, op in _ops(vsr).items():
        out = op(r).to_numpy()
        assert out.shape == shape, name


@pytest.mark.parametrize("shape", [(1, 1), (1, 9), (9, 1), (2, 2)])
def test_tiny_rasters_match_the_oracle(vsr, shape):
    rng = np.random.default_rng(sum(shape))
    d = (100 + rng.normal(0, 5, shape)).astype(np.float32)
    r = vsr.from_numpy(d, nodata=-9999.0, affine=AFF)
    ops = _ops(vsr)
    s = ops["slope"](r).to_numpy().astype(np.float64)
    rs, ra = oracle.slope_aspect(d, AFF, -9999.0)
    assert np.abs(s - rs).max() <= 1e-4
    a = ops["aspect"](r).to_numpy().astype(np.float64)
    da = np.abs(a - ra)
    assert np.minimum(da, 360 - da).max() <= 1e-4
    h = ops["hillshade"](r).to_numpy().astype(int)
    rh, _ = oracle.hillshade(d, AFF, -9999.0)
    assert np.abs(h - rh.astype(int)).max() <= 1
    c = ops["convolve"](r).to_numpy()
    np.testing.assert_allclose(c, oracle.convolve_normalized(d, np.full((3, 3), 1.0 / 9.0), -9999.0), rtol=1e-6)
    g = ops["gaussian"](r).to_numpy()
    np.testing.assert_allclose(g, oracle.convolve_normalized(d, oracle.gaussian_weights(1.0), -9999.0), rtol=1e-6)
    np.testing.assert_allclose(ops["mean"](r).to_numpy(), oracle.focal_mean(d, 1, 1, -9999.0), rtol=1e-12)
    for stat in ("min", "std", "variety"):
        np.testing.assert_allclose(ops[stat](r).to_numpy(), oracle.focal_stat(d, 1, 1, -9999.0, stat), rtol=1e-12,
                                   atol=1e-12, err_msg=stat)
    t, _ = oracle.terrain_derivative(d, AFF, -9999.0, oracle.TRI)
    np.testing.assert_allclose(ops["tri"](r).to_numpy(), t, rtol=1e-12, atol=1e-9)


def test_all_nodata_raster(vsr):
    d = np.full((20, 33), -9999.0, np.float32)
    r = vsr.from_numpy(d, nodata=-9999.0, affine=AFF)
    ops = _ops(vsr)
    for name in ("slope", "aspect", "convolve", "gaussian", "mean", "min"):
        np.testing.assert_array_equal(ops[name](r).to_numpy(), -9999.0, err_msg=name)
    np.testing.assert_array_equal(ops["hillshade"](r).to_numpy(), 0)
