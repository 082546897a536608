"""Host-side API contract (no GPU): signatures, dtype rules, errors, buffers.

Restates the reference's CPU-checkable expectations for the focal path's
Python surface (src/vibespatial/raster/algebra.py, buffers.py).
"""

from __future__ import annotations

import inspect
import warnings

import numpy as np
import pytest

import vsr_gb300 as vsr
from vsr_gb300 import algebra


def test_signatures_match_reference():
    sig = inspect.signature(vsr.raster_slope)
    assert list(sig.parameters)[:2] == ["dem", "use_gpu"]
    sig = inspect.signature(vsr.raster_hillshade)
    p = sig.parameters
    assert (p["azimuth"].default, p["altitude"].default, p["z_factor"].default) == (315.0, 45.0, 1.0)
    assert p["use_gpu"].default is None


def test_use_gpu_false_raises_no_cpu_path():
    r = vsr.from_numpy(np.zeros((4, 4), np.float32))
    with pytest.raises(NotImplementedError, match="GPU only"):
        vsr.raster_slope(r, use_gpu=False)
    with pytest.raises(NotImplementedError):
        vsr.raster_hillshade(r, use_gpu=False)


def test_terrain_derivative_api_matches_reference():
    """raster_tri / raster_tpi / raster_curvature(dem, *, use_gpu=None)
    (algebra.py:3448-3525); output nodata = the raster's, else -9999
    (algebra.py:3376); GPU only."""
    for fn in (vsr.raster_tri, vsr.raster_tpi, vsr.raster_curvature):
        p = inspect.signature(fn).parameters
        assert list(p) == ["dem", "use_gpu"] and p["use_gpu"].default is None
        assert p["use_gpu"].kind is inspect.Parameter.KEYWORD_ONLY
    r = vsr.from_numpy(np.zeros((4, 4), np.float32))
    for fn in (vsr.raster_tri, vsr.raster_tpi, vsr.raster_curvature, vsr.raster_terrain_derivatives):
        with pytest.raises(NotImplementedError):
            fn(r, use_gpu=False)
    assert algebra.derivative_nodata(r) == -9999.0
    assert algebra.derivative_nodata(vsr.from_numpy(np.zeros((4, 4), np.int16), nodata=-32768)) == -32768.0
    assert np.isnan(algebra.derivative_nodata(vsr.from_numpy(np.zeros((4, 4), np.float32), nodata=float("nan"))))


def test_cellsize_rule():
    # |a|, |e|, 1.0 for zero; rotation ignored (algebra.py:2307-2308)
    assert algebra.cellsize((-2.0, 0.5, 0.0, 0.3, 3.0, 0.0)) == (2.0, 3.0)
    assert algebra.cellsize((0.0, 0, 0, 0, 0.0, 0)) == (1.0, 1.0)
    assert algebra.cellsize((30.0, 0, 0, 0, -30.0, 0)) == (30.0, 30.0)


def test_terrain_dtype_rule():
    f = algebra._terrain_out_dtype
    assert f(np.float32) == np.float32
    assert f(np.float64) == np.float64
    assert f(np.int16) == np.float64
    assert f(np.uint16) == np.float64
    assert f(np.float16) == np.float16


def test_nodata_kind():
    assert algebra.nodata_kind(vsr.from_numpy(np.zeros((2, 2), np.float32)))[0] == 0
    assert algebra.nodata_kind(vsr.from_numpy(np.zeros((2, 2), np.float32), nodata=-9999.0)) == (1, -9999.0)
    assert algebra.nodata_kind(vsr.from_numpy(np.zeros((2, 2), np.float32), nodata=float("nan")))[0] == 2


def test_from_numpy_contract():
    with pytest.raises(ValueError, match="2D or 3D"):
        vsr.from_numpy(np.zeros(5))
    with pytest.raises(ValueError, match="NaN"):
        vsr.from_numpy(np.zeros((2, 2), np.int16), nodata=float("nan"))
    r = vsr.from_numpy(np.zeros((3, 5, 7), np.uint16), nodata=0)
    assert (r.band_count, r.height, r.width, r.pixel_count) == (3, 5, 7, 35)
    assert r.diagnostics[-1].detail.startswith("from_numpy")
    assert r.residency == vsr.Residency.HOST


def test_nodata_mask_rules():
    d = np.array([[1.0, np.nan], [-9999.0, 2.0]], np.float32)
    np.testing.assert_array_equal(vsr.from_numpy(d, nodata=-9999.0).nodata_mask, [[False, False], [True, False]])
    np.testing.assert_array_equal(vsr.from_numpy(d, nodata=float("nan")).nodata_mask, [[False, True], [False, False]])
    r = vsr.from_numpy(np.zeros((2, 2), np.int16))
    r.nodata = float("nan")
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        assert not r.nodata_mask.any()
        assert any("NaN" in str(x.message) for x in w)


def test_from_band_stack_validation():
    a = vsr.from_numpy(np.zeros((4, 4), np.float32), nodata=-1.0)
    b = vsr.from_numpy(np.zeros((4, 4), np.float64), nodata=-1.0)
    c = vsr.from_numpy(np.zeros((4, 5), np.float32), nodata=-1.0)
    src = vsr.from_numpy(np.zeros((2, 4, 4), np.float32), nodata=-1.0)
    with pytest.raises(ValueError, match="empty"):
        vsr.OwnedRasterArray.from_band_stack([], source=src)
    with pytest.raises(ValueError, match="dtype mismatch"):
        vsr.OwnedRasterArray.from_band_stack([a, b], source=src)
    with pytest.raises(ValueError, match="shape mismatch"):
        vsr.OwnedRasterArray.from_band_stack([a, c], source=src)
    s = vsr.OwnedRasterArray.from_band_stack([a, vsr.from_numpy(np.ones((4, 4), np.float32), nodata=-1.0)], source=src)
    assert s.shape == (2, 4, 4) and s.nodata == -1.0


def test_bounds():
    r = vsr.from_numpy(np.zeros((10, 20), np.float32), affine=(2.0, 0.0, 100.0, 0.0, -3.0, 50.0))
    assert r.bounds == (100.0, 20.0, 140.0, 50.0)
