"""GPU parity of the focal statistics (min, max, std, range, variety) with the
oracle, which is pinned bit for bit to the reference's CPU functions
(algebra.py:3041-3164).

Tolerances: min, max, range and variety exact (NaN and nodata placement
included); std within 1e-12 relative plus 1e-12 of the data's magnitude
(8/16-bit rasters are summed exactly, floats in two float64 passes; the
reference sums in another order).
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

STATS = ("min", "max", "std", "range", "variety")


def _check(out, ref, data, stat, name=""):
    out = np.asarray(out, np.float64)
    ref = np.asarray(ref, np.float64)
    np.testing.assert_array_equal(np.isnan(out), np.isnan(ref), err_msg=f"{name} {stat} NaN placement")
    m = ~np.isnan(ref)
    if stat != "std":
        np.testing.assert_array_equal(out[m], ref[m], err_msg=f"{name} {stat}")
        return
    fin = np.asarray(data, np.float64)
    fin = fin[np.isfinite(fin)]
    scale = float(np.abs(fin).max()) if fin.size else 1.0
    err = np.abs(out[m] - ref[m])
    bound = 1e-12 * np.abs(ref[m]) + 1e-12 * max(scale, 1.0)
    assert (err <= bound).all(), f"{name} std max err {err.max():.3e}"


def _run(vsr, data, nodata, stat, radius, out_dtype=np.float64):
    r = vsr.from_numpy(data, nodata=nodata)
    fn = getattr(vsr, f"raster_focal_{stat}")
    return fn(r, radius, out_dtype=out_dtype)


def test_focal_stats_reference_golden(vsr, golden):
    """The reference's own CPU outputs, through the GPU."""
    arrays, manifest = golden
    for case in manifest["focal_mean"]:
        name = case["name"]
        data = arrays[f"focal_mean/{name}/input"]
        ry, rx = case["radius"]
        for stat in manifest["focal_stats"]:
            out = _run(vsr, data, case["nodata"], stat, (ry, rx))
            assert out.dtype == np.float64
            _check(out.to_numpy(), arrays[f"focal_{stat}/{name}/output"], data, stat, name)


def _data(dtype, shape, rng):
    if dtype == np.uint8:
        return rng.integers(0, 12, shape).astype(np.uint8)  # many repeats for variety
    if dtype == np.int16:
        return rng.integers(-300, 300, shape).astype(np.int16)
    if dtype == np.uint16:
        return rng.integers(0, 65535, shape).astype(np.uint16)
    if dtype == np.int32:
        return rng.integers(-(2**31), 2**31 - 1, shape, dtype=np.int64).astype(np.int32)
    base = np.linspace(1000.0, 1200.0, shape[0] * shape[1]).reshape(shape)
    return (base + rng.normal(0, 3, shape)).astype(dtype)


@pytest.mark.parametrize("dtype", [np.uint8, np.int16, np.uint16, np.int32, np.float32, np.float64])
@pytest.mark.parametrize("radius", [1, (2, 1), 3])
def test_focal_stats_dtypes_vs_oracle(vsr, dtype, radius):
    rng = np.random.default_rng(7 + np.dtype(dtype).itemsize)
    shape = (75, 131)
    d = _data(dtype, shape, rng)
    nodata = {np.uint8: 3, np.int16: -299, np.uint16: 5, np.int32: int(d[4, 4])}.get(dtype, -9999.0)
    if np.dtype(dtype).kind == "f":
        d[rng.random(shape) < 0.05] = nodata
    ry, rx = (radius, radius) if isinstance(radius, int) else radius
    for stat in STATS:
        for nd in (None, nodata):
            out = _run(vsr, d, nd, stat, radius).to_numpy()
            _check(out, oracle.focal_stat(d, ry, rx, nd, stat), d, stat, f"{np.dtype(dtype).name} nd={nd}")


def test_focal_stats_nan_and_inf(vsr):
    """NaN data propagates through min / max and is excluded by the others;
    +-inf data is excluded by min / max when it equals the placeholder."""
    rng = np.random.default_rng(11)
    d = rng.normal(0, 10, (40, 57)).astype(np.float32)
    d[rng.random(d.shape) < 0.04] = np.nan
    d[rng.random(d.shape) < 0.02] = np.inf
    d[rng.random(d.shape) < 0.02] = -np.inf
    d[10:14, 20:26] = np.inf  # windows holding only +inf
    for nd in (None, -9999.0, float("nan")):
        dd = d.copy()
        if nd is not None and not np.isnan(nd):
            dd[rng.random(d.shape) < 0.05] = nd
        for stat in STATS:
            out = _run(vsr, dd, nd, stat, 1).to_numpy()
            _check(out, oracle.focal_stat(dd, 1, 1, nd, stat), dd, stat, f"nd={nd}")


def test_focal_stats_all_nodata_and_thin_rasters(vsr):
    d = np.full((6, 9), -1.0, np.float32)
    for stat in STATS:
        out = _run(vsr, d, -1.0, stat, 2).to_numpy()
        np.testing.assert_array_equal(out, np.full(d.shape, -1.0))
    rng = np.random.default_rng(3)
    for shape in ((1, 70), (70, 1), (1, 1), (2, 3)):
        d = rng.integers(0, 5, shape).astype(np.int16)
        for stat in STATS:
            out = _run(vsr, d, None, stat, (2, 3)).to_numpy()
            _check(out, oracle.focal_stat(d, 2, 3, None, stat), d, stat, str(shape))


def test_focal_stats_large_radius_and_float32_output(vsr):
    rng = np.random.default_rng(5)
    d = rng.integers(0, 1000, (150, 170)).astype(np.uint16)
    d[rng.random(d.shape) < 0.1] = 0
    for stat in ("min", "max", "range", "std"):
        out = _run(vsr, d, 0, stat, (31, 17)).to_numpy()
        _check(out, oracle.focal_stat(d, 31, 17, 0, stat), d, stat, "r31x17")
    out = _run(vsr, d, 0, "variety", 7).to_numpy()
    _check(out, oracle.focal_stat(d, 7, 7, 0, "variety"), d, "variety", "r7")
    out32 = _run(vsr, d, 0, "range", 2, out_dtype=np.float32)
    assert out32.dtype == np.float32
    np.testing.assert_array_equal(out32.to_numpy(), oracle.focal_stat(d, 2, 2, 0, "range").astype(np.float32))


def test_focal_stats_radius_limits(vsr):
    r = vsr.from_numpy(np.zeros((10, 10), np.float32))
    with pytest.raises(NotImplementedError):
        vsr.raster_focal_variety(r, 8)
    with pytest.raises(NotImplementedError):
        vsr.raster_focal_min(r, 32)
    with pytest.raises(ValueError):
        vsr.raster_focal_min(r, -1)


def test_focal_stats_bands_one_launch(vsr):
    """A band stack in one launch equals each band on its own."""
    rng = np.random.default_rng(9)
    stack = rng.integers(0, 50, (3, 64, 80)).astype(np.int16)
    for stat in STATS:
        out = _run(vsr, stack, 7, stat, 2).to_numpy()
        assert out.shape == stack.shape
        for b in range(3):
            _check(out[b], oracle.focal_stat(stack[b], 2, 2, 7, stat), stack[b], stat, f"band {b}")


@pytest.mark.parametrize("dtype", [np.uint8, np.int16, np.uint16])
@pytest.mark.parametrize("r", [1, 2, 3, 4])
def test_focal_stats_register_resident_kernel(vsr, dtype, r):
    """8/16-bit rasters whose rows are aligned to 4 elements take the
    register-resident min / max / range and std kernels for square radii up
    to 4:
    120-column warp strips (ragged at 964 = 2 x 480 + 4 columns), 256-row
    strips, a raster narrower than a lane group, signed values; outputs equal
    to the oracle (float64 and float32).  The 8/16-bit std with a float32
    output is sqrt(n^2 var)/n rounded once to float32: within one float32 ulp
    of the float64 oracle, equal to it rounded on (nearly) every pixel."""
    rng = np.random.default_rng(100 * r + np.dtype(dtype).itemsize)
    lo, hi = {np.uint8: (0, 254), np.int16: (-32767, 32767), np.uint16: (0, 65534)}[dtype]
    nd = {np.uint8: 255, np.int16: -32768, np.uint16: 65535}[dtype]
    for shape in [(530, 964), (300, 1024), (9, 4)]:
        d = rng.integers(lo, hi, shape, endpoint=True).astype(dtype)
        d[rng.random(shape) < 0.03] = nd
        d[:12, :14] = nd  # empty windows
        for stat in ("min", "max", "range"):
            ref = oracle.focal_stat(d, r, r, nd, stat)
            _check(_run(vsr, d, nd, stat, r).to_numpy(), ref, d, stat, f"{shape} r{r}")
            out32 = _run(vsr, d, nd, stat, r, out_dtype=np.float32).to_numpy()
            np.testing.assert_array_equal(out32, ref.astype(np.float32), err_msg=f"{shape} r{r} {stat} f32")
        ref = oracle.focal_stat(d, r, r, nd, "std")
        _check(_run(vsr, d, nd, "std", r).to_numpy(), ref, d, "std", f"{shape} r{r}")
        out32 = _run(vsr, d, nd, "std", r, out_dtype=np.float32).to_numpy()
        r32 = ref.astype(np.float32)
        m = ~np.isnan(ref)
        np.testing.assert_array_equal(np.isnan(out32), np.isnan(r32))
        ulp = np.abs(out32[m].view(np.int32).astype(np.int64) - r32[m].view(np.int32).astype(np.int64))
        assert ulp.max() <= 1, f"{shape} r{r} std f32 ulp {ulp.max()}"
        assert (ulp == 0).mean() >= 0.9999
