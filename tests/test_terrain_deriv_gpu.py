"""GPU parity of TRI / TPI / profile curvature vs the reference and the oracle.

The reference computes the three derivatives in float64
(algebra.py:3352-3445, kernels/focal.py:487-647).  libvsr evaluates 8/16-bit
and float32 DEMs in double-float FP32 (error-free differences, compensated
sums) and int32 / float64 DEMs in FP64, so the bound asserted here is float64
quality: |out - ref| <= 1e-12 * (|ref| + max |elevation|).  Border pixels and
the nodata dilation are compared exactly, NaN placement too.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

KINDS = ("tri", "tpi", "curvature")


def _assert_f64_quality(out, ref, data, name=""):
    out = np.asarray(out, np.float64)
    ref = np.asarray(ref, np.float64)
    np.testing.assert_array_equal(np.isnan(out), np.isnan(ref), err_msg=name)
    m = np.isfinite(ref)
    np.testing.assert_array_equal(out[~m & ~np.isnan(ref)], ref[~m & ~np.isnan(ref)], err_msg=name)
    z = np.asarray(data, np.float64)
    zmax = float(np.max(np.abs(z[np.isfinite(z)]), initial=1.0))
    err = np.abs(out[m] - ref[m])
    bound = 1e-12 * (np.abs(ref[m]) + zmax)
    assert (err <= bound).all(), f"{name}: max err {np.max(err, initial=0):.3e} (zmax {zmax})"


def test_matches_reference_golden(vsr, golden):
    """Every golden terrain case (float32, float64, int16, NaN nodata, 1x1 / 1xN /
    Nx1, rotated and zero affines) against the reference's own CPU outputs."""
    arrays, manifest = golden
    for case in manifest["terrain"]:
        name = case["name"]
        data = arrays[f"terrain/{name}/input"]
        dem = vsr.from_numpy(data, nodata=case["nodata"], affine=tuple(case["affine"]))
        res = vsr.raster_terrain_derivatives(dem)
        for k in KINDS:
            out = res[k].to_numpy()
            assert out.dtype == np.float64
            _assert_f64_quality(out, arrays[f"terrain/{name}/{k}"], data, f"{name} {k}")
            nd = case["deriv_nodata"]
            assert (np.isnan(nd) and np.isnan(res[k].nodata)) or res[k].nodata == nd


@pytest.mark.parametrize("dtype,nodata", [(np.float32, -9999.0), (np.uint16, 0), (np.float32, float("nan")),
                                          (np.int32, -1), (np.float64, None)])
def test_matches_oracle(vsr, dtype, nodata):
    rng = np.random.default_rng(5)
    h, w = 300, 257
    yy, xx = np.mgrid[0:h, 0:w]
    z = 1500 + 800 * np.sin(yy / 37.0) * np.cos(xx / 23.0) + rng.normal(0, 3, (h, w))
    if np.issubdtype(dtype, np.integer):
        z = np.round(z)
    d = z.astype(dtype)
    if nodata is not None:
        d[rng.random((h, w)) < 0.04] = nodata
    aff = (12.5, 0.0, 0.0, 0.0, -7.5, 0.0)
    res = vsr.raster_terrain_derivatives(vsr.from_numpy(d, nodata=nodata, affine=aff))
    for k in KINDS:
        ref, nd = oracle.terrain_derivative(d, aff, nodata, k)
        _assert_f64_quality(res[k].to_numpy(), ref, d, k)


def test_non_finite_values_propagate(vsr):
    """Without nodata, NaN and +-inf enter the arithmetic as in the reference; a
    non-finite corner leaves the curvature (which does not read corners) exact."""
    rng = np.random.default_rng(9)
    d = rng.uniform(100, 200, (40, 45)).astype(np.float32)
    d[10, 10] = np.nan
    d[20, 30] = np.inf
    d[30, 5] = -np.inf
    d[21, 31] = np.inf
    res = vsr.raster_terrain_derivatives(vsr.from_numpy(d))
    for k in KINDS:
        with np.errstate(invalid="ignore"):
            ref, _ = oracle.terrain_derivative(d, (1.0, 0, 0, 0, -1.0, 0), None, k)
        _assert_f64_quality(res[k].to_numpy(), ref, d, k)


def test_bands_and_float32_output(vsr):
    from vsr_gb300 import algebra

    rng = np.random.default_rng(3)
    stack = (1000 + rng.normal(0, 50, (2, 64, 70))).astype(np.float32)
    stack[:, 5, 5] = -9999.0
    r = vsr.from_numpy(stack, nodata=-9999.0, affine=(30.0, 0, 0, 0, -30.0, 0))
    t64 = [t.cpu().numpy() for t in algebra.terrain_derivatives(r)]
    t32 = [t.cpu().numpy() for t in algebra.terrain_derivatives(r, out_dtype=np.float32)]
    for a, b in zip(t64, t32):
        np.testing.assert_array_equal(b, a.astype(np.float32))
    for band in range(2):
        one = vsr.raster_terrain_derivatives(vsr.from_numpy(stack[band], nodata=-9999.0,
                                                            affine=(30.0, 0, 0, 0, -30.0, 0)))
        for k, a in zip(KINDS, t64):
            np.testing.assert_array_equal(one[k].to_numpy(), a[band])


def test_api_contract(vsr):
    d = np.arange(36, dtype=np.float32).reshape(6, 6)
    r = vsr.from_numpy(d)
    tri = vsr.raster_tri(r)
    assert tri.nodata == -9999.0 and tri.to_numpy().dtype == np.float64
    assert any(e.detail.startswith("gpu_terrain_TRI 6x6") for e in tri.diagnostics)
    assert any(e.detail.startswith("gpu_terrain_TPI") for e in vsr.raster_tpi(r).diagnostics)
    assert any(e.detail.startswith("gpu_terrain_curvature") for e in vsr.raster_curvature(r).diagnostics)
    # a plane: TPI and curvature 0 inside, TRI = mean |neighbour step|
    np.testing.assert_array_equal(vsr.raster_tpi(r).to_numpy()[1:-1, 1:-1], 0.0)
    np.testing.assert_array_equal(vsr.raster_curvature(r).to_numpy()[1:-1, 1:-1], 0.0)
    np.testing.assert_allclose(tri.to_numpy()[1:-1, 1:-1], (1 + 6 + 7 + 5 + 1 + 5 + 6 + 7) / 8.0)
    assert (tri.to_numpy()[0] == -9999.0).all()
    with pytest.raises(NotImplementedError):
        vsr.raster_tri(r, use_gpu=False)


@pytest.mark.parametrize("kind,data,centre", [
    ("tri", np.add.outer(np.arange(5.0), np.arange(1.0, 6.0)), 1.0),
    ("tpi", np.where(np.add.outer(np.abs(np.arange(5) - 2), np.abs(np.arange(5) - 2)) == 0, 10.0, 1.0), 9.0),
    ("curvature", np.array([[0, 0, 0, 0, 0], [0, 0, 1, 0, 0], [0, 1, 4, 1, 0], [0, 0, 1, 0, 0], [0, 0, 0, 0, 0]],
                           np.float64), 1200.0),
])
def test_reference_known_answers(vsr, kind, data, centre):
    """Reference tests/test_terrain_derivatives.py:116-139, 187-206, 255-278
    (float64 DEMs, unit cells), and the same DEMs as float32."""
    for dt in (np.float64, np.float32):
        r = vsr.from_numpy(data.astype(dt), affine=(1.0, 0.0, 0.0, 0.0, -1.0, 5.0))
        out = vsr.raster_terrain_derivatives(r)[kind].to_numpy()
        assert out[2, 2] == centre and out[0, 0] == -9999.0
