"""Pin the oracle against golden vectors produced by the reference's own CPU code.

The fixtures come from tests/golden/make_golden.py, which runs
vibespatial-raster 0.1.7's ``_cpu_slope_aspect`` / ``_hillshade_cpu`` /
``_focal_mean_cpu`` / ``_focal_*_cpu`` (min, max, std, range, variety) /
``_terrain_derivative_cpu`` and captures the Gaussian weights it builds.  CPU only.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle


def _terrain(golden):
    arrays, manifest = golden
    for case in manifest["terrain"]:
        yield case, arrays


def test_oracle_slope_aspect_matches_reference(golden):
    arrays, manifest = golden
    for case in manifest["terrain"]:
        name = case["name"]
        data = arrays[f"terrain/{name}/input"]
        nodata = case["nodata"]
        s, a = oracle.slope_aspect(data, case["affine"], nodata)
        dt = oracle.terrain_out_dtype(data.dtype)
        assert str(dt) == case["slope_dtype"], name
        ref_s = arrays[f"terrain/{name}/slope"]
        ref_a = arrays[f"terrain/{name}/aspect"]
        # identical float64 arithmetic -> bit-identical after the same cast
        np.testing.assert_array_equal(s.astype(dt), ref_s, err_msg=name)
        np.testing.assert_array_equal(a.astype(dt), ref_a, err_msg=name)


def test_oracle_terrain_derivatives_match_reference(golden):
    """TRI, TPI and profile curvature bit for bit against the reference's
    ``_terrain_derivative_cpu`` (borders and dilated nodata set to the raster's
    nodata, else -9999)."""
    arrays, manifest = golden
    for case in manifest["terrain"]:
        name = case["name"]
        data = arrays[f"terrain/{name}/input"]
        for kind in (oracle.TRI, oracle.TPI, oracle.CURVATURE):
            with np.errstate(invalid="ignore"):
                out, nd = oracle.terrain_derivative(data, case["affine"], case["nodata"], kind)
            np.testing.assert_array_equal(out, arrays[f"terrain/{name}/{kind}"], err_msg=f"{name} {kind}")
            ref_nd = case["deriv_nodata"]
            assert (np.isnan(nd) and np.isnan(ref_nd)) or nd == ref_nd, name


def test_oracle_hillshade_matches_reference(golden):
    arrays, manifest = golden
    for case in manifest["terrain"]:
        name = case["name"]
        data = arrays[f"terrain/{name}/input"]
        for k, hp in enumerate(manifest["hillshade_params"]):
            out, nd = oracle.hillshade(data, case["affine"], case["nodata"], **hp)
            ref = arrays[f"terrain/{name}/hillshade{k}"]
            assert out.dtype == np.uint8
            assert nd == case["hillshade_nodata"], name
            if case["nodata"] is not None and np.isnan(case["nodata"]):
                # NaN -> uint8 is platform-defined in numpy, but every such
                # pixel lies inside the dilated nodata ring and is set to 0.
                pass
            np.testing.assert_array_equal(out, ref, err_msg=f"{name} hs{k}")


def test_oracle_focal_mean_matches_reference(golden):
    arrays, manifest = golden
    for case in manifest["focal_mean"]:
        name = case["name"]
        data = arrays[f"focal_mean/{name}/input"]
        ry, rx = case["radius"]
        out = oracle.focal_mean(data, ry, rx, case["nodata"])
        ref = arrays[f"focal_mean/{name}/output"]
        np.testing.assert_allclose(out, ref, rtol=1e-13, atol=1e-12, err_msg=name)


def test_oracle_focal_statistics_match_reference(golden):
    """min / max / range / variety bit for bit, std within 1e-13 relative
    (summation order), against the reference's ``_focal_*_cpu``."""
    arrays, manifest = golden
    for case in manifest["focal_mean"]:
        name = case["name"]
        data = arrays[f"focal_mean/{name}/input"]
        ry, rx = case["radius"]
        for stat in manifest["focal_stats"]:
            out = oracle.focal_stat(data, ry, rx, case["nodata"], stat)
            ref = arrays[f"focal_{stat}/{name}/output"]
            if stat == "std":
                np.testing.assert_array_equal(np.isnan(out), np.isnan(ref), err_msg=name)
                np.testing.assert_allclose(out, ref, rtol=1e-13, atol=0, err_msg=name)
            else:
                np.testing.assert_array_equal(out, ref, err_msg=f"{name} {stat}")


def test_oracle_gaussian_weights_match_reference(golden):
    arrays, manifest = golden
    for g in manifest["gaussian"]:
        w = oracle.gaussian_weights(g["sigma"], g["kernel_size"])
        np.testing.assert_array_equal(w, arrays[g["key"]], err_msg=g["key"])
    for sigma, msg in manifest["gaussian_errors"]:
        with pytest.raises(ValueError, match="sigma must be positive"):
            oracle.gaussian_weights(sigma)
        assert "sigma must be positive" in msg


@pytest.mark.parametrize("shape,k,nodata", [((9, 11), (3, 3), None), ((7, 13), (5, 3), -9999.0),
                                             ((6, 5), (2, 4), -1.0), ((5, 8), (7, 7), float("nan")),
                                             ((1, 9), (3, 5), None), ((4, 4), (1, 1), -9999.0)])
def test_convolve_oracle_matches_literal_kernel_loop(shape, k, nodata):
    rng = np.random.default_rng(3)
    d = rng.uniform(-3, 10, shape).astype(np.float32)
    if nodata is not None:
        d[rng.random(shape) < 0.2] = nodata
    w = rng.uniform(-0.2, 1.0, k)
    a = oracle.convolve_normalized(d, w, nodata)
    b = oracle.convolve_normalized_loop(d, w, nodata)
    np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-12)


def test_convolve_known_answers():
    """tests/test_raster_algebra.py:372-418 of the reference, restated."""
    d = np.arange(20, dtype=np.float32).reshape(4, 5)
    np.testing.assert_array_equal(oracle.convolve_normalized(d, np.ones((1, 1)), None), d)
    ones = np.ones((6, 6), np.float32)
    np.testing.assert_allclose(oracle.convolve_normalized(ones, np.ones((3, 3)) / 9.0, None), 1.0)
    imp = np.zeros((11, 11), np.float32)
    imp[5, 5] = 100.0
    g = oracle.convolve_normalized(imp, oracle.gaussian_weights(1.0), None)
    assert g[5, 5] < 100.0 and g[5, 6] > 0.0 and g[4, 5] > 0.0
    # a zero-sum kernel has no positive weight sum inside the raster -> nodata
    # value 0.0; on the right border the -1 tap falls outside and is skipped,
    # leaving weight sum 1 and value 1.
    z = oracle.convolve_normalized(ones, np.array([[1.0, 0.0, -1.0]]), None)
    np.testing.assert_array_equal(z[:, :-1], 0.0)
    np.testing.assert_array_equal(z[:, -1], 1.0)


# Known answers of the reference's own terrain-derivative tests
# (tests/test_terrain_derivatives.py:116-139, 187-206, 255-278): 5x5 DEMs,
# unit cells, value at the centre pixel.
TERRAIN_KNOWN_ANSWERS = [
    ("tri", np.add.outer(np.arange(5.0), np.arange(1.0, 6.0)), 1.0),
    ("tpi", np.where(np.add.outer(np.abs(np.arange(5) - 2), np.abs(np.arange(5) - 2)) == 0, 10.0, 1.0), 9.0),
    ("curvature", np.array([[0, 0, 0, 0, 0], [0, 0, 1, 0, 0], [0, 1, 4, 1, 0], [0, 0, 1, 0, 0], [0, 0, 0, 0, 0]],
                           np.float64), 1200.0),
]


@pytest.mark.parametrize("kind,data,centre", TERRAIN_KNOWN_ANSWERS)
def test_oracle_terrain_known_answers(kind, data, centre):
    out, nd = oracle.terrain_derivative(data, (1.0, 0.0, 0.0, 0.0, -1.0, 5.0), None, kind)
    assert out[2, 2] == centre and nd == -9999.0 and out[0, 0] == nd
