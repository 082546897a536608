"""GeoTIFF decode on the GPU (vsr_gb300.io.read_raster): every layout the
reader accepts round-trips bit for bit (strips and tiles with partial edge
tiles, uncompressed and DEFLATE, predictors 1 / 2 / 3, both byte orders,
classic and BigTIFF, interleaved and planar samples), windows and band
selections equal slices of the full read with the window's affine, and the
result feeds the stencils directly.  The files come from the test writer
(tests/tiff_writer.py); the reference's own reader needs rasterio or
nvimgcodec, neither of which is available here, so these are property
tests of the TIFF format rather than a comparison with the reference."""

from __future__ import annotations

import itertools

import numpy as np
import pytest

from tiff_writer import write_geotiff

pytestmark = pytest.mark.gpu

CASES = []
for dt, tile, pred, be, planar, comp in itertools.product(
        (np.uint8, np.int16, np.uint16, np.int32, np.float32, np.float64), (None, (32, 16)), (1, 2, 3),
        (False, True), (False, True), (False, True)):
    if (pred == 3) != (np.dtype(dt).kind == "f") and pred != 1:
        continue
    CASES.append((dt, tile, pred, be, planar, comp))


def _data(dt, shape, rng):
    if np.dtype(dt).kind == "f":
        return (rng.normal(1000, 300, shape)).astype(dt)
    info = np.iinfo(dt)
    return rng.integers(info.min, info.max, shape, endpoint=True, dtype=np.int64).astype(dt)


@pytest.mark.parametrize("dt,tile,pred,be,planar,comp", CASES)
def test_round_trip(vsr, tmp_path, dt, tile, pred, be, planar, comp):
    from vsr_gb300 import io

    rng = np.random.default_rng(len(CASES))
    d = _data(dt, (3, 45, 77), rng)
    p = tmp_path / "r.tif"
    write_geotiff(p, d, tile=tile, rows_per_strip=7, predictor=pred, big_endian=be, planar=planar, compress=comp)
    r = io.read_raster(p)
    out = r.to_numpy()
    assert out.dtype == np.dtype(dt) and out.shape == d.shape
    np.testing.assert_array_equal(out.view(f"u{out.dtype.itemsize}"), d.view(f"u{d.dtype.itemsize}"))
    assert r.affine == (10.0, 0.0, 500000.0, 0.0, -10.0, 4000000.0)
    assert r.crs == "EPSG:32633"


def test_bigtiff_single_band_with_nodata(vsr, tmp_path):
    from vsr_gb300 import io

    d = np.arange(300 * 200, dtype=np.float32).reshape(300, 200)
    d[5, 7] = -9999.0
    p = tmp_path / "b.tif"
    write_geotiff(p, d, tile=(64, 64), bigtiff=True, compress=True, predictor=3, nodata=-9999)
    r = io.read_raster(p, residency=vsr.Residency.DEVICE)
    assert r.residency is vsr.Residency.DEVICE
    assert r.to_numpy().shape == (300, 200)
    np.testing.assert_array_equal(r.to_numpy(), d)
    assert r.nodata == -9999.0
    assert any("read_raster backend=vsr_gpu" in e.detail for e in r.diagnostics)


def test_window_and_bands(vsr, tmp_path):
    from vsr_gb300 import io

    rng = np.random.default_rng(1)
    d = rng.integers(0, 60000, (4, 130, 170)).astype(np.uint16)
    for planar in (False, True):
        p = tmp_path / f"w{planar}.tif"
        write_geotiff(p, d, tile=(48, 32), planar=planar, compress=True, predictor=2,
                      affine=(2.0, 0.0, 100.0, 0.0, -3.0, 900.0))
        w = io.RasterWindow(col_off=37, row_off=21, width=90, height=77)
        r = io.read_raster(p, window=w, bands=[4, 2])
        np.testing.assert_array_equal(r.to_numpy(), d[[3, 1], 21:98, 37:127])
        assert r.affine == (2.0, 0.0, 100.0 + 37 * 2.0, 0.0, -3.0, 900.0 - 21 * 3.0)
        one = io.read_raster(p, bands=[3])
        np.testing.assert_array_equal(one.to_numpy(), d[2])


def test_decoded_raster_feeds_the_stencils(vsr, tmp_path):
    import oracle
    from vsr_gb300 import io

    yy, xx = np.mgrid[0:96, 0:128]
    dem = (400 + 30 * np.sin(yy / 7.0) + 20 * np.cos(xx / 5.0)).astype(np.float32)
    p = tmp_path / "dem.tif"
    write_geotiff(p, dem, tile=(64, 32), compress=True, predictor=3, affine=(30.0, 0.0, 0.0, 0.0, -30.0, 0.0),
                  nodata=-9999)
    r = io.read_raster(p, residency=vsr.Residency.DEVICE)
    s = vsr.raster_slope(r).to_numpy().astype(np.float64)
    rs, _ = oracle.slope_aspect(dem, (30.0, 0.0, 0.0, 0.0, -30.0, 0.0), -9999.0)
    assert np.abs(s - rs).max() <= 1e-4


def test_unsupported_codec_and_backend(vsr, tmp_path):
    from vsr_gb300 import io

    p = tmp_path / "c.tif"
    write_geotiff(p, np.zeros((8, 8), np.uint8))
    raw = bytearray(p.read_bytes())
    # rewrite the compression tag value (259) to LZW (5): find it in the first IFD
    n = int.from_bytes(raw[8:10], "little")
    for k in range(n):
        e = 10 + 12 * k
        if int.from_bytes(raw[e:e + 2], "little") == 259:
            raw[e + 8:e + 10] = (5).to_bytes(2, "little")
    p.write_bytes(bytes(raw))
    with pytest.raises(NotImplementedError):
        io.read_raster(p)
    with pytest.raises(NotImplementedError):
        io.read_raster(p, decode_backend="rasterio")


@pytest.mark.parametrize("dt", [np.uint8, np.int16, np.uint16, np.int32, np.float32, np.float64])
@pytest.mark.parametrize("tiled,compress", [(True, "deflate"), (False, "deflate"), (True, None)])
def test_write_raster_read_raster_round_trip(vsr, tmp_path, dt, tiled, compress):
    from vsr_gb300 import io

    rng = np.random.default_rng(7)
    d = _data(dt, (2, 300, 257), rng)
    r = vsr.from_numpy(d, nodata=None, affine=(3.0, 0.0, 1.0, 0.0, -3.0, 2.0), crs="EPSG:3857")
    p = tmp_path / "wr.tif"
    io.write_raster(p, r, compress=compress, tiled=tiled, blockxsize=128, blockysize=64)
    back = io.read_raster(p)
    np.testing.assert_array_equal(back.to_numpy().view(f"u{np.dtype(dt).itemsize}"), d.view(f"u{np.dtype(dt).itemsize}"))
    assert back.affine == r.affine and back.crs == "EPSG:3857"
