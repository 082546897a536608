"""GeoTIFF directory parsing on the host (no GPU): metadata of files written
by the test writer in every layout the reader accepts."""

from __future__ import annotations

import numpy as np
import pytest

from tiff_writer import write_geotiff


@pytest.mark.parametrize("big_endian,bigtiff,tiled", [(False, False, False), (True, False, True), (False, True, True)])
def test_metadata(tmp_path, big_endian, bigtiff, tiled):
    from vsr_gb300 import io

    d = np.arange(3 * 50 * 70, dtype=np.int16).reshape(3, 50, 70)
    p = tmp_path / "m.tif"
    write_geotiff(p, d, tile=(32, 16) if tiled else None, rows_per_strip=7, big_endian=big_endian, bigtiff=bigtiff,
                  affine=(30.0, 0.0, 600000.0, 0.0, -30.0, 5000000.0), epsg=32633, nodata=-32768)
    m = io.read_raster_metadata(p)
    assert (m.height, m.width, m.band_count) == (50, 70, 3)
    assert m.dtype == np.int16
    assert m.nodata == -32768 and isinstance(m.nodata, np.int16)
    assert m.affine == (30.0, 0.0, 600000.0, 0.0, -30.0, 5000000.0)
    assert m.crs == "EPSG:32633"


def test_transformation_and_float_nodata(tmp_path):
    from vsr_gb300 import io

    p = tmp_path / "t.tif"
    write_geotiff(p, np.zeros((4, 5), np.float32), transformation=True, affine=(2.0, 0.5, 10.0, 0.25, -3.0, 20.0),
                  epsg=4326, nodata="nan")
    m = io.read_raster_metadata(p)
    assert m.affine == (2.0, 0.5, 10.0, 0.25, -3.0, 20.0)
    assert m.crs == "EPSG:4326"
    assert np.isnan(m.nodata)


def test_rejects_non_tiff(tmp_path):
    from vsr_gb300 import io

    p = tmp_path / "x.tif"
    p.write_bytes(b"not a tiff at all")
    with pytest.raises(ValueError):
        io.read_raster_metadata(p)


def test_write_raster_metadata_and_layout(tmp_path):
    """write_raster's files parse back to the raster's shape, dtype, affine,
    CRS and nodata, and their chunks cover the image."""
    from vsr_gb300 import io
    from vsr_gb300.buffers import from_numpy

    d = np.arange(2 * 70 * 90, dtype=np.float32).reshape(2, 70, 90)
    r = from_numpy(d, nodata=-9999.0, affine=(5.0, 0.0, 10.0, 0.0, -5.0, 20.0), crs="EPSG:32632")
    for tiled in (True, False):
        p = tmp_path / f"w{tiled}.tif"
        io.write_raster(p, r, tiled=tiled, blockxsize=32, blockysize=16)
        m = io.read_raster_metadata(p)
        assert (m.band_count, m.height, m.width) == (2, 70, 90) and m.dtype == np.float32
        assert m.affine == (5.0, 0.0, 10.0, 0.0, -5.0, 20.0) and m.crs == "EPSG:32632" and m.nodata == -9999.0
        with open(p, "rb") as f:
            t = io._read_ifds(f)[0].tags
        _, _, geo = io._chunk_layout(t, 70, 90, 2, False)
        assert len(geo) == (15 if tiled else 5)
        assert t[259] == (8,) and t[317] == (3,)
