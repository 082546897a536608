"""Streamed host-to-host terrain pass == the in-memory fused pass, bit for bit."""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,strip", [((1000, 777), 97), ((515, 1024), 128), ((64, 256), 1000), ((9, 16), 1)])
def test_streamed_equals_in_memory(vsr, shape, strip):
    from vsr_gb300 import stream

    rng = np.random.default_rng(shape[0])
    yy, xx = np.mgrid[0 : shape[0], 0 : shape[1]]
    d = (1500 + 400 * np.sin(yy / 31.0) * np.cos(xx / 17.0) + rng.uniform(0, 2, shape)).astype(np.float32)
    d[rng.random(shape) < 0.01] = -9999.0
    aff = (10.0, 0, 0, 0, -10.0, 0)
    r = vsr.from_numpy(d, nodata=-9999.0, affine=aff)
    ref = vsr.raster_terrain(r)
    out = stream.raster_terrain_host(r, strip_rows=strip)
    for k in ("slope", "aspect", "hillshade"):
        np.testing.assert_array_equal(out[k].to_numpy(), ref[k].to_numpy(), err_msg=k)
    assert out["hillshade"].nodata == 0 and out["slope"].nodata == -9999.0
