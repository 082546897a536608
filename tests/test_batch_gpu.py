"""One persistent batched launch over uneven tiles == per-tile calls == oracle.

Tiles mix odd widths (rows not 16-byte aligned), -9999 and NaN nodata and
per-tile cell sizes, as the 512-tile workload does.  Tolerances as for the
single-raster paths: slope/aspect 1e-4 degrees (aspect on the circle),
Gaussian 1e-5 relative; nodata and NaN placement exact.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _tiles(vsr, n=23, seed=0, lo=20, hi=700):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        h = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        w = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        yy, xx = np.mgrid[0:h, 0:w]
        z = (800 + 300 * np.sin(yy / (9 + i)) * np.cos(xx / (13 + i)) + rng.uniform(0, 3, (h, w))).astype(np.float32)
        nd = -9999.0 if i % 2 == 0 else float("nan")
        z[rng.random((h, w)) < rng.uniform(0, 0.05)] = nd
        cell = float(rng.uniform(1, 90))
        out.append(vsr.from_numpy(z, nodata=nd, affine=(cell, 0, 0, 0, -cell, 0)))
    return out


def _circ(a, b):
    d = np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64))
    return np.minimum(d, 360.0 - d)


def _check(res, r):
    z = r.to_numpy()
    nd = r.nodata
    rs, ra = oracle.slope_aspect(z, r.affine, nd)
    s = res["slope"].to_numpy()
    a = res["aspect"].to_numpy()
    np.testing.assert_array_equal(np.isnan(s), np.isnan(rs))
    m = ~np.isnan(rs)
    assert np.abs(s[m] - rs[m]).max(initial=0) <= 1e-4
    m = ~np.isnan(ra)
    assert _circ(a[m], ra[m]).max(initial=0) <= 1e-4
    g = res["smooth"].to_numpy()
    rg = oracle.convolve_normalized(z, oracle.gaussian_weights(1.0, 5), nd)
    np.testing.assert_array_equal(np.isnan(g), np.isnan(rg))
    m = ~np.isnan(rg)
    if not np.isnan(nd):
        np.testing.assert_array_equal(g[m] == nd, rg[m] == nd)
    assert (np.abs(g[m] - rg[m]) <= 1e-5 * np.maximum(np.abs(rg[m]), 100.0)).all()


def test_batch_matches_oracle_and_per_tile(vsr):
    from vsr_gb300 import batch

    rasters = _tiles(vsr)
    b = batch.TerrainBatch(rasters, sigma=1.0, kernel_size=5)
    b.run()
    res = b.results()
    for r, d in zip(rasters, res):
        _check(d, r)
    # same answers as the per-tile launches
    per = batch.per_tile_launches(rasters)
    for (s, a, g), d in zip(per, res):
        np.testing.assert_allclose(d["slope"].to_numpy(), s[0].cpu().numpy(), atol=1e-4)
        ga = g[0].cpu().numpy()
        gb = d["smooth"].to_numpy()
        np.testing.assert_array_equal(np.isnan(ga), np.isnan(gb))


def test_batch_graph_replay_and_all_configs_agree(vsr):
    import torch

    from vsr_gb300 import _lib, batch

    rasters = _tiles(vsr, n=9, seed=1)
    b = batch.TerrainBatch(rasters, sigma=1.0, kernel_size=5)
    b.run()
    ref = [{k: v.to_numpy().copy() for k, v in d.items()} for d in b.results()]
    for (s, a, g) in b.outputs:
        s.fill_(0)
        a.fill_(0)
        g.fill_(0)
    b.capture()
    b.replay()
    torch.cuda.synchronize()
    for d0, d in zip(ref, b.results()):
        for k in d0:
            np.testing.assert_array_equal(d[k].to_numpy(), d0[k])
    lib = _lib.load()
    for cfg in range(lib.vsr_tuning_count(_lib.VSR_OP_BATCH)):
        _lib.check(lib.vsr_tuning_set(_lib.VSR_OP_BATCH, cfg), "set")
        b.replan()
        b.run()
        for d0, d in zip(ref, b.results()):
            for k in d0:
                np.testing.assert_array_equal(d[k].to_numpy(), d0[k], err_msg=f"config {cfg} {k}")
    _lib.check(lib.vsr_tuning_set(_lib.VSR_OP_BATCH, 0), "set")


def test_batch_rejects_bad_plans(vsr):
    from vsr_gb300 import batch

    with pytest.raises(ValueError):
        batch.TerrainBatch([])
    r = vsr.from_numpy(np.zeros((8, 8), np.float64))
    with pytest.raises(ValueError, match="float32"):
        batch.TerrainBatch([r])
    r = vsr.from_numpy(np.zeros((8, 8), np.float32))
    with pytest.raises(NotImplementedError):
        batch.TerrainBatch([r], sigma=3.0, kernel_size=19)


def test_batch_run_keeps_the_plans_shape(vsr):
    """A tuning change between plan and run does not change what the run writes."""
    import ctypes

    import torch

    from vsr_gb300 import _lib, batch

    lib = _lib.load()
    rasters = _tiles(vsr, n=5, seed=2)
    _lib.check(lib.vsr_tuning_set(_lib.VSR_OP_BATCH, 2), "set")  # 16-row blocks
    b = batch.TerrainBatch(rasters, sigma=1.0, kernel_size=5)
    b.run()
    ref = [{k: v.to_numpy().copy() for k, v in d.items()} for d in b.results()]
    for (s, a, g) in b.outputs:
        s.fill_(0)
        a.fill_(0)
        g.fill_(0)
    _lib.check(lib.vsr_tuning_set(_lib.VSR_OP_BATCH, 1), "set")  # 64-row blocks, not re-planned
    b.run()
    torch.cuda.synchronize()
    for d0, d in zip(ref, b.results()):
        for k in d0:
            np.testing.assert_array_equal(d[k].to_numpy(), d0[k])
    code = ctypes.c_uint32(0)
    _lib.check(lib.vsr_poll_device_error(None, ctypes.byref(code)), "poll")
    assert code.value == 0
    # a Gaussian width other than the plan's is refused on the host
    st = lib.vsr_batch_run(b.plan, 3, torch.cuda.current_stream().cuda_stream)
    assert st == _lib.VSR_ERR_INVALID_ARG and "does not match" in _lib.last_error()
    _lib.check(lib.vsr_tuning_set(_lib.VSR_OP_BATCH, 0), "set")
