"""Batched focal work over many rasters in one persistent launch.

``TerrainBatch`` plans slope + aspect and a small Gaussian for a list of
float32 DEM tiles of uneven sizes -- each with its own cell size (from its
affine) and nodata -- and runs them as ONE work-queue-scheduled persistent
launch (``vsr_batch_run``), optionally recorded once into a CUDA graph and
replayed.  It replaces per-raster / per-band launch loops such as the
reference's ``dispatch_per_band_gpu`` (dispatch.py:417-506).  Results equal
``raster_slope`` / ``raster_aspect`` / ``raster_gaussian_filter`` on each tile.
"""

from __future__ import annotations

import ctypes


import numpy as np

from vsr_gb300 import _lib
from vsr_gb300.algebra import cellsize, gaussian_kernel_size, nodata_kind
from vsr_gb300.buffers import OwnedRasterArray, from_device


class BatchTile(ctypes.Structure):
    """Mirror of ``vsr_batch_tile`` in include/vsr.h."""

    _fields_ = [
        ("src", ctypes.c_void_p),
        ("height", ctypes.c_int64),
        ("width", ctypes.c_int64),
        ("pitch", ctypes.c_int64),
        ("slope", ctypes.c_void_p),
        ("aspect", ctypes.c_void_p),
        ("smooth", ctypes.c_void_p),
        ("out_pitch", ctypes.c_int64),
        ("cell_x", ctypes.c_double),
        ("cell_y", ctypes.c_double),
        ("nodata", ctypes.c_double),
        ("nodata_kind", ctypes.c_int32),
        ("flags", ctypes.c_uint32),
    ]


def _bind(lib):
    if getattr(lib, "_vsr_batch_bound", False):
        return
    lib.vsr_batch_plan.argtypes = [ctypes.POINTER(BatchTile), ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                   ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_int64), ctypes.c_void_p]
    lib._vsr_batch_bound = True


class TerrainBatch:
    """Plan once, run (or replay a captured graph) many times."""

    def __init__(self, rasters: list[OwnedRasterArray], *, terrain: bool = True, sigma: float | None = 1.0,
                 kernel_size: int | None = 5):
        import torch

        if not rasters:
            raise ValueError("need at least one raster")
        self.lib = _lib.load()
        _bind(self.lib)
        self.rasters = rasters
        self.k = gaussian_kernel_size(sigma, kernel_size) if sigma is not None else 0
        self.sigma = float(sigma) if sigma is not None else 0.0
        self.inputs, self.outputs = [], []
        arr = (BatchTile * len(rasters))()
        for i, r in enumerate(rasters):
            if r.data.ndim != 2 or np.dtype(r.dtype) != np.float32:
                raise ValueError("batched tiles must be single-band float32 rasters")
            t = r.device_data().contiguous()
            H, W = t.shape
            # outputs with rows padded to 16 bytes (views of W columns): the kernel
            # then stores 4 pixels per 128-bit store whatever the tile's width
            Wp = (W + 3) // 4 * 4
            mk = lambda: torch.empty((H, Wp), dtype=torch.float32, device=t.device)[:, :W]  # noqa: E731
            slope = mk() if terrain else None
            aspect = mk() if terrain else None
            smooth = mk() if self.k else None
            self.inputs.append(t)
            self.outputs.append((slope, aspect, smooth))
            kind, ndv = nodata_kind(r)
            cx, cy = cellsize(r.affine)
            arr[i] = BatchTile(t.data_ptr(), H, W, W,
                               slope.data_ptr() if slope is not None else None,
                               aspect.data_ptr() if aspect is not None else None,
                               smooth.data_ptr() if smooth is not None else None,
                               Wp, cx, cy, ndv if kind != _lib.VSR_NODATA_NONE else 0.0, kind,
                               _lib.VSR_HORN_SA_NAN_UNMASKED)
        self._tiles = arr
        nbytes = self.lib.vsr_batch_plan_size(len(rasters))
        self._plan_buf = torch.empty(nbytes + 256, dtype=torch.uint8, device=self.inputs[0].device)
        self.plan = (self._plan_buf.data_ptr() + 255) // 256 * 256
        self.plan_bytes = nbytes
        self.total_items = 0
        self.graph = None
        self.replan()

    def replan(self):
        """(Re)build the device plan, e.g. after the tuning table changed."""
        import torch

        total = ctypes.c_int64(0)
        st = self.lib.vsr_batch_plan(self._tiles, len(self.rasters), self.sigma, self.k, self.plan, self.plan_bytes,
                                     ctypes.byref(total), torch.cuda.current_stream().cuda_stream)
        _lib.check(st, "vsr_batch_plan")
        self.total_items = total.value
        self.graph = None

    def run(self):
        """Enqueue the single batched launch on the current stream."""
        import torch

        _lib.check(self.lib.vsr_batch_run(self.plan, self.k, torch.cuda.current_stream().cuda_stream),
                   "vsr_batch_run")

    def capture(self):
        """Record the launch (counter reset + kernel) into a CUDA graph."""
        import torch

        self.run()  # warm-up outside capture (sets kernel attributes)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run()
        self.graph = g
        return g

    def replay(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()

    def results(self) -> list[dict[str, OwnedRasterArray]]:
        out = []
        for r, (s, a, g) in zip(self.rasters, self.outputs):
            d = {}
            if s is not None:
                d["slope"] = from_device(s, nodata=r.nodata, affine=r.affine, crs=r.crs)
                d["aspect"] = from_device(a, nodata=r.nodata, affine=r.affine, crs=r.crs)
            if g is not None:
                d["smooth"] = from_device(g, nodata=r.nodata if r.nodata is not None else None,
                                          affine=r.affine, crs=r.crs)
            out.append(d)
        return out


def per_tile_launches(rasters: list[OwnedRasterArray], *, sigma: float = 1.0, kernel_size: int = 5, outs=None):
    """The unbatched comparison: one Horn launch and one Gaussian launch per tile."""
    from vsr_gb300 import algebra

    res = []
    for i, r in enumerate(rasters):
        o = outs[i] if outs is not None else (None, None, None)
        s, a, _ = algebra.horn_fused(r, slope=True, aspect=True, hillshade=False,
                                     out=(o[0], o[1], None) if outs is not None else None)
        g = algebra.gaussian_bands(r, sigma, kernel_size, precision="fp32", out_dtype=np.float32,
                                   out=o[2] if outs is not None else None)
        res.append((s, a, g))
    return res


class PerTileGraph:
    """The unbatched comparison in its fastest form: one Horn launch and one
    Gaussian call per tile (``per_tile_launches``), recorded once into a CUDA
    graph and replayed, so that a replay costs the kernels and not Python."""

    def __init__(self, rasters: list[OwnedRasterArray], *, sigma: float = 1.0, kernel_size: int = 5):
        import torch

        self.rasters = rasters
        self.outs = []
        for r in rasters:
            t = r.device_data()
            H, W = t.shape[-2:]
            self.outs.append(tuple(torch.empty((1, H, W), dtype=torch.float32, device=t.device) for _ in range(3)))
        self.sigma, self.k = sigma, kernel_size
        per_tile_launches(rasters, sigma=sigma, kernel_size=kernel_size, outs=self.outs)  # warm-up outside capture
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            per_tile_launches(rasters, sigma=sigma, kernel_size=kernel_size, outs=self.outs)
        # per tile: the Horn kernel, the Gaussian tap build and the separable Gaussian
        self.launches = 3 * len(rasters)

    def replay(self):
        self.graph.replay()


def autotune_batch(batch: TerrainBatch, *, repeats: int = 3) -> dict:
    """Time every batch launch configuration on ``batch`` and keep the fastest."""
    import torch

    lib = batch.lib
    n = lib.vsr_tuning_count(_lib.VSR_OP_BATCH)
    times = {}
    stream = torch.cuda.current_stream()
    for cfg in range(n):
        _lib.check(lib.vsr_tuning_set(_lib.VSR_OP_BATCH, cfg), "vsr_tuning_set")
        batch.replan()
        batch.run()
        samples = []
        for _ in range(repeats):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            batch.run()
            e1.record(stream)
            e1.synchronize()
            samples.append(e0.elapsed_time(e1))
        times[cfg] = sorted(samples)[len(samples) // 2]
    best = min(times, key=times.get)
    _lib.check(lib.vsr_tuning_set(_lib.VSR_OP_BATCH, best), "vsr_tuning_set")
    batch.replan()
    return {"config": best, "ms": times}


BATCH_CONFIGS = [(32, 128), (48, 128), (64, 256), (16, 128)]  # kBatchConfigs: (rows per block, threads)

__all__ = ["TerrainBatch", "PerTileGraph", "per_tile_launches", "autotune_batch", "BATCH_CONFIGS"]


