"""Streamed host-to-host focal passes: row strips with a halo, copies overlapped.

The GB300 counterpart of the reference's out-of-core tiling
(``dispatch_tiled_halo``, src/vibespatial/raster/tiling.py:468-659, with its
halo/affine rules at :564-579) for the fused Horn pass (one-row halo) and,
at the end of this module, for the normalised convolution, the Gaussian and
the focal statistics (a halo of the window's rows).  The DEM stays in
host memory (ideally page-locked); it is cut into row strips that carry a
one-row halo above and below, and each strip goes through

    host -> device copy  |  vsr_horn_fused on the strip  |  device -> host copy

on its own CUDA stream, round-robin over ``n_streams`` streams, so the
copy engines (one per direction) and the SMs work on different strips at
the same time.  Output rows of a strip are taken from its inner rows, whose
neighbours are real data; the raster's own first and last rows keep the
reference's edge replication.  Results are identical to ``raster_terrain``
on the whole raster.
"""

from __future__ import annotations

import math

import numpy as np

from vsr_gb300 import _lib
from vsr_gb300.algebra import NODATA_CENTER, NODATA_WINDOW, cellsize, nodata_kind
from vsr_gb300.buffers import OwnedRasterArray, from_numpy


def _pinned_view(a: np.ndarray):
    import torch

    t = torch.from_numpy(a)
    return t, bool(t.is_pinned())


def terrain_host(dem: np.ndarray, affine, nodata, *, slope_out: np.ndarray | None = None,
                 aspect_out: np.ndarray | None = None, hs_out: np.ndarray | None = None,
                 azimuth: float = 315.0, altitude: float = 45.0, z_factor: float = 1.0,
                 nodata_mode: str = NODATA_WINDOW, strip_rows: int = 1024, n_streams: int = 3,
                 phase_events: list | None = None):
    """Fill the given host arrays (float32 slope/aspect, uint8 hillshade) from a host DEM.

    ``phase_events``: a list that receives, per strip, four CUDA events
    recorded on the strip's stream before its host->device copy, after it,
    after the kernel and after its device->host copies (see phase_summary).
    """
    import torch

    if dem.ndim != 2 or dem.dtype != np.float32:
        raise ValueError("terrain_host streams single-band float32 DEMs")
    H, W = dem.shape
    outs = [o for o in (slope_out, aspect_out, hs_out)]
    for o, dt in zip(outs, (np.float32, np.float32, np.uint8)):
        if o is not None and (o.shape != (H, W) or o.dtype != dt or not o.flags.c_contiguous):
            raise ValueError("outputs must be C-contiguous (H, W) arrays: float32 slope/aspect, uint8 hillshade")
    if slope_out is None and aspect_out is None and hs_out is None:
        return
    lib = _lib.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    src_t, _ = _pinned_view(np.ascontiguousarray(dem))
    host_outs = [torch.from_numpy(o) if o is not None else None for o in outs]
    kind = nodata_kind(OwnedRasterArray(data=dem, nodata=nodata, dtype=dem.dtype, affine=tuple(affine)))[0]
    ndv = float(nodata) if nodata is not None else 0.0
    if kind == _lib.VSR_NODATA_NAN:
        ndv = float("nan")
    flags = _lib.VSR_HORN_CENTER_ONLY if nodata_mode == NODATA_CENTER else _lib.VSR_HORN_SA_NAN_UNMASKED
    cx, cy = cellsize(affine)
    zen = math.radians(90.0 - float(altitude))
    az = math.radians(float(azimuth))
    sr = max(1, min(int(strip_rows), H))
    cap = sr + 2
    streams = [torch.cuda.Stream(device=dev) for _ in range(n_streams)]
    bufs = []
    for _ in range(n_streams):
        bufs.append((
            torch.empty((cap, W), dtype=torch.float32, device=dev),
            torch.empty((cap, W), dtype=torch.float32, device=dev) if slope_out is not None else None,
            torch.empty((cap, W), dtype=torch.float32, device=dev) if aspect_out is not None else None,
            torch.empty((cap, W), dtype=torch.uint8, device=dev) if hs_out is not None else None,
        ))
    cur = torch.cuda.current_stream(dev)
    for s in streams:
        s.wait_stream(cur)  # buffers were allocated on the current stream
    n_strips = (H + sr - 1) // sr
    for i in range(n_strips):
        y0, y1 = i * sr, min(H, (i + 1) * sr)
        lo, hi = max(0, y0 - 1), min(H, y1 + 1)  # strip with its halo rows
        rows = hi - lo
        s = streams[i % n_streams]
        d_in, d_s, d_a, d_h = bufs[i % n_streams]
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)] if phase_events is not None else None
        with torch.cuda.stream(s):
            if ev:
                ev[0].record(s)
            d_in[:rows].copy_(src_t[lo:hi], non_blocking=True)
            if ev:
                ev[1].record(s)
            st = lib.vsr_horn_fused(
                d_in.data_ptr(), _lib.VSR_F32, rows, W, W, cx, cy, ndv, kind, flags,
                d_s.data_ptr() if d_s is not None else None, d_a.data_ptr() if d_a is not None else None,
                _lib.VSR_F32, W, d_h.data_ptr() if d_h is not None else None, W, float(z_factor), zen, az,
                s.cuda_stream)
            _lib.check(st, "vsr_horn_fused")
            if ev:
                ev[2].record(s)
            a, b = y0 - lo, y1 - lo  # inner rows of the strip
            for d, h in zip((d_s, d_a, d_h), host_outs):
                if d is not None:
                    h[y0:y1].copy_(d[a:b], non_blocking=True)
            if ev:
                ev[3].record(s)
                phase_events.append(ev)
    for s in streams:
        cur.wait_stream(s)
    cur.synchronize()


def phase_summary(phase_events: list) -> dict:
    """Per-phase device time of a streamed pass from terrain_host's events:
    the summed host->device, kernel and device->host times over the strips,
    and the span from the first strip's start to the last strip's end (the
    phases of different strips overlap, so the sums exceed the span)."""
    if not phase_events:
        return {}
    h2d = sum(e[0].elapsed_time(e[1]) for e in phase_events)
    ker = sum(e[1].elapsed_time(e[2]) for e in phase_events)
    d2h = sum(e[2].elapsed_time(e[3]) for e in phase_events)
    first = phase_events[0][0]
    span = max(first.elapsed_time(e[3]) for e in phase_events)
    return {"strips": len(phase_events), "h2d_ms": h2d, "kernel_ms": ker, "d2h_ms": d2h, "span_ms": span}


def raster_terrain_host(dem: OwnedRasterArray, *, slope: bool = True, aspect: bool = True, hillshade: bool = True,
                        azimuth: float = 315.0, altitude: float = 45.0, z_factor: float = 1.0,
                        nodata_mode: str = NODATA_WINDOW, out=None, strip_rows: int = 1024,
                        n_streams: int = 3, phase_events: list | None = None) -> dict[str, OwnedRasterArray]:
    """``raster_terrain`` for a host-resident DEM with host-resident results.

    Streams row strips through the GPU (copies overlapped with the fused
    kernel) instead of copying the whole raster in and out; works for DEMs
    larger than device memory.  ``out`` may give preallocated host arrays
    (slope, aspect, hillshade) -- page-locked ones make the copies
    asynchronous.
    """
    z = dem.to_numpy()
    if z.ndim == 3:
        if z.shape[0] != 1:
            raise ValueError("raster_terrain_host streams single-band DEMs")
        z = z[0]
    H, W = z.shape
    o_s, o_a, o_h = out if out is not None else (None, None, None)
    if slope and o_s is None:
        o_s = np.empty((H, W), np.float32)
    if aspect and o_a is None:
        o_a = np.empty((H, W), np.float32)
    if hillshade and o_h is None:
        o_h = np.empty((H, W), np.uint8)
    terrain_host(np.asarray(z, dtype=np.float32), dem.affine, dem.nodata, slope_out=o_s if slope else None,
                 aspect_out=o_a if aspect else None, hs_out=o_h if hillshade else None, azimuth=azimuth,
                 altitude=altitude, z_factor=z_factor, nodata_mode=nodata_mode, strip_rows=strip_rows,
                 n_streams=n_streams, phase_events=phase_events)
    res = {}
    if slope:
        res["slope"] = from_numpy(o_s, nodata=dem.nodata, affine=dem.affine, crs=dem.crs)
    if aspect:
        res["aspect"] = from_numpy(o_a, nodata=dem.nodata, affine=dem.affine, crs=dem.crs)
    if hillshade:
        res["hillshade"] = from_numpy(o_h, nodata=0 if dem.nodata is not None else None, affine=dem.affine,
                                      crs=dem.crs)
    return res


# ---------------------------------------------------------------------------
# Streamed normalised convolution, Gaussian and focal statistics
# ---------------------------------------------------------------------------


def _focal_host(data: np.ndarray, halo_up: int, halo_down: int, launch, out: np.ndarray, *,
                strip_rows: int, n_streams: int, ws_bytes: int = 0):
    """Stream ``data`` (H, W) through ``launch`` in row strips.

    Each strip carries ``halo_up`` / ``halo_down`` real rows around its output
    rows (fewer at the raster's own edges, where the kernels' out-of-bounds
    rule applies, as on the whole raster), goes host -> device, through
    ``launch(d_in, rows, d_out, workspace, workspace_bytes, stream)`` and
    back into the matching rows of ``out``, round-robin over ``n_streams``
    CUDA streams so copies and kernels of different strips overlap.
    """
    import torch

    H, W = data.shape
    lib = _lib.load()
    del lib  # loaded (and checked) before any stream work
    dev = torch.device("cuda", torch.cuda.current_device())
    src_t = torch.from_numpy(np.ascontiguousarray(data))
    dst_t = torch.from_numpy(out)
    sr = max(1, min(int(strip_rows), H))
    cap = min(H, sr + halo_up + halo_down)
    streams = [torch.cuda.Stream(device=dev) for _ in range(n_streams)]
    bufs = [(torch.empty((cap, W), dtype=src_t.dtype, device=dev), torch.empty((cap, W), dtype=dst_t.dtype, device=dev),
             torch.empty(max(int(ws_bytes), 256) + 256, dtype=torch.uint8, device=dev)) for _ in range(n_streams)]
    cur = torch.cuda.current_stream(dev)
    for s in streams:
        s.wait_stream(cur)  # buffers were allocated on the current stream
    for i in range((H + sr - 1) // sr):
        y0, y1 = i * sr, min(H, (i + 1) * sr)
        lo, hi = max(0, y0 - halo_up), min(H, y1 + halo_down)
        s = streams[i % n_streams]
        d_in, d_out, ws = bufs[i % n_streams]
        with torch.cuda.stream(s):
            d_in[: hi - lo].copy_(src_t[lo:hi], non_blocking=True)
            launch(d_in, hi - lo, d_out, (ws.data_ptr() + 255) // 256 * 256, int(ws_bytes), s.cuda_stream)
            dst_t[y0:y1].copy_(d_out[y0 - lo:y1 - lo], non_blocking=True)
    for s in streams:
        cur.wait_stream(s)
    cur.synchronize()


def _pinned_empty(shape, dtype) -> np.ndarray:
    """A page-locked host array (the device -> host copies of the strips then
    run asynchronously instead of blocking the host between strips)."""
    import torch

    from vsr_gb300.buffers import torch_dtype

    return torch.empty(shape, dtype=torch_dtype(np.dtype(dtype)), pin_memory=True).numpy()


def _host_plane(raster: OwnedRasterArray):
    from vsr_gb300.algebra import _WIDEN

    z = np.asarray(raster.to_numpy())
    if z.ndim == 2:
        z = z[None]
    dt = np.dtype(z.dtype)
    if dt in _WIDEN:
        z = z.astype(_WIDEN[dt])
    return z


def _stream_result(raster: OwnedRasterArray, outs: np.ndarray) -> OwnedRasterArray:
    data = outs[0] if np.asarray(raster.data).ndim == 2 else outs
    return from_numpy(data, nodata=raster.nodata, affine=raster.affine, crs=raster.crs)


def raster_convolve_host(raster: OwnedRasterArray, kernel: np.ndarray, *, precision: str = "auto",
                         out_dtype=np.float64, strip_rows: int = 2048, n_streams: int = 3) -> OwnedRasterArray:
    """``raster_convolve`` for a host-resident raster with a host-resident result,
    streamed in row strips with a halo of the kernel's rows (the reference's
    out-of-core tiling, tiling.py:468-659, halo rule :564-579); for rasters
    larger than device memory.  Equal to the resident call up to the
    floating-point order of the per-tile sums."""
    from vsr_gb300.algebra import _out_code, _precision_code

    w = np.ascontiguousarray(np.asarray(kernel, dtype=np.float64))
    if w.ndim != 2:
        raise ValueError(f"kernel must be 2D, got {w.ndim}D")
    kh, kw = w.shape
    z = _host_plane(raster)
    B, H, W = z.shape
    kind, ndv = nodata_kind(raster)
    nd = float(raster.nodata) if kind == _lib.VSR_NODATA_VALUE else ndv
    ocode, odt = _out_code(out_dtype)
    prec = _precision_code(precision)
    lib = _lib.load()
    nbytes = lib.vsr_convolve_workspace_size(kh, kw, prec)
    wp = w.ctypes.data_as(_lib._c.POINTER(_lib._c.c_double))
    code = _lib.dtype_code(z.dtype)
    outs = _pinned_empty((B, H, W), odt)

    def launch(d_in, rows, d_out, ws, ws_bytes, stream):
        _lib.check(lib.vsr_convolve(d_in.data_ptr(), code, rows, W, W, wp, kh, kw, nd, kind, d_out.data_ptr(), ocode,
                                    W, prec, ws, ws_bytes, stream), "vsr_convolve")

    for b in range(B):
        _focal_host(z[b], kh // 2, kh - 1 - kh // 2, launch, outs[b], strip_rows=strip_rows, n_streams=n_streams,
                    ws_bytes=nbytes)
    return _stream_result(raster, outs)


def raster_gaussian_filter_host(raster: OwnedRasterArray, sigma: float, *, kernel_size: int | None = None,
                                precision: str = "auto", out_dtype=np.float64, strip_rows: int = 2048,
                                n_streams: int = 3) -> OwnedRasterArray:
    """``raster_gaussian_filter`` streamed from and to host memory in row strips
    with a halo of k // 2 rows (see raster_convolve_host)."""
    from vsr_gb300.algebra import _out_code, _precision_code, gaussian_kernel_size

    k = gaussian_kernel_size(sigma, kernel_size)
    z = _host_plane(raster)
    B, H, W = z.shape
    kind, ndv = nodata_kind(raster)
    nd = float(raster.nodata) if kind == _lib.VSR_NODATA_VALUE else ndv
    ocode, odt = _out_code(out_dtype)
    prec = _precision_code(precision)
    lib = _lib.load()
    code = _lib.dtype_code(z.dtype)
    rows_max = min(H, int(strip_rows) + 2 * (k // 2))
    nbytes = lib.vsr_gaussian_workspace_bytes(rows_max, W, code, float(sigma), k, prec)
    outs = _pinned_empty((B, H, W), odt)

    def launch(d_in, rows, d_out, ws, ws_bytes, stream):
        _lib.check(lib.vsr_gaussian(d_in.data_ptr(), code, rows, W, W, float(sigma), k, nd, kind, d_out.data_ptr(),
                                    ocode, W, prec, ws, ws_bytes, stream), "vsr_gaussian")

    for b in range(B):
        _focal_host(z[b], k // 2, k // 2, launch, outs[b], strip_rows=strip_rows, n_streams=n_streams,
                    ws_bytes=nbytes)
    return _stream_result(raster, outs)


def raster_focal_host(raster: OwnedRasterArray, stat: str, radius=1, *, out_dtype=np.float64,
                      strip_rows: int = 2048, n_streams: int = 3) -> OwnedRasterArray:
    """A focal statistic (``min``, ``max``, ``mean``, ``std``, ``range``,
    ``variety``; see raster_focal_min etc.) streamed from and to host memory in
    row strips with a halo of radius_y rows."""
    from vsr_gb300.algebra import _out_code, _parse_radius

    if stat not in _lib.VSR_STAT:
        raise ValueError(f"unknown focal statistic {stat!r}; expected one of {sorted(_lib.VSR_STAT)}")
    ry, rx = _parse_radius(radius)
    z = _host_plane(raster)
    B, H, W = z.shape
    kind, ndv = nodata_kind(raster)
    nd = float(raster.nodata) if kind == _lib.VSR_NODATA_VALUE else ndv
    ocode, odt = _out_code(out_dtype)
    lib = _lib.load()
    code = _lib.dtype_code(z.dtype)
    outs = _pinned_empty((B, H, W), odt)

    def launch(d_in, rows, d_out, ws, ws_bytes, stream):
        _lib.check(lib.vsr_focal_stat(d_in.data_ptr(), code, rows, W, W, _lib.VSR_STAT[stat], ry, rx, nd, kind,
                                      d_out.data_ptr(), ocode, W, stream), "vsr_focal_stat")

    for b in range(B):
        _focal_host(z[b], ry, ry, launch, outs[b], strip_rows=strip_rows, n_streams=n_streams)
    return _stream_result(raster, outs)
