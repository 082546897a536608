"""Focal-stencil operations on OwnedRasterArray, backed by libvsr (sm_103a).

Drop-in counterparts of the reference's public functions in
src/vibespatial/raster/algebra.py -- same names, arguments, dtype rules,
nodata conventions, diagnostics prefixes and errors:

=====================  ==============================  ==========================
function               reference                        libvsr entry point
=====================  ==============================  ==========================
raster_slope           algebra.py:2386-2459             vsr_horn_fused
raster_aspect          algebra.py:2462-2535             vsr_horn_fused
raster_hillshade       algebra.py:2778-2818             vsr_horn_fused
raster_convolve        algebra.py:2101-2117             vsr_convolve
raster_gaussian_filter algebra.py:2120-2154             vsr_gaussian
raster_focal_mean      algebra.py:3582-3604             vsr_focal_mean
raster_focal_min       algebra.py:3531-3554             vsr_focal_stat_bands
raster_focal_max       algebra.py:3557-3579             vsr_focal_stat_bands
raster_focal_std       algebra.py:3607-3631             vsr_focal_stat_bands
raster_focal_range     algebra.py:3634-3656             vsr_focal_stat_bands
raster_focal_variety   algebra.py:3659-3684             vsr_focal_stat_bands
=====================  ==============================  ==========================

``raster_terrain`` is new: slope, aspect and hillshade from ONE pass over the
DEM (the reference needs three calls and three passes).

There is no CPU path.  ``use_gpu`` is accepted for signature compatibility;
``use_gpu=False`` raises, and ``None`` always selects the GPU.
"""

from __future__ import annotations

import math
import time

import numpy as np

from vsr_gb300 import _lib
from vsr_gb300.buffers import (
    OwnedRasterArray,
    RasterDiagnosticEvent,
    RasterDiagnosticKind,
    from_device,
    torch_dtype,
)
from vsr_gb300.residency import Residency

_GPU_ONLY = (
    "vsr_gb300 runs focal operations on the GPU only; use the reference package "
    "for its CPU path (use_gpu=False)"
)


def _torch():
    import torch

    return torch


def _should_use_gpu(raster: OwnedRasterArray, threshold: int = 10_000) -> bool:
    """The reference's auto-dispatch test (algebra.py:3009-3019).

    Kept for API parity; this package always runs on the GPU.
    """
    torch = _torch()
    return bool(torch.cuda.is_available()) and raster.pixel_count >= threshold


def _require_gpu(use_gpu) -> None:
    if use_gpu is False:
        raise NotImplementedError(_GPU_ONLY)
    torch = _torch()
    if not torch.cuda.is_available():
        raise RuntimeError("vsr_gb300 needs a CUDA device (GB300, sm_103a)")
    _lib.load()


def _stream_handle():
    return _torch().cuda.current_stream().cuda_stream


def cellsize(affine) -> tuple[float, float]:
    """|a|, |e| of the affine with 1.0 for zero (algebra.py:2307-2308)."""
    a = float(affine[0])
    e = float(affine[4])
    return (abs(a) if a != 0 else 1.0, abs(e) if e != 0 else 1.0)


def nodata_kind(raster: OwnedRasterArray) -> tuple[int, float]:
    nd = raster.nodata
    if nd is None:
        return _lib.VSR_NODATA_NONE, 0.0
    if isinstance(nd, float) and math.isnan(nd):
        return _lib.VSR_NODATA_NAN, float("nan")
    return _lib.VSR_NODATA_VALUE, float(nd)


# Element types libvsr reads natively; others are widened exactly on the device.
_WIDEN = {
    np.dtype(np.int8): np.dtype(np.int16),
    np.dtype(np.uint32): np.dtype(np.float64),
    np.dtype(np.int64): np.dtype(np.float64),
    np.dtype(np.uint64): np.dtype(np.float64),
    np.dtype(np.float16): np.dtype(np.float32),
    np.dtype(np.bool_): np.dtype(np.uint8),
}


def _device_bands(raster: OwnedRasterArray):
    """(B, H, W) contiguous device tensor of a natively readable dtype."""
    t = raster.device_data()
    if t.ndim == 2:
        t = t.unsqueeze(0)
    dt = np.dtype(raster.dtype)
    if dt in _WIDEN:
        t = t.to(torch_dtype(_WIDEN[dt]))
        dt = _WIDEN[dt]
    if not t.is_contiguous():
        t = t.contiguous()
    return t, dt


def _shape_like(raster: OwnedRasterArray, t):
    """Return ``t`` (B, H, W) shaped like the input: 2-D when the input is 2-D."""
    return t[0] if raster.data.ndim == 2 else t


def _shared_layout(*tensors) -> tuple[int, int]:
    """(band stride, row pitch) in elements shared by the given (B, H, W)
    output tensors (None entries skipped); rows must be contiguous."""
    lay = {(t.stride(0), t.stride(1)) for t in tensors if t is not None}
    if any(t.stride(2) != 1 for t in tensors if t is not None) or len(lay) > 1:
        raise ValueError("output tensors must share one (band, row) layout with contiguous rows")
    return lay.pop() if lay else (0, 0)


def _record(result: OwnedRasterArray, detail: str, elapsed: float = 0.0) -> OwnedRasterArray:
    result.diagnostics.append(
        RasterDiagnosticEvent(
            kind=RasterDiagnosticKind.RUNTIME,
            detail=detail,
            residency=Residency.DEVICE,
            visible_to_user=True,
            elapsed_seconds=elapsed,
        )
    )
    return result


# ---------------------------------------------------------------------------
# Horn 3x3 family
# ---------------------------------------------------------------------------

NODATA_WINDOW = "window"  # reference CPU rule (algebra.py:2218-2247); default
NODATA_CENTER = "center"  # reference GPU kernel rule (kernels/focal.py:245-250)


def _terrain_out_dtype(dt: np.dtype) -> np.dtype:
    """float input keeps its dtype, anything else gives float64 (algebra.py:2419-2427)."""
    dt = np.dtype(dt)
    if np.issubdtype(dt, np.floating) and dt != np.float64:
        return dt
    return np.dtype(np.float64)


def horn_fused(
    dem: OwnedRasterArray,
    *,
    slope: bool = True,
    aspect: bool = True,
    hillshade: bool = True,
    azimuth: float = 315.0,
    altitude: float = 45.0,
    z_factor: float = 1.0,
    nodata_mode: str = NODATA_WINDOW,
    out=None,
):
    """One vsr_horn_fused_bands launch over every band; returns (slope, aspect, hs) tensors.

    ``out`` may supply preallocated (B, H, W) device tensors for the three
    outputs (None entries are allocated).
    """
    torch = _torch()
    src, dt = _device_bands(dem)
    B, H, W = src.shape
    kind, ndv = nodata_kind(dem)
    flags = 0
    if nodata_mode == NODATA_CENTER:
        flags |= _lib.VSR_HORN_CENTER_ONLY
    elif nodata_mode != NODATA_WINDOW:
        raise ValueError(f"nodata_mode must be 'window' or 'center', got {nodata_mode!r}")
    else:
        flags |= _lib.VSR_HORN_SA_NAN_UNMASKED
    out_np = _terrain_out_dtype(dem.dtype)
    compute_np = np.dtype(np.float64) if out_np == np.float64 else np.dtype(np.float32)
    o_s, o_a, o_h = out if out is not None else (None, None, None)
    dev = src.device
    s_t = (o_s if o_s is not None else torch.empty((B, H, W), dtype=torch_dtype(compute_np), device=dev)) if slope else None
    a_t = (o_a if o_a is not None else torch.empty((B, H, W), dtype=torch_dtype(compute_np), device=dev)) if aspect else None
    h_t = (o_h if o_h is not None else torch.empty((B, H, W), dtype=torch.uint8, device=dev)) if hillshade else None
    cx, cy = cellsize(dem.affine)
    zen = math.radians(90.0 - float(altitude))
    az = math.radians(float(azimuth))
    lib = _lib.load()
    code = _lib.dtype_code(dt)
    ocode = _lib.VSR_F64 if compute_np == np.float64 else _lib.VSR_F32
    stream = _stream_handle()
    sa_bs, sa_p = _shared_layout(s_t, a_t)
    h_bs, h_p = _shared_layout(h_t)
    st = lib.vsr_horn_fused_bands(
        src.data_ptr(), code, B, H * W, H, W, W, cx, cy, ndv, kind, flags,
        s_t.data_ptr() if s_t is not None else None,
        a_t.data_ptr() if a_t is not None else None,
        ocode, sa_bs, sa_p,
        h_t.data_ptr() if h_t is not None else None, h_bs, h_p,
        float(z_factor), zen, az, stream,
    )
    _lib.check(st, "vsr_horn_fused_bands")
    if out_np not in (np.dtype(np.float32), np.dtype(np.float64)):
        s_t = s_t.to(torch_dtype(out_np)) if s_t is not None else None
        a_t = a_t.to(torch_dtype(out_np)) if a_t is not None else None
    return s_t, a_t, h_t


def raster_slope(dem: OwnedRasterArray, *, use_gpu: bool | None = None,
                 nodata_mode: str = NODATA_WINDOW) -> OwnedRasterArray:
    """Slope in degrees (Horn 3x3), reference algebra.py:2386-2459."""
    _require_gpu(use_gpu)
    t0 = time.perf_counter()
    s, _, _ = horn_fused(dem, slope=True, aspect=False, hillshade=False, nodata_mode=nodata_mode)
    res = from_device(_shape_like(dem, s), nodata=dem.nodata, affine=dem.affine, crs=dem.crs)
    return _record(res, f"gpu_slope_fused {dem.width}x{dem.height}", time.perf_counter() - t0)


def raster_aspect(dem: OwnedRasterArray, *, use_gpu: bool | None = None,
                  nodata_mode: str = NODATA_WINDOW) -> OwnedRasterArray:
    """Aspect in compass degrees (0 = north, clockwise), reference algebra.py:2462-2535."""
    _require_gpu(use_gpu)
    t0 = time.perf_counter()
    _, a, _ = horn_fused(dem, slope=False, aspect=True, hillshade=False, nodata_mode=nodata_mode)
    res = from_device(_shape_like(dem, a), nodata=dem.nodata, affine=dem.affine, crs=dem.crs)
    return _record(res, f"gpu_aspect_fused {dem.width}x{dem.height}", time.perf_counter() - t0)


def raster_hillshade(dem: OwnedRasterArray, *, azimuth: float = 315.0, altitude: float = 45.0,
                     z_factor: float = 1.0, use_gpu: bool | None = None) -> OwnedRasterArray:
    """uint8 hillshade, reference algebra.py:2778-2818 (nodata 0 if the input has nodata)."""
    _require_gpu(use_gpu)
    t0 = time.perf_counter()
    _, _, h = horn_fused(dem, slope=False, aspect=False, hillshade=True, azimuth=azimuth,
                         altitude=altitude, z_factor=z_factor)
    res = from_device(_shape_like(dem, h), nodata=0 if dem.nodata is not None else None,
                      affine=dem.affine, crs=dem.crs)
    return _record(res, f"gpu_hillshade {dem.width}x{dem.height}", time.perf_counter() - t0)


def raster_terrain(dem: OwnedRasterArray, *, slope: bool = True, aspect: bool = True, hillshade: bool = True,
                   azimuth: float = 315.0, altitude: float = 45.0, z_factor: float = 1.0,
                   nodata_mode: str = NODATA_WINDOW, use_gpu: bool | None = None) -> dict[str, OwnedRasterArray]:
    """Slope, aspect and hillshade from one fused pass over the DEM.

    Each result equals what raster_slope / raster_aspect / raster_hillshade
    return for the same DEM; returns a dict with the requested keys.
    """
    _require_gpu(use_gpu)
    t0 = time.perf_counter()
    s, a, h = horn_fused(dem, slope=slope, aspect=aspect, hillshade=hillshade, azimuth=azimuth,
                         altitude=altitude, z_factor=z_factor, nodata_mode=nodata_mode)
    dt = time.perf_counter() - t0
    out = {}
    if s is not None:
        out["slope"] = _record(from_device(_shape_like(dem, s), nodata=dem.nodata, affine=dem.affine, crs=dem.crs),
                               f"gpu_slope_fused {dem.width}x{dem.height}", dt)
    if a is not None:
        out["aspect"] = _record(from_device(_shape_like(dem, a), nodata=dem.nodata, affine=dem.affine, crs=dem.crs),
                                f"gpu_aspect_fused {dem.width}x{dem.height}", dt)
    if h is not None:
        out["hillshade"] = _record(
            from_device(_shape_like(dem, h), nodata=0 if dem.nodata is not None else None, affine=dem.affine,
                        crs=dem.crs),
            f"gpu_hillshade {dem.width}x{dem.height}", dt)
    return out


# ---------------------------------------------------------------------------
# Normalised focal convolution, Gaussian, focal mean
# ---------------------------------------------------------------------------

# "split": tcgen05 split-precision GEMMs (BF16 high parts, F16 low parts; see
# VSR_PREC_SPLIT in vsr.h); "split_bf16" is its earlier name, kept as an alias.
_PRECISION = {"auto": _lib.VSR_PREC_AUTO, "fp32": _lib.VSR_PREC_FP32, "split": _lib.VSR_PREC_SPLIT,
              "split_bf16": _lib.VSR_PREC_SPLIT}


# ---------------------------------------------------------------------------
# Terrain derivatives (TRI, TPI, profile curvature)
# ---------------------------------------------------------------------------

_DERIV_NAMES = {"tri": "TRI", "tpi": "TPI", "curvature": "curvature"}


def derivative_nodata(dem: OwnedRasterArray) -> float:
    """Output nodata of the terrain derivatives: the raster's, else -9999 (algebra.py:3376)."""
    return float(dem.nodata) if dem.nodata is not None else -9999.0


def terrain_derivatives(dem: OwnedRasterArray, *, tri: bool = True, tpi: bool = True, curvature: bool = True,
                        out_dtype=np.float64, out=None):
    """One vsr_terrain_derivatives_bands launch over every band; returns (tri, tpi, curvature) (B, H, W) tensors.

    ``out`` may supply preallocated device tensors (None entries are allocated).
    """
    torch = _torch()
    src, dt = _device_bands(dem)
    B, H, W = src.shape
    kind, ndv = nodata_kind(dem)
    ocode, odt = _out_code(out_dtype)
    o_t, o_p, o_c = out if out is not None else (None, None, None)
    dev = src.device
    mk = lambda o, want: (o if o is not None else torch.empty((B, H, W), dtype=torch_dtype(odt), device=dev)) if want else None  # noqa: E731
    t_t, p_t, c_t = mk(o_t, tri), mk(o_p, tpi), mk(o_c, curvature)
    cx, cy = cellsize(dem.affine)
    lib = _lib.load()
    stream = _stream_handle()
    o_bs, o_p = _shared_layout(t_t, p_t, c_t)
    st = lib.vsr_terrain_derivatives_bands(
        src.data_ptr(), _lib.dtype_code(dt), B, H * W, H, W, W, cx, cy, ndv, kind,
        derivative_nodata(dem),
        t_t.data_ptr() if t_t is not None else None,
        p_t.data_ptr() if p_t is not None else None,
        c_t.data_ptr() if c_t is not None else None,
        ocode, o_bs, o_p, stream,
    )
    _lib.check(st, "vsr_terrain_derivatives_bands")
    return t_t, p_t, c_t


def raster_terrain_derivatives(dem: OwnedRasterArray, *, tri: bool = True, tpi: bool = True,
                               curvature: bool = True, use_gpu: bool | None = None) -> dict[str, OwnedRasterArray]:
    """TRI, TPI and profile curvature from one pass over the DEM.

    Each result equals what raster_tri / raster_tpi / raster_curvature return
    for the same DEM (float64, nodata = the raster's, else -9999); returns a dict
    with the requested keys.
    """
    _require_gpu(use_gpu)
    t0 = time.perf_counter()
    ts = terrain_derivatives(dem, tri=tri, tpi=tpi, curvature=curvature)
    el = time.perf_counter() - t0
    nd = derivative_nodata(dem)
    res = {}
    for key, t in zip(("tri", "tpi", "curvature"), ts):
        if t is None:
            continue
        r = from_device(_shape_like(dem, t), nodata=nd, affine=dem.affine, crs=dem.crs)
        res[key] = _record(r, f"gpu_terrain_{_DERIV_NAMES[key]} {dem.width}x{dem.height}", el)
    return res


def raster_tri(dem: OwnedRasterArray, *, use_gpu: bool | None = None) -> OwnedRasterArray:
    """Terrain Ruggedness Index (mean |z_i - z4| over the 8 neighbours), reference algebra.py:3448-3471."""
    return raster_terrain_derivatives(dem, tri=True, tpi=False, curvature=False, use_gpu=use_gpu)["tri"]


def raster_tpi(dem: OwnedRasterArray, *, use_gpu: bool | None = None) -> OwnedRasterArray:
    """Topographic Position Index (z4 - mean of the 8 neighbours), reference algebra.py:3474-3498."""
    return raster_terrain_derivatives(dem, tri=False, tpi=True, curvature=False, use_gpu=use_gpu)["tpi"]


def raster_curvature(dem: OwnedRasterArray, *, use_gpu: bool | None = None) -> OwnedRasterArray:
    """Profile curvature (Zevenbergen & Thorne 1987), reference algebra.py:3501-3525."""
    return raster_terrain_derivatives(dem, tri=False, tpi=False, curvature=True, use_gpu=use_gpu)["curvature"]


def _precision_code(precision: str) -> int:
    try:
        return _PRECISION[precision]
    except KeyError:
        raise ValueError(f"precision must be one of {sorted(_PRECISION)}, got {precision!r}") from None


def _out_code(out_dtype) -> tuple[int, object]:
    dt = np.dtype(out_dtype)
    if dt == np.float64:
        return _lib.VSR_F64, dt
    if dt == np.float32:
        return _lib.VSR_F32, dt
    raise ValueError(f"out_dtype must be float32 or float64, got {dt}")


def _workspace(nbytes: int, device):
    torch = _torch()
    return torch.empty(max(int(nbytes), 256) + 256, dtype=torch.uint8, device=device)


def _aligned_ptr(t, align: int = 256) -> int:
    p = t.data_ptr()
    return (p + align - 1) // align * align


def convolve_bands(raster: OwnedRasterArray, kernel: np.ndarray, *, precision: str = "auto",
                   out_dtype=np.float64, out=None):
    """One vsr_convolve_bands launch over every band; returns a (B, H, W) device tensor."""
    torch = _torch()
    src, dt = _device_bands(raster)
    B, H, W = src.shape
    kh, kw = kernel.shape
    kind, ndv = nodata_kind(raster)
    nd_out = float(raster.nodata) if raster.nodata is not None else 0.0
    ocode, odt = _out_code(out_dtype)
    dst = out if out is not None else torch.empty((B, H, W), dtype=torch_dtype(odt), device=src.device)
    lib = _lib.load()
    prec = _precision_code(precision)
    nbytes = lib.vsr_convolve_workspace_size(kh, kw, prec)
    ws = _workspace(nbytes, src.device)
    w = np.ascontiguousarray(kernel, dtype=np.float64)
    wp = w.ctypes.data_as(_lib._c.POINTER(_lib._c.c_double))
    o_bs, o_p = _shared_layout(dst)
    st = lib.vsr_convolve_bands(src.data_ptr(), _lib.dtype_code(dt), B, H * W, H, W, W, wp, kh, kw,
                                nd_out if kind == _lib.VSR_NODATA_VALUE else ndv, kind, dst.data_ptr(), ocode,
                                o_bs, o_p, prec, _aligned_ptr(ws), nbytes, _stream_handle())
    _lib.check(st, "vsr_convolve_bands")
    return dst


def raster_convolve(raster: OwnedRasterArray, kernel: np.ndarray, *, precision: str = "auto",
                    out_dtype=np.float64) -> OwnedRasterArray:
    """Nodata-aware normalised 2-D correlation, reference algebra.py:2101-2117.

    Result dtype float64 as in the reference (``out_dtype=np.float32`` halves
    the output bytes); nodata and affine/crs carried over.
    """
    kernel = np.asarray(kernel, dtype=np.float64)
    if kernel.ndim != 2:
        raise ValueError(f"kernel must be 2D, got {kernel.ndim}D")
    _require_gpu(None)
    t0 = time.perf_counter()
    out = convolve_bands(raster, kernel, precision=precision, out_dtype=out_dtype)
    res = from_device(_shape_like(raster, out), nodata=raster.nodata, affine=raster.affine, crs=raster.crs)
    kh, kw = kernel.shape
    return _record(res, f"gpu_convolve {raster.width}x{raster.height} kernel={kw}x{kh}", time.perf_counter() - t0)


def gaussian_kernel_size(sigma: float, kernel_size: int | None) -> int:
    """Reference size rule (algebra.py:2142-2147)."""
    if sigma <= 0:
        raise ValueError(f"sigma must be positive, got {sigma}")
    k = int(2 * np.ceil(3 * sigma) + 1) if kernel_size is None else int(kernel_size)
    if k % 2 == 0:
        k += 1
    return k


def gaussian_bands(raster: OwnedRasterArray, sigma: float, kernel_size: int | None = None, *,
                   precision: str = "auto", out_dtype=np.float64, out=None):
    torch = _torch()
    k = gaussian_kernel_size(sigma, kernel_size)
    src, dt = _device_bands(raster)
    B, H, W = src.shape
    kind, ndv = nodata_kind(raster)
    nd_out = float(raster.nodata) if raster.nodata is not None else 0.0
    ocode, odt = _out_code(out_dtype)
    dst = out if out is not None else torch.empty((B, H, W), dtype=torch_dtype(odt), device=src.device)
    lib = _lib.load()
    prec = _precision_code(precision)
    # the tensor-core line passes (split, and auto on 8/16-bit integer rasters
    # from k = 35) keep the row pass's sums in about 8 bytes per pixel of
    # workspace; room for every band's sums runs the stack in one launch per pass
    nbytes = lib.vsr_gaussian_bands_workspace_bytes(B, H, W, _lib.dtype_code(dt), float(sigma), k, prec)
    ws = _workspace(nbytes, src.device)
    stream = _stream_handle()
    # all bands in one launch (band-first stack, H*W elements apart)
    st = lib.vsr_gaussian_bands(src.data_ptr(), _lib.dtype_code(dt), B, H * W, H, W, W, float(sigma), k,
                                nd_out if kind == _lib.VSR_NODATA_VALUE else ndv, kind, dst.data_ptr(), ocode,
                                H * W, W, prec, _aligned_ptr(ws), nbytes, stream)
    _lib.check(st, "vsr_gaussian_bands")
    return dst


def raster_gaussian_filter(raster: OwnedRasterArray, sigma: float, *, kernel_size: int | None = None,
                           precision: str = "auto", out_dtype=np.float64) -> OwnedRasterArray:
    """Gaussian filter, reference algebra.py:2120-2154 (ValueError for sigma <= 0)."""
    k = gaussian_kernel_size(sigma, kernel_size)
    _require_gpu(None)
    t0 = time.perf_counter()
    out = gaussian_bands(raster, sigma, k, precision=precision, out_dtype=out_dtype)
    res = from_device(_shape_like(raster, out), nodata=raster.nodata, affine=raster.affine, crs=raster.crs)
    return _record(res, f"gpu_convolve {raster.width}x{raster.height} kernel={k}x{k} gaussian sigma={sigma}",
                   time.perf_counter() - t0)


def _parse_radius(radius) -> tuple[int, int]:
    """(radius_y, radius_x) from an int or a 2-tuple (algebra.py:3022-3035)."""
    if isinstance(radius, (list, tuple)):
        if len(radius) != 2:
            raise ValueError(f"radius tuple must have 2 elements, got {len(radius)}")
        return int(radius[0]), int(radius[1])
    r = int(radius)
    return r, r


def focal_mean_bands(raster: OwnedRasterArray, ry: int, rx: int, *, out_dtype=np.float64, out=None):
    torch = _torch()
    src, dt = _device_bands(raster)
    B, H, W = src.shape
    kind, ndv = nodata_kind(raster)
    nd_out = float(raster.nodata) if raster.nodata is not None else 0.0
    ocode, odt = _out_code(out_dtype)
    dst = out if out is not None else torch.empty((B, H, W), dtype=torch_dtype(odt), device=src.device)
    lib = _lib.load()
    stream = _stream_handle()
    st = lib.vsr_focal_mean_bands(src.data_ptr(), _lib.dtype_code(dt), B, H * W, H, W, W, ry, rx,
                                  nd_out if kind == _lib.VSR_NODATA_VALUE else ndv, kind, dst.data_ptr(), ocode,
                                  H * W, W, stream)
    _lib.check(st, "vsr_focal_mean_bands")
    return dst


def raster_focal_mean(raster: OwnedRasterArray, radius=1, *, use_gpu: bool | None = None,
                      out_dtype=np.float64) -> OwnedRasterArray:
    """Focal mean over a (2ry+1) x (2rx+1) window, reference algebra.py:3582-3604."""
    ry, rx = _parse_radius(radius)
    _require_gpu(use_gpu)
    t0 = time.perf_counter()
    out = focal_mean_bands(raster, ry, rx, out_dtype=out_dtype)
    res = from_device(_shape_like(raster, out), nodata=raster.nodata, affine=raster.affine, crs=raster.crs)
    return _record(res, f"gpu_focal_mean {raster.width}x{raster.height} radius=({ry},{rx})", time.perf_counter() - t0)


def focal_stat_bands(raster: OwnedRasterArray, stat: str, ry: int, rx: int, *, out_dtype=np.float64, out=None):
    """One focal statistic over every band in one launch; (B, H, W) device tensor."""
    torch = _torch()
    if stat not in _lib.VSR_STAT:
        raise ValueError(f"unknown focal statistic {stat!r}; expected one of {sorted(_lib.VSR_STAT)}")
    src, dt = _device_bands(raster)
    B, H, W = src.shape
    kind, ndv = nodata_kind(raster)
    nd_out = float(raster.nodata) if raster.nodata is not None else 0.0
    ocode, odt = _out_code(out_dtype)
    dst = out if out is not None else torch.empty((B, H, W), dtype=torch_dtype(odt), device=src.device)
    lib = _lib.load()
    st = lib.vsr_focal_stat_bands(src.data_ptr(), _lib.dtype_code(dt), B, H * W, H, W, W, _lib.VSR_STAT[stat], ry, rx,
                                  nd_out if kind == _lib.VSR_NODATA_VALUE else ndv, kind, dst.data_ptr(), ocode,
                                  H * W, W, _stream_handle())
    _lib.check(st, "vsr_focal_stat_bands")
    return dst


def _raster_focal(raster: OwnedRasterArray, stat: str, radius, use_gpu, out_dtype) -> OwnedRasterArray:
    ry, rx = _parse_radius(radius)
    _require_gpu(use_gpu)
    t0 = time.perf_counter()
    out = focal_stat_bands(raster, stat, ry, rx, out_dtype=out_dtype)
    res = from_device(_shape_like(raster, out), nodata=raster.nodata, affine=raster.affine, crs=raster.crs)
    return _record(res, f"gpu_focal_{stat} {raster.width}x{raster.height} radius=({ry},{rx})",
                   time.perf_counter() - t0)


def raster_focal_min(raster: OwnedRasterArray, radius=1, *, use_gpu: bool | None = None,
                     out_dtype=np.float64) -> OwnedRasterArray:
    """Focal minimum, reference algebra.py:3531-3554 (CPU semantics :3041-3059)."""
    return _raster_focal(raster, "min", radius, use_gpu, out_dtype)


def raster_focal_max(raster: OwnedRasterArray, radius=1, *, use_gpu: bool | None = None,
                     out_dtype=np.float64) -> OwnedRasterArray:
    """Focal maximum, reference algebra.py:3557-3579 (CPU semantics :3062-3081)."""
    return _raster_focal(raster, "max", radius, use_gpu, out_dtype)


def raster_focal_std(raster: OwnedRasterArray, radius=1, *, use_gpu: bool | None = None,
                     out_dtype=np.float64) -> OwnedRasterArray:
    """Focal population standard deviation, reference algebra.py:3607-3631 (:3104-3122)."""
    return _raster_focal(raster, "std", radius, use_gpu, out_dtype)


def raster_focal_range(raster: OwnedRasterArray, radius=1, *, use_gpu: bool | None = None,
                       out_dtype=np.float64) -> OwnedRasterArray:
    """Focal range (max - min), reference algebra.py:3634-3656 (:3125-3143)."""
    return _raster_focal(raster, "range", radius, use_gpu, out_dtype)


def raster_focal_variety(raster: OwnedRasterArray, radius=1, *, use_gpu: bool | None = None,
                         out_dtype=np.float64) -> OwnedRasterArray:
    """Number of distinct values in the window, reference algebra.py:3659-3684 (:3146-3163)."""
    return _raster_focal(raster, "variety", radius, use_gpu, out_dtype)
