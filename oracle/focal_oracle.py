"""Float64 restatement of the reference's focal-stencil algorithms (oracle only).

TEST INFRASTRUCTURE: used by tests, smoke() and the CPU baseline of bench.py
as the checker; never by the product path.

Every function cites the reference file:line it restates (paths relative to
the vibespatial-raster 0.1.7 source tree).  The numpy operation sequence
follows the reference's CPU code so that timing it is a fair stand-in for
timing the reference itself (same float64 temporaries, same single-threaded
ufunc passes).
"""

from __future__ import annotations

import warnings

import numpy as np

# ---------------------------------------------------------------------------
# Shared conventions
# ---------------------------------------------------------------------------


def cellsize_from_affine(affine) -> tuple[float, float]:
    """|a| and |e| of a GDAL affine, 1.0 where zero.

    Reference: src/vibespatial/raster/algebra.py:2182-2183 (slope/aspect) and
    :2573-2574 (hillshade).  Rotation terms b and d are ignored.
    """
    cx = abs(float(affine[0])) if float(affine[0]) != 0 else 1.0
    cy = abs(float(affine[4])) if float(affine[4]) != 0 else 1.0
    return cx, cy


def nodata_mask(data: np.ndarray, nodata) -> np.ndarray:
    """Boolean nodata mask, buffers.py:304-328 (``OwnedRasterArray.nodata_mask``).

    ``None`` -> all False; NaN -> ``isnan`` for float data and all False (with a
    warning) for integer data; otherwise ``data == nodata``.
    """
    if nodata is None:
        return np.zeros(data.shape, bool)
    if np.isnan(nodata):
        if not np.issubdtype(data.dtype, np.floating):
            warnings.warn("NaN nodata on integer data: mask is all False", stacklevel=2)
            return np.zeros(data.shape, bool)
        return np.isnan(data)
    return data == nodata


def terrain_out_dtype(in_dtype) -> np.dtype:
    """Slope/aspect output dtype rule, algebra.py:2419-2427 / 2444-2445.

    Float inputs other than float64 are cast back to their own dtype; integer
    inputs keep the float64 the computation produced.
    """
    dt = np.dtype(in_dtype)
    if np.issubdtype(dt, np.floating) and dt != np.float64:
        return dt
    return np.dtype(np.float64)


def _shifted3x3(padded: np.ndarray):
    """The nine views of an edge-padded array, row-major (nw, n, ne, w, c, e, sw, s, se)."""
    h = padded.shape[0] - 2
    w = padded.shape[1] - 2
    return [padded[dy : dy + h, dx : dx + w] for dy in range(3) for dx in range(3)]


def _horn(padded: np.ndarray, cell_x: float, cell_y: float, z_factor: float | None):
    """Horn 3x3 gradients on an edge-padded float64 array.

    algebra.py:2215-2216 (slope/aspect, no z factor) and :2581-2597 (hillshade,
    times z_factor).  Window letters: a b c / d e f / g h i.
    """
    a, b, c, d, _e, f, g, h, i = _shifted3x3(padded)
    dzdx = ((c + 2.0 * f + i) - (a + 2.0 * d + g)) / (8.0 * cell_x)
    dzdy = ((g + 2.0 * h + i) - (a + 2.0 * b + c)) / (8.0 * cell_y)
    if z_factor is not None:
        dzdx = dzdx * z_factor
        dzdy = dzdy * z_factor
    return dzdx, dzdy


# ---------------------------------------------------------------------------
# Slope / aspect
# ---------------------------------------------------------------------------


def slope_aspect(data: np.ndarray, affine, nodata, *, compute_slope=True, compute_aspect=True):
    """Reference CPU slope/aspect, algebra.py:2162-2249 (``_cpu_slope_aspect``).

    Returns float64 (slope_deg, aspect_deg); either is None when not asked for.
    Nodata: the mask is ``data == nodata`` (so a NaN nodata never matches and
    NaN propagates through the arithmetic instead, algebra.py:2188-2189); it is
    edge-padded and any pixel whose 3x3 window touches it is set to nodata
    (algebra.py:2219-2247).  Aspect is ``(90 - degrees(atan2(-q, p))) % 360``
    (algebra.py:2240-2243).  The caller casts to ``terrain_out_dtype``.
    """
    z = np.asarray(data).astype(np.float64)
    if z.ndim == 3:
        z = z[0]
    cell_x, cell_y = cellsize_from_affine(affine)
    nd_val = float(nodata) if nodata is not None else None
    if nd_val is not None:
        mask = z == nd_val
    else:
        mask = np.zeros(z.shape, bool)
    padded = np.pad(z, 1, mode="edge")
    mpad = np.pad(mask, 1, mode="edge")
    dzdx, dzdy = _horn(padded, cell_x, cell_y, None)
    ring = np.zeros(z.shape, bool)
    for v in _shifted3x3(mpad):
        ring |= v
    slope = aspect = None
    if compute_slope:
        slope = np.degrees(np.arctan(np.sqrt(dzdx**2 + dzdy**2)))
        if nd_val is not None:
            slope[ring] = nd_val
    if compute_aspect:
        aspect = (90.0 - np.degrees(np.arctan2(-dzdy, dzdx))) % 360.0
        if nd_val is not None:
            aspect[ring] = nd_val
    return slope, aspect


def nodata_ring(data: np.ndarray, nodata) -> np.ndarray:
    """Pixels that the reference CPU slope/aspect set to nodata.

    algebra.py:2186-2228: mask ``data == nodata`` (float64 compare; NaN never
    matches), edge-padded, OR-ed over the 3x3 window.
    """
    z = np.asarray(data).astype(np.float64)
    if nodata is None:
        return np.zeros(z.shape, bool)
    m = np.pad(z == float(nodata), 1, mode="edge")
    ring = np.zeros(z.shape, bool)
    for v in _shifted3x3(m):
        ring |= v
    return ring


def slope_aspect_center_only(data: np.ndarray, affine, nodata):
    """Reference GPU slope/aspect semantics, kernels/focal.py:173-283.

    Same Horn arithmetic with edge clamping (focal.py:163-171), but the nodata
    test looks only at the centre pixel (focal.py:245-250; mask from
    ``device_nodata_mask``, buffers.py:487-510, so NaN nodata does mask) and
    neighbours' raw values enter the gradient.  Aspect uses C ``fmod`` plus a
    +360 correction (focal.py:275-279), which equals Python's ``%`` here.
    """
    z = np.asarray(data).astype(np.float64)
    cell_x, cell_y = cellsize_from_affine(affine)
    padded = np.pad(z, 1, mode="edge")
    dzdx, dzdy = _horn(padded, cell_x, cell_y, None)
    slope = np.degrees(np.arctan(np.sqrt(dzdx**2 + dzdy**2)))
    aspect = np.fmod(90.0 - np.degrees(np.arctan2(-dzdy, dzdx)), 360.0)
    aspect = np.where(aspect < 0.0, aspect + 360.0, aspect)
    if nodata is not None:
        m = nodata_mask(z, nodata)
        slope[m] = float(nodata)
        aspect[m] = float(nodata)
    return slope, aspect


# ---------------------------------------------------------------------------
# Hillshade
# ---------------------------------------------------------------------------


def hillshade(data: np.ndarray, affine, nodata, *, azimuth=315.0, altitude=45.0, z_factor=1.0):
    """Reference CPU hillshade, algebra.py:2543-2629 (``_hillshade_cpu``).

    hs = cos(zen) cos(slope) + sin(zen) sin(slope) cos(az - atan2(-q, p)),
    clipped to [0, 1], ``uint8(hs * 255 + 0.5)`` (truncating cast).  Nodata:
    the ``nodata_mask`` (isnan for NaN nodata) dilated over the in-bounds 3x3
    window (zero-padded, algebra.py:2610-2619) sets the output to 0.
    Returns (uint8 array, output nodata: 0 if the input has nodata else None).
    """
    z = np.asarray(data).astype(np.float64)
    if z.ndim == 3:
        z = z[0]
    cell_x, cell_y = cellsize_from_affine(affine)
    padded = np.pad(z, 1, mode="edge")
    dzdx, dzdy = _horn(padded, cell_x, cell_y, float(z_factor))
    slope = np.arctan(np.sqrt(dzdx**2 + dzdy**2))
    aspect = np.arctan2(-dzdy, dzdx)
    zen = np.radians(90.0 - altitude)
    az = np.radians(azimuth)
    hs = np.cos(zen) * np.cos(slope) + np.sin(zen) * np.sin(slope) * np.cos(az - aspect)
    hs = np.clip(hs, 0.0, 1.0)
    with np.errstate(invalid="ignore"):
        scaled = hs * 255.0 + 0.5
        out = np.where(np.isnan(scaled), 0.0, scaled).astype(np.uint8)
    if nodata is None:
        return out, None
    m = nodata_mask(np.asarray(data) if np.asarray(data).ndim == 2 else np.asarray(data)[0], nodata)
    mp = np.pad(m, 1, mode="constant", constant_values=False)
    ring = np.zeros(z.shape, bool)
    for v in _shifted3x3(mp):
        ring |= v
    out[ring] = 0
    return out, 0


# ---------------------------------------------------------------------------
# Normalised focal convolution / Gaussian
# ---------------------------------------------------------------------------


TRI, TPI, CURVATURE = "tri", "tpi", "curvature"


def terrain_derivative(data: np.ndarray, affine, nodata, kind: str) -> tuple[np.ndarray, float]:
    """Reference CPU terrain derivative, algebra.py:3352-3445 (``_terrain_derivative_cpu``).

    Returns (float64 output, output nodata value).  On the edge-padded float64
    window z0..z8 (row-major, z4 the centre): TRI = mean |z_i - z4| over the 8
    neighbours (Riley 1999), TPI = z4 - mean of the neighbours, profile
    curvature (Zevenbergen & Thorne 1987) = -2 (D + E) 100 with
    D = ((z3 + z5)/2 - z4) / cx^2, E = ((z1 + z7)/2 - z4) / cy^2.  Border pixels
    and every pixel whose 3x3 window (constant-padded mask) touches nodata are
    set to the output nodata: the raster's nodata, else -9999.0.
    """
    z = np.asarray(data).astype(np.float64)
    if z.ndim == 3:
        z = z[0]
    h, w = z.shape
    nd_out = float(nodata) if nodata is not None else -9999.0
    p = np.pad(z, 1, mode="edge")
    z0, z1, z2, z3, z4, z5, z6, z7, z8 = _shifted3x3(p)
    if kind == TRI:
        res = (np.abs(z0 - z4) + np.abs(z1 - z4) + np.abs(z2 - z4) + np.abs(z3 - z4) + np.abs(z5 - z4)
               + np.abs(z6 - z4) + np.abs(z7 - z4) + np.abs(z8 - z4)) / 8.0
    elif kind == TPI:
        res = z4 - (z0 + z1 + z2 + z3 + z5 + z6 + z7 + z8) / 8.0
    elif kind == CURVATURE:
        cx, cy = cellsize_from_affine(affine)
        d = ((z3 + z5) / 2.0 - z4) / (cx * cx)
        e = ((z1 + z7) / 2.0 - z4) / (cy * cy)
        res = -2.0 * (d + e) * 100.0
    else:
        raise ValueError(f"unknown terrain derivative {kind!r}")
    out = np.full((h, w), nd_out, np.float64)
    out[1:-1, 1:-1] = res[1:-1, 1:-1]
    if nodata is not None:
        m = np.pad(nodata_mask(z, nodata), 1, mode="constant", constant_values=False)
        ring = np.zeros((h, w), bool)
        for v in _shifted3x3(m):
            ring |= v
        out[ring] = nd_out
    return out, nd_out


def gaussian_weights(sigma: float, kernel_size: int | None = None) -> np.ndarray:
    """Reference Gaussian weights, algebra.py:2120-2152 (``raster_gaussian_filter``).

    Default size ``int(2*ceil(3*sigma)+1)``, even sizes bumped to odd,
    ``g = exp(-0.5 (ax/sigma)^2)`` with ``ax = arange(k) - k//2``,
    ``K = outer(g, g) / sum``.  Raises ValueError for sigma <= 0.
    """
    if sigma <= 0:
        raise ValueError(f"sigma must be positive, got {sigma}")
    k = int(2 * np.ceil(3 * sigma) + 1) if kernel_size is None else int(kernel_size)
    if k % 2 == 0:
        k += 1
    ax = np.arange(k) - k // 2
    g = np.exp(-0.5 * (ax / sigma) ** 2)
    w = np.outer(g, g)
    return w / w.sum()


def convolve_normalized(data: np.ndarray, weights: np.ndarray, nodata) -> np.ndarray:
    """Nodata-aware normalised correlation, the reference kernel's arithmetic.

    Restates kernels/focal.py:36-146 (``convolve_normalized``) as launched by
    algebra.py:1961-2098: correlation orientation (no kernel flip), tap
    (i, j) reads v[y + i - kh//2, x + j - kw//2]; out-of-bounds taps are
    skipped (focal.py:127-130); nodata taps contribute neither to the sum nor
    to the weight sum; a nodata centre, or a weight sum <= 0, gives the nodata
    value (0.0 when the raster has none, algebra.py:2003).  float64 result.

    The kernel masks by multiplication (``val * w * valid``, focal.py:140), so
    a NaN value anywhere in the in-bounds window -- nodata or not, whatever
    its weight -- makes the sum NaN (NaN * 0 = NaN); with NaN nodata every
    pixel whose window touches a hole therefore comes out NaN.  That is kept.

    Evaluated with float64 ``scipy.ndimage.correlate`` passes (constant 0
    outside the raster, which skips out-of-bounds taps exactly; scipy's
    centre for an even size k is index k//2, the same as pad = k//2 in the
    reference) plus a box pass that marks the NaN-poisoned windows.
    """
    from scipy.ndimage import correlate

    z = np.asarray(data).astype(np.float64)
    w = np.asarray(weights, dtype=np.float64)
    valid = ~nodata_mask(np.asarray(data), nodata) if nodata is not None else np.ones(z.shape, bool)
    with np.errstate(invalid="ignore"):
        vz = z * valid
    nan_tap = np.isnan(vz)
    num = correlate(np.where(nan_tap, 0.0, vz), w, mode="constant", cval=0.0)
    den = correlate(valid.astype(np.float64), w, mode="constant", cval=0.0)
    poisoned = correlate(nan_tap.astype(np.float64), np.ones(w.shape), mode="constant", cval=0.0) > 0.5
    nd_val = float(nodata) if nodata is not None else 0.0
    with np.errstate(invalid="ignore", divide="ignore"):
        out = np.where(den > 0.0, num / np.where(den > 0.0, den, 1.0), nd_val)
    out[poisoned & (den > 0.0)] = np.nan
    out[~valid] = nd_val
    return out


def convolve_normalized_loop(data: np.ndarray, weights: np.ndarray, nodata) -> np.ndarray:
    """Literal per-pixel loop over kernels/focal.py:101-145 (small inputs only)."""
    z = np.asarray(data).astype(np.float64)
    w = np.asarray(weights, dtype=np.float64)
    H, W = z.shape
    kh, kw = w.shape
    py, px = kh // 2, kw // 2
    nd = nodata_mask(np.asarray(data), nodata) if nodata is not None else np.zeros(z.shape, bool)
    nd_val = float(nodata) if nodata is not None else 0.0
    out = np.empty((H, W), np.float64)
    for y in range(H):
        for x in range(W):
            if nd[y, x]:
                out[y, x] = nd_val
                continue
            s = 0.0
            ws = 0.0
            for i in range(kh):
                r = y + i - py
                if r < 0 or r >= H:
                    continue
                for j in range(kw):
                    c = x + j - px
                    if c < 0 or c >= W:
                        continue
                    valid = 0.0 if nd[r, c] else 1.0
                    s += z[r, c] * w[i, j] * valid
                    ws += w[i, j] * valid
            out[y, x] = s / ws if ws > 0.0 else nd_val
    return out


# ---------------------------------------------------------------------------
# Focal mean
# ---------------------------------------------------------------------------


FOCAL_STATS = ("min", "max", "mean", "std", "range", "variety")


def focal_stat(data: np.ndarray, radius_y: int, radius_x: int, nodata, stat: str) -> np.ndarray:
    """Reference CPU focal statistics, algebra.py:3041-3164 (``_focal_{stat}_cpu``) via
    ``_focal_stat_cpu`` (:3177-3213).  float64.

    Over the in-bounds taps of the (2ry+1) x (2rx+1) window (out-of-bounds
    taps are the placeholder):
      min / max  nodata -> +inf / -inf placeholders, excluded with every tap
                 equal to the placeholder (valid +-inf data too); NaN data
                 propagates;
      mean, std (population), range, variety (count of distinct values)
                 nodata -> NaN placeholder, excluded with NaN data.
    A window with no valid tap gives the nodata value (0.0 when the raster has
    none, :3196) -- 0.0 for std and variety; a nodata centre gives the nodata
    value.  Evaluated on sliding-window views (mean and std sum in another
    order than the reference: agreement within ~1e-13 relative).
    """
    from numpy.lib.stride_tricks import sliding_window_view

    if stat not in FOCAL_STATS:
        raise ValueError(f"unknown focal statistic {stat!r}")
    z = np.asarray(data).astype(np.float64)
    if z.ndim == 3:
        z = z[0]
    nd = nodata_mask(np.asarray(data), nodata) if nodata is not None else np.zeros(z.shape, bool)
    nd_val = float(nodata) if nodata is not None else 0.0
    ph = {"min": np.inf, "max": -np.inf}.get(stat, np.nan)
    work = np.where(nd, ph, z)
    pad = np.pad(work, ((radius_y, radius_y), (radius_x, radius_x)), mode="constant", constant_values=ph)
    win = sliding_window_view(pad, (2 * radius_y + 1, 2 * radius_x + 1)).reshape(z.shape + (-1,))
    with np.errstate(invalid="ignore"):
        if stat in ("min", "max"):
            excl = win == ph
            nvalid = (~excl).sum(axis=-1)
            has_nan = np.isnan(win).any(axis=-1)
            fill = np.where(excl | np.isnan(win), ph, win)
            out = fill.min(axis=-1) if stat == "min" else fill.max(axis=-1)
            out = np.where(has_nan, np.nan, out)
            out = np.where(nvalid > 0, out, nd_val)
        else:
            ok = ~np.isnan(win)
            nvalid = ok.sum(axis=-1)
            if stat == "mean":
                out = np.where(nvalid > 0, np.nanmean(np.where(nvalid[..., None] > 0, win, 0.0), axis=-1), nd_val)
            elif stat == "std":
                out = np.where(nvalid > 0, np.nanstd(np.where(nvalid[..., None] > 0, win, 0.0), axis=-1), 0.0)
            elif stat == "range":
                lo = np.where(ok, win, np.inf).min(axis=-1)
                hi = np.where(ok, win, -np.inf).max(axis=-1)
                out = np.where(nvalid > 0, hi - lo, nd_val)
            else:  # variety: distinct valid values (NaN sorts last)
                srt = np.sort(win, axis=-1)
                k = np.arange(1, srt.shape[-1])
                new = (srt[..., 1:] != srt[..., :-1]) & (k < nvalid[..., None])
                out = np.where(nvalid > 0, 1.0 + new.sum(axis=-1), 0.0)
    out = out.astype(np.float64)
    if nodata is not None:
        out[nd] = nd_val
    return out


def focal_mean(data: np.ndarray, radius_y: int, radius_x: int, nodata) -> np.ndarray:
    """Reference focal mean, algebra.py:3083-3101 (``_focal_mean_cpu``) via :3177-3230.

    Mean of the in-bounds, non-nodata values of the (2ry+1) x (2rx+1) window
    (``generic_filter`` with cval=NaN, nodata set to NaN first); a window with
    no valid value gives the nodata value (0.0 when the raster has none,
    algebra.py:3196); a nodata centre gives the nodata value.  float64.
    Evaluated exactly as sum / count with float64 box correlations.
    """
    from scipy.ndimage import correlate

    z = np.asarray(data).astype(np.float64)
    nd = nodata_mask(np.asarray(data), nodata) if nodata is not None else np.zeros(z.shape, bool)
    valid = ~nd & ~np.isnan(z)
    box = np.ones((2 * radius_y + 1, 2 * radius_x + 1))
    s = correlate(np.where(valid, z, 0.0), box, mode="constant", cval=0.0)
    n = correlate(valid.astype(np.float64), box, mode="constant", cval=0.0)
    nd_val = float(nodata) if nodata is not None else 0.0
    with np.errstate(invalid="ignore", divide="ignore"):
        out = np.where(n > 0, s / np.where(n > 0, n, 1.0), nd_val)
    if nodata is not None:
        out[nd] = nd_val
    return out
