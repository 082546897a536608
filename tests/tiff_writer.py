"""Minimal GeoTIFF writer for the decode tests (test infrastructure).

Writes classic TIFF (or BigTIFF) in either byte order, as strips or tiles,
uncompressed or DEFLATE, with predictor 1, 2 (horizontal differencing) or 3
(floating-point byte planes), pixel-interleaved or planar-separate samples,
and the GeoTIFF tags the reader uses (ModelPixelScale, ModelTiepoint or
ModelTransformation, GeoKeyDirectory with an EPSG code, GDAL_NODATA).  The
encoding follows the TIFF 6.0 specification and Adobe's floating-point
predictor note; the decode tests check read(write(x)) == x.
"""

from __future__ import annotations

import struct
import zlib

import numpy as np


def _predict(block: np.ndarray, predictor: int, big_endian: bool) -> bytes:
    """Encode one chunk (rows, cols, samples) with the predictor."""
    rows, cols, ns = block.shape
    if predictor == 1:
        a = block.astype(block.dtype.newbyteorder(">" if big_endian else "<"))
        return a.tobytes()
    if predictor == 2:  # differences of consecutive samples, modulo the sample width
        ut = np.dtype(f"u{block.dtype.itemsize}")
        u = np.ascontiguousarray(block).view(ut)
        d = u.copy()
        d[:, 1:, :] = u[:, 1:, :] - u[:, :-1, :]
        return d.astype(ut.newbyteorder(">" if big_endian else "<")).tobytes()
    # predictor 3: per row, bytes of each value big-endian, split into planes
    # (most significant first), then byte-wise differencing over the row
    esz = block.dtype.itemsize
    res = bytearray()
    for r in range(rows):
        vals = block[r].reshape(-1).astype(block.dtype.newbyteorder(">"))
        b = np.frombuffer(vals.tobytes(), np.uint8).reshape(-1, esz)
        planes = b.T.reshape(-1).astype(np.int32)
        diff = planes.copy()
        diff[1:] = (planes[1:] - planes[:-1]) & 0xFF
        res += diff.astype(np.uint8).tobytes()
    return bytes(res)


def write_geotiff(path, data: np.ndarray, *, tile: tuple[int, int] | None = None, rows_per_strip: int | None = None,
                  compress: bool = False, predictor: int = 1, big_endian: bool = False, planar: bool = False,
                  bigtiff: bool = False, affine=(10.0, 0.0, 500000.0, 0.0, -10.0, 4000000.0), epsg: int | None = 32633,
                  nodata=None, transformation: bool = False) -> None:
    """Write ``data`` ((H, W) or (B, H, W)) as a GeoTIFF."""
    a = np.asarray(data)
    if a.ndim == 2:
        a = a[None]
    B, H, W = a.shape
    e = ">" if big_endian else "<"
    esz = a.dtype.itemsize
    fmt = {"u": 1, "i": 2, "f": 3}[a.dtype.kind]
    chunks = []
    if tile:
        tw, th = tile
        across, down = -(-W // tw), -(-H // th)
        planes = range(B) if planar else [None]
        for p in planes:
            for ty in range(down):
                for tx in range(across):
                    blk = np.zeros((th, tw, 1 if planar else B), a.dtype)
                    src = a[p:p + 1] if planar else a
                    part = src[:, ty * th:(ty + 1) * th, tx * tw:(tx + 1) * tw]
                    blk[: part.shape[1], : part.shape[2], :] = np.moveaxis(part, 0, -1)
                    chunks.append(blk)
    else:
        rps = rows_per_strip or H
        planes = range(B) if planar else [None]
        for p in planes:
            for y0 in range(0, H, rps):
                src = a[p:p + 1] if planar else a
                chunks.append(np.ascontiguousarray(np.moveaxis(src[:, y0:y0 + rps, :], 0, -1)))
    payload = []
    for blk in chunks:
        raw = _predict(blk, predictor, big_endian)
        payload.append(zlib.compress(raw, 6) if compress else raw)
    entries = []

    def tag(t, typ, values):
        entries.append((t, typ, values))

    tag(256, 4, [W])
    tag(257, 4, [H])
    tag(258, 3, [8 * esz] * B)
    tag(259, 3, [8 if compress else 1])
    tag(262, 3, [1])
    tag(277, 3, [B])
    tag(284, 3, [2 if planar else 1])
    if predictor != 1:
        tag(317, 3, [predictor])
    tag(339, 3, [fmt] * B)
    if tile:
        tag(322, 3, [tile[0]])
        tag(323, 3, [tile[1]])
        tag(324, 16 if bigtiff else 4, [0] * len(payload))  # patched below
        tag(325, 16 if bigtiff else 4, [len(p) for p in payload])
    else:
        tag(273, 16 if bigtiff else 4, [0] * len(payload))
        tag(278, 4, [rows_per_strip or H])
        tag(279, 16 if bigtiff else 4, [len(p) for p in payload])
    if transformation:
        m = [affine[0], affine[1], 0.0, affine[2], affine[3], affine[4], 0.0, affine[5], 0, 0, 0, 0, 0, 0, 0, 1.0]
        tag(34264, 12, m)
    else:
        tag(33550, 12, [affine[0], -affine[4], 0.0])
        tag(33922, 12, [0.0, 0.0, 0.0, affine[2], affine[5], 0.0])
    if epsg is not None:
        tag(34735, 3, [1, 1, 0, 1, 3072 if epsg >= 20000 else 2048, 0, 1, epsg])
    if nodata is not None:
        tag(42113, 2, str(nodata).encode() + b"\0")
    entries.sort(key=lambda x: x[0])
    codes = {3: "H", 4: "I", 12: "d", 16: "Q", 2: "s"}
    sizes = {3: 2, 4: 4, 12: 8, 16: 8, 2: 1}
    inline = 8 if bigtiff else 4
    ent = 20 if bigtiff else 12
    head = 16 if bigtiff else 8
    ifd_size = (8 if bigtiff else 2) + ent * len(entries) + (8 if bigtiff else 4)
    # layout: header | IFD | out-of-line values | chunk data
    extra = bytearray()
    extra_off = head + ifd_size
    vals = []
    for t, typ, v in entries:
        n = len(v)
        nbytes = sizes[typ] * n
        vals.append((t, typ, v, n, nbytes))
    ool_pos = {}
    for t, typ, v, n, nbytes in vals:
        if nbytes > inline:
            ool_pos[t] = extra_off + len(extra)
            extra += bytes(nbytes)
            while len(extra) % 8:
                extra += b"\0"
    data_off = extra_off + len(extra)
    offs = []
    pos = data_off
    for p in payload:
        offs.append(pos)
        pos += len(p)
    for i, (t, typ, v, n, nbytes) in enumerate(vals):
        if t in (273, 324):
            vals[i] = (t, typ, offs, n, nbytes)

    def pack(typ, v):
        if typ == 2:
            return bytes(v)
        return struct.pack(e + codes[typ] * len(v), *v)

    out = bytearray()
    if bigtiff:
        out += (b"MM" if big_endian else b"II") + struct.pack(e + "HHHQ", 43, 8, 0, head)
        out += struct.pack(e + "Q", len(vals))
    else:
        out += (b"MM" if big_endian else b"II") + struct.pack(e + "HI", 42, head)
        out += struct.pack(e + "H", len(vals))
    for t, typ, v, n, nbytes in vals:
        body = pack(typ, v)
        if nbytes > inline:
            extra[ool_pos[t] - extra_off: ool_pos[t] - extra_off + nbytes] = body
            ptr = struct.pack(e + ("Q" if bigtiff else "I"), ool_pos[t])
        else:
            ptr = body + bytes(inline - len(body))
        out += struct.pack(e + ("HHQ" if bigtiff else "HHI"), t, typ, n) + ptr
    out += bytes(8 if bigtiff else 4)  # no next IFD
    out += extra
    for p in payload:
        out += p
    with open(path, "wb") as f:
        f.write(out)
