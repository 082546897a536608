"""Seeded synthetic rasters of the benchmark shapes (no public dataset exists).

* ``fbm_dem``       -- fractional-Brownian surface: a sum of value-noise
                       octaves (bilinear upsampling of seeded uniform grids,
                       frequency doubling, amplitude 2^(-H o) with Hurst H),
                       rescaled to [lo, hi] metres.
* ``terrain_2048``  -- 2048 x 2048 float32, 0-3000 m, 30 m cells, -9999 on 1 %
                       of pixels chosen uniformly (seed 0).
* ``terrain_16k``   -- 16384 x 16384 float32, 0-4500 m, 10 m cells, -9999 in
                       200 disc holes of radius U[5, 80] px (seed 1).
* ``trend_noise``   -- U[0, 1) noise plus a 0-100 row-major linear trend
                       (seed 2) for the focal convolution workloads.
* ``tile_batch``    -- many DEM tiles with log-uniform sides, per-tile cell
                       size U[1, 90] m and per-tile nodata (-9999 or NaN) on
                       U[0, 5] % of pixels (seed 3).
* ``gamma_stack``   -- B bands of uint16 gamma(k=2, theta=800) clipped to
                       [0, 10000] with 3 % zeros as nodata (seed 4).

Generation runs with torch on the requested device (random draws on the CPU
generator, so a seed gives the same grids on every machine).
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


def _torch():
    import torch

    return torch


def fbm_dem(height: int, width: int, *, seed: int, lo: float, hi: float, octaves: int = 8,
            hurst: float = 0.8, base_cells: int = 4, device="cpu"):
    torch = _torch()
    import torch.nn.functional as F

    g = torch.Generator().manual_seed(seed)
    acc = torch.zeros((height, width), dtype=torch.float32, device=device)
    for o in range(octaves):
        n = base_cells * (2**o) + 1
        grid = torch.rand((1, 1, n, n), generator=g, dtype=torch.float32).to(device)
        up = F.interpolate(grid, size=(height, width), mode="bilinear", align_corners=True)[0, 0]
        acc.add_(up, alpha=2.0 ** (-hurst * o))
        del up
    mn, mx = acc.min(), acc.max()
    acc.sub_(mn).mul_((hi - lo) / float(mx - mn)).add_(lo)
    return acc


@dataclass
class Dem:
    data: object  # torch tensor (H, W) float32
    nodata: float | None
    affine: tuple


def terrain_2048(device="cpu") -> Dem:
    torch = _torch()
    d = fbm_dem(2048, 2048, seed=0, lo=0.0, hi=3000.0, device=device)
    g = torch.Generator().manual_seed(100)
    idx = torch.randperm(d.numel(), generator=g)[: d.numel() // 100].to(device)
    d.view(-1)[idx] = -9999.0
    return Dem(d, -9999.0, (30.0, 0.0, 500000.0, 0.0, -30.0, 4500000.0))


def disc_holes(d, n_discs: int, seed: int, rmin: float, rmax: float, value: float) -> None:
    """Set ``value`` inside ``n_discs`` seeded discs (in place)."""
    torch = _torch()
    H, W = d.shape
    rng = np.random.default_rng(seed)
    cy = rng.uniform(0, H, n_discs)
    cx = rng.uniform(0, W, n_discs)
    rr = rng.uniform(rmin, rmax, n_discs)
    for y, x, r in zip(cy, cx, rr):
        y0, y1 = max(0, int(y - r)), min(H, int(y + r) + 1)
        x0, x1 = max(0, int(x - r)), min(W, int(x + r) + 1)
        yy = torch.arange(y0, y1, device=d.device, dtype=torch.float32)[:, None]
        xx = torch.arange(x0, x1, device=d.device, dtype=torch.float32)[None, :]
        m = (yy - float(y)) ** 2 + (xx - float(x)) ** 2 <= float(r) ** 2
        d[y0:y1, x0:x1][m] = value


def terrain_16k(device="cpu", size: int = 16384) -> Dem:
    d = fbm_dem(size, size, seed=1, lo=0.0, hi=4500.0, device=device)
    disc_holes(d, 200, seed=101, rmin=5.0, rmax=80.0, value=-9999.0)
    return Dem(d, -9999.0, (10.0, 0.0, 600000.0, 0.0, -10.0, 5000000.0))


def trend_noise(height: int = 8192, width: int = 8192, device="cpu"):
    torch = _torch()
    g = torch.Generator().manual_seed(2)
    noise = torch.rand((height, width), generator=g, dtype=torch.float32).to(device)
    ramp = torch.arange(height * width, device=device, dtype=torch.float64).reshape(height, width)
    return (noise.double() + ramp * (100.0 / (height * width))).float()


def random_weights(k: int, seed: int) -> np.ndarray:
    """Seeded non-negative k x k weights normalised to sum 1 (float64)."""
    w = np.random.default_rng(seed).random((k, k))
    return w / w.sum()


@dataclass
class Tile:
    data: object
    nodata: float
    cell: float

    @property
    def affine(self):
        return (self.cell, 0.0, 0.0, 0.0, -self.cell, 0.0)


def tile_batch(n: int = 512, lo: int = 256, hi: int = 4096, seed: int = 3, device="cpu") -> list[Tile]:
    torch = _torch()
    rng = np.random.default_rng(seed)
    tiles = []
    for i in range(n):
        h = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        w = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        cell = float(rng.uniform(1.0, 90.0))
        nodata = -9999.0 if rng.random() < 0.5 else float("nan")
        frac = float(rng.uniform(0.0, 0.05))
        d = fbm_dem(h, w, seed=1000 + i, lo=0.0, hi=3000.0, octaves=6, device=device)
        k = int(frac * h * w)
        if k:
            g = torch.Generator().manual_seed(5000 + i)
            idx = torch.randperm(h * w, generator=g)[:k].to(device)
            d.view(-1)[idx] = nodata
        tiles.append(Tile(d, nodata, cell))
    return tiles


def gamma_stack(bands: int = 12, size: int = 10980, seed: int = 4, device="cpu"):
    torch = _torch()
    g = torch.Generator(device=device).manual_seed(seed) if str(device).startswith("cuda") else torch.Generator().manual_seed(seed)
    out = torch.empty((bands, size, size), dtype=torch.uint16, device=device)
    conc = torch.tensor(2.0, device=device)
    rate = torch.tensor(1.0 / 800.0, device=device)
    dist = torch.distributions.Gamma(conc, rate)
    for b in range(bands):
        torch.manual_seed(seed * 1000 + b)
        v = dist.sample((size, size)).clamp_(0, 10000)
        zero = torch.rand((size, size), generator=g, device=device) < 0.03
        v[zero] = 0
        out[b] = v.to(torch.int32).to(torch.uint16)
        del v, zero
    return out
