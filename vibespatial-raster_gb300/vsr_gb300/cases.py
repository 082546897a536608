"""Single-operation timing cases on synthetic device rasters.

``python -m vsr_gb300.cases <op> [options]`` builds one seeded synthetic
input on ``cuda:0`` (the shapes and value distributions of the benchmark
workloads), runs the operation through the public API a few times to warm
up, then times ``--reps`` calls with CUDA events and prints one JSON line.
It is the small, single-kernel command to run under a profiler:

    conv        trend-plus-noise float32 raster, seeded normalised k x k weights
                (the 8192^2 convolution workload at a chosen size)
    focal_mean  uint16 band stack, gamma-like values 0..9999, 3 % nodata 0
                (the 12 x 10980^2 multiband workload, fewer bands)
    focal_stat  the same stack, one focal statistic (--stat), float32 output
    gaussian    the same uint16 stack, Gaussian sigma / kernel size
                (--precision split_bf16: the tensor-core line passes;
                fp32: the separable CUDA-core kernels)
    horn        fused slope + aspect + hillshade on the fBm DEM with 200
                -9999 disc holes (the 16384^2 terrain workload at a chosen
                size), one launch configuration of the Horn kernel
                (--config, an index into the tuning table)
    batch       the first --tiles tiles of the uneven DEM tile batch
                (slope + aspect + 5 x 5 Gaussian per tile, or --part) in one
                persistent launch, one launch configuration (--config)

Run with ``PYTHONPATH=vibespatial-raster_gb300`` from the repository root.
"""

from __future__ import annotations

import argparse
import json

import numpy as np


def _timed(fn, reps: int) -> float:
    import torch

    for _ in range(3):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    b.synchronize()
    return a.elapsed_time(b) / reps


def _uint16_stack(bands: int, size: int):
    import torch

    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev).manual_seed(4)
    x = torch.randint(1, 10000, (bands, size, size), generator=g, device=dev, dtype=torch.int32)
    hole = torch.rand((bands, size, size), generator=g, device=dev) < 0.03
    x[hole] = 0
    return x.to(torch.uint16)


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("op", choices=["conv", "focal_mean", "focal_stat", "gaussian", "horn", "batch"])
    ap.add_argument("--stat", default="std", choices=["min", "max", "std", "range", "variety"],
                    help="focal_stat: the statistic")
    ap.add_argument("--size", type=int, default=None, help="raster side (default: 4096 conv, 10980 others)")
    ap.add_argument("--bands", type=int, default=1)
    ap.add_argument("--k", type=int, default=31, help="kernel side (conv, gaussian)")
    ap.add_argument("--sigma", type=float, default=8.0)
    ap.add_argument("--radius", type=int, default=3)
    ap.add_argument("--precision", default="split_bf16", choices=["auto", "fp32", "split", "split_bf16"])
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--config", type=int, default=0, help="launch configuration (horn, batch)")
    ap.add_argument("--tiles", type=int, default=512, help="tiles of the batch (batch)")
    ap.add_argument("--part", default="all", choices=["all", "horn", "gauss"],
                    help="batch: slope + aspect + Gaussian, or one of the two alone")
    ap.add_argument("--no-nodata", action="store_true", help="batch: tiles without a nodata value")
    args = ap.parse_args(argv)

    import torch

    import vsr_gb300 as vsr
    from vsr_gb300 import algebra, workloads

    vsr.load_library()
    dev = torch.device("cuda", 0)
    if args.op == "conv":
        n = args.size or 4096
        r = vsr.from_device(workloads.trend_noise(n, n, device=dev))
        w = workloads.random_weights(args.k, 200 + args.k)
        out = torch.empty((1, n, n), dtype=torch.float32, device=dev)
        ms = _timed(lambda: algebra.convolve_bands(r, w, precision=args.precision, out_dtype=np.float32, out=out),
                    args.reps)
        px = n * n
    elif args.op == "horn":
        from vsr_gb300 import _lib

        n = args.size or 8192
        dem = workloads.terrain_16k(device=dev, size=n)
        r = vsr.from_device(dem.data, nodata=dem.nodata, affine=dem.affine)
        lib = _lib.load()
        _lib.check(lib.vsr_tuning_set(_lib.VSR_OP_HORN, args.config), "vsr_tuning_set")
        outs = (torch.empty((1, n, n), dtype=torch.float32, device=dev),
                torch.empty((1, n, n), dtype=torch.float32, device=dev),
                torch.empty((1, n, n), dtype=torch.uint8, device=dev))
        ms = _timed(lambda: algebra.horn_fused(r, out=outs), args.reps)
        px = n * n
    elif args.op == "batch":
        from vsr_gb300 import _lib, batch

        lib = _lib.load()
        _lib.check(lib.vsr_tuning_set(_lib.VSR_OP_BATCH, args.config), "vsr_tuning_set")
        tiles = workloads.tile_batch(device=dev)[: args.tiles]
        rs = [vsr.from_device(t.data, nodata=None if args.no_nodata else t.nodata, affine=t.affine) for t in tiles]
        b = batch.TerrainBatch(rs, terrain=args.part != "gauss", sigma=None if args.part == "horn" else 1.0,
                               kernel_size=5)
        ms = _timed(b.run, args.reps)
        n = 0
        px = sum(int(t.data.numel()) for t in tiles)
    else:
        n = args.size or 10980
        r = vsr.from_device(_uint16_stack(args.bands, n), nodata=0)
        out = torch.empty((args.bands, n, n), dtype=torch.float32, device=dev)
        if args.op == "focal_mean":
            fn = lambda: algebra.focal_mean_bands(r, args.radius, args.radius, out_dtype=np.float32, out=out)  # noqa: E731
        elif args.op == "focal_stat":
            fn = lambda: algebra.focal_stat_bands(r, args.stat, args.radius, args.radius,  # noqa: E731
                                                  out_dtype=np.float32, out=out)
        else:
            fn = lambda: algebra.gaussian_bands(r, args.sigma, args.k, precision=args.precision,  # noqa: E731
                                                out_dtype=np.float32, out=out)
        ms = _timed(fn, args.reps)
        px = args.bands * n * n
    print(json.dumps({"op": args.op, "size": n, "bands": args.bands, "ms": ms, "gpix_s": px / ms / 1e6,
                      "options": {k: v for k, v in vars(args).items() if k not in ("op", "size", "bands")}}))


if __name__ == "__main__":
    main()
