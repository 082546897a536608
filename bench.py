"""Benchmark of the focal-stencil hot path on GB300.

Default workload: fused slope + aspect + hillshade (azimuth 315, altitude 45)
over one 16384 x 16384 float32 fBm DEM (0-4500 m, 10 m cells, -9999 in 200
disc holes).  A step is one fused pass over the whole DEM.  Inputs (1 GiB)
and outputs (2.25 GiB) are far larger than the 129 MB L2, so no flush is
needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl vsr|reference]

Prints ONE JSON line (rank 0).  ``value`` is device throughput (Gpixel/s) with
the DEM resident in HBM; ``e2e`` is the same metric through the public API
(from_numpy of a pinned host DEM -> raster_terrain_host into pinned host
buffers: row strips streamed through the GPU with the copies overlapped),
copies included.  ``--impl reference`` times the reference's
CPU algorithm (the float64 numpy restatement in oracle/, the reference being
pure Python) on the host cores.  Under torchrun each rank runs its own
replica (the path shards by raster; no collective on the data path).
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for _p in (str(ROOT), str(ROOT / "vibespatial-raster_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "Gpixel/s & % roofline: slope/aspect, conv; batched/split-BF16 vs plain FP32"
UNIT = "Gpixel/s"
BYTES_PER_PX = 13  # read f32 DEM 4 + slope 4 + aspect 4 + hillshade 1
WORKLOAD = "fused slope+aspect+hillshade, 16384x16384 f32 fBm DEM, 10 m cells, 200 -9999 disc holes"


def _dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi SM clock / throttle sampler running during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def _roofline_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ----------------------------------------------------------------- CPU legs --
def _oracle_terrain_strip(dem: np.ndarray, y0: int, y1: int, affine, nodata):
    """Reference CPU path (slope, aspect, hillshade: three calls) on rows [y0, y1)."""
    import oracle

    lo, hi = max(0, y0 - 1), min(dem.shape[0], y1 + 1)
    strip = dem[lo:hi]
    s, _ = oracle.slope_aspect(strip, affine, nodata, compute_slope=True, compute_aspect=False)
    _, a = oracle.slope_aspect(strip, affine, nodata, compute_slope=False, compute_aspect=True)
    h, _ = oracle.hillshade(strip, affine, nodata)
    return s.astype(np.float32), a.astype(np.float32), h


def cpu_sample(dem_host: np.ndarray, affine, nodata, rows: int, threads: int):
    """Time the oracle over ``rows`` rows split into strips over ``threads`` threads."""
    H = dem_host.shape[0]
    y0 = (H - rows) // 2
    strips = max(1, threads)
    step = (rows + strips - 1) // strips
    spans = [(y0 + i * step, min(y0 + rows, y0 + (i + 1) * step)) for i in range(strips)]
    t0 = time.perf_counter()
    if threads <= 1:
        for a, b in spans:
            _oracle_terrain_strip(dem_host, a, b, affine, nodata)
    else:
        with ThreadPoolExecutor(max_workers=threads) as ex:
            list(ex.map(lambda s: _oracle_terrain_strip(dem_host, s[0], s[1], affine, nodata), spans))
    dt = time.perf_counter() - t0
    return rows * dem_host.shape[1], dt


def run_reference(args, ws, rank):
    """--impl reference: the reference CPU algorithm on all host cores."""
    if rank != 0:
        return
    import torch

    from vsr_gb300 import workloads

    dem = workloads.terrain_16k(device="cuda" if torch.cuda.is_available() else "cpu")
    host = dem.data.cpu().numpy()
    cores = len(os.sched_getaffinity(0))
    rows = 1024
    for _ in range(args.warmup):
        cpu_sample(host, dem.affine, dem.nodata, rows, cores)
    times = []
    px = 0
    for _ in range(args.steps):
        n, dt = cpu_sample(host, dem.affine, dem.nodata, rows, cores)
        times.append(dt)
        px += n
    total = sum(times)
    value = px / total / 1e9
    sample = f"{rows} rows x 16384 of the DEM per step, split into {cores} row strips (1-row halo) over {cores} threads"
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "cpu_path": "reference float64 numpy algorithm (oracle port: slope, aspect, hillshade as 3 calls)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- GPU leg --
def run_vsr(args, ws, rank, local):
    import torch

    import vsr_gb300 as vsr
    from vsr_gb300 import algebra, workloads

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    vsr.load_library()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    dem = workloads.terrain_16k(device=dev, size=args.dem_size)
    H, W = dem.data.shape
    px = H * W
    r = vsr.from_device(dem.data, nodata=dem.nodata, affine=dem.affine)
    outs = (torch.empty((1, H, W), dtype=torch.float32, device=dev),
            torch.empty((1, H, W), dtype=torch.float32, device=dev),
            torch.empty((1, H, W), dtype=torch.uint8, device=dev))

    def step():
        algebra.horn_fused(r, out=outs)

    from vsr_gb300 import autotune

    tuned = autotune.autotune_horn(r, outputs=outs)
    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # per-launch duration of the dominant kernel (one launch per step): an
    # event pair around every launch of the timed region, read after it ends
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    e0.record(stream)
    for i in range(args.steps):
        ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
    e1.record(stream)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    ms = e0.elapsed_time(e1)
    launch_ms = [a.elapsed_time(b) for a, b in ev]

    # ---- end-to-end through the public API with host buffers ----
    host_in = torch.empty((H, W), dtype=torch.float32, pin_memory=True)
    host_in.copy_(dem.data)
    host_out = [torch.empty((H, W), dtype=torch.float32, pin_memory=True),
                torch.empty((H, W), dtype=torch.float32, pin_memory=True),
                torch.empty((H, W), dtype=torch.uint8, pin_memory=True)]
    in_np = host_in.numpy()
    out_np = [t.numpy() for t in host_out]

    from vsr_gb300 import stream as vstream

    def e2e_step():
        # public API, host in -> host out: row strips streamed through the GPU
        # with host->device, kernel and device->host overlapped on 3 streams
        rr = vsr.from_numpy(in_np, nodata=dem.nodata, affine=dem.affine)
        vstream.raster_terrain_host(rr, out=out_np)

    e2e_step()
    torch.cuda.synchronize()
    e2e_steps = max(3, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    clocks = sampler.stop()

    # max over ranks
    from vsr_gb300 import replicas

    t_step, e2e_s = replicas.max_over_ranks([ms / args.steps, e2e_s], device=dev)
    value = ws * px / (t_step * 1e-3) / 1e9
    e2e_value = ws * px / e2e_s / 1e9

    if rank == 0:
        peak, peak_kind = _roofline_peak()
        lmed = statistics.mean(launch_ms)
        achieved = BYTES_PER_PX * px / (lmed * 1e-3) / 1e9
        # dram read + write bytes per launch from the ncu capture summarised in
        # profiles/ (8192^2 capture scaled to 16384^2 by pixel count)
        traffic = None
        summary = ROOT / "profiles" / "horn_f32_tma_terrain8k_ncu.md"
        if summary.exists() and H == 16384:
            for line in summary.read_text().splitlines():
                if line.strip().startswith("traffic_bytes_per_launch_16384"):
                    traffic = int(line.split("=")[1])
        # CPU baseline: the oracle, single thread, on a bounded row sample.
        host = in_np
        cpu_rows = 512
        n, dt = cpu_sample(host, dem.affine, dem.nodata, cpu_rows, 1)
        n2, dt2 = cpu_sample(host, dem.affine, dem.nodata, cpu_rows, 1)
        cpu_val = (n + n2) / (dt + dt2) / 1e9
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD if H == 16384 else WORKLOAD.replace("16384x16384", f"{H}x{W}"), "pixels": px, "bytes_per_pixel": BYTES_PER_PX,
                       "l2": "inputs+outputs (3.5 GB/step) exceed L2; no flush",
                       "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
                       "autotuned": {"rows_per_tile": tuned["shape"][0], "tma_stages": tuned["shape"][1],
                                     "threads_per_cta": tuned["shape"][2], "tma_store_tiles": tuned["shape"][3],
                                     "ms_by_config": {str(k): round(v, 4) for k, v in tuned["ms"].items()}}},
            "gpu_launches": args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                         "kernel": "horn_f32_tma", "launch_ms": lmed},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": px * 4,
                    "d2h_bytes_per_step": px * 9, "ms_per_step": e2e_s * 1e3},
            "cpu_baseline": {"value": cpu_val, "unit": UNIT, "cores": 1, "kind": "port",
                             "sample": f"2 x {cpu_rows} rows x {W} px (1-row halo) of the same DEM, reference "
                                       "float64 numpy algorithm, 3 calls (slope, aspect, hillshade), 1 thread"},
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


# ------------------------------------------------------- secondary workloads --
def _time_ms(fn, steps, stream):
    import torch

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    return 6800.0, 1900.0, "fallback"


def run_conv(args, ws, rank, local):
    """8192^2 trend+noise raster: normalised convolution, plain FP32 vs split-BF16."""
    import torch

    import vsr_gb300 as vsr
    from vsr_gb300 import algebra, autotune, workloads  # noqa: F401

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    vsr.load_library()
    H = W = 8192
    x = workloads.trend_noise(H, W, device=dev)
    r = vsr.from_device(x)
    stream = torch.cuda.current_stream()
    kernels = {"k15": workloads.random_weights(15, 215), "k31": workloads.random_weights(31, 231),
               "gauss41": None}
    import oracle  # CPU baseline only

    kernels["gauss41"] = oracle.gaussian_weights(5.0, 41)
    out = torch.empty((1, H, W), dtype=torch.float32, device=dev)
    hbm, bf16, src = _peaks()
    res = {}
    for name, w in kernels.items():
        k = w.shape[0]
        t = {}
        for prec in ("fp32", "split_bf16"):
            fn = lambda: algebra.convolve_bands(r, w, precision=prec, out_dtype=np.float32, out=out)  # noqa: E731
            for _ in range(max(3, args.warmup)):
                fn()
            t[prec] = _time_ms(fn, args.steps, stream)
        kp = ((64 + k - 1) + 15) // 16 * 16
        # 3 split products per kernel row; a 128 x 64 output tile multiplies
        # K = kp (window width rounded to 16): 2 * kp flops per output per row
        issued = 3 * 2 * H * W * k * kp
        res[name] = {"k": k, "fp32_ms": t["fp32"], "split_bf16_ms": t["split_bf16"],
                     "speedup": t["fp32"] / t["split_bf16"],
                     "fp32_gpix_s": H * W / t["fp32"] / 1e6, "split_bf16_gpix_s": H * W / t["split_bf16"] / 1e6,
                     "useful_tflops_split": 2 * k * k * H * W / t["split_bf16"] / 1e9,
                     "issued_tensor_tflops": issued / t["split_bf16"] / 1e9}
    # CPU baseline: float64 scipy restatement on a 1024^2 crop, one thread
    crop = x[:1024, :1024].cpu().numpy()
    t0 = time.perf_counter()
    oracle.convolve_normalized(crop, kernels["k31"], None)
    cpu_s = time.perf_counter() - t0
    main = res["k31"]
    line = {
        "metric": METRIC, "value": main["split_bf16_gpix_s"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": main["split_bf16_ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16x3 (split) / f32 accumulate", "data": "synthetic",
        "config": {"workload": "normalised focal convolution, 8192x8192 f32 U[0,1)+0-100 trend, no nodata, "
                               "f32 output; headline kernel 31x31 split-BF16", "kernels": res,
                   "l2": "256 MiB in + 256 MiB out per step exceed L2; no flush"},
        "gpu_launches": args.steps * 2,
        "roofline": {"bound": "tensor", "achieved": main["issued_tensor_tflops"], "peak": bf16, "unit": "TFLOP/s",
                     "frac": main["issued_tensor_tflops"] / bf16, "traffic": None, "peak_source": src,
                     "kernel": "conv_tc_kernel"},
        "cpu_baseline": {"value": 1024 * 1024 / cpu_s / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": "1024x1024 crop, 31x31 kernel, float64 scipy correlate restatement, 1 thread"},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_batch(args, ws, rank, local):
    """512 uneven DEM tiles: slope+aspect + 5x5 Gaussian, one persistent graph launch vs per-tile."""
    import torch

    import vsr_gb300 as vsr
    from vsr_gb300 import batch, workloads

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    vsr.load_library()
    tiles = workloads.tile_batch(device=dev)
    rasters = [vsr.from_device(t.data, nodata=t.nodata, affine=t.affine) for t in tiles]
    px = sum(int(t.data.numel()) for t in tiles)
    stream = torch.cuda.current_stream()
    b = batch.TerrainBatch(rasters, sigma=1.0, kernel_size=5)
    tuned = batch.autotune_batch(b)
    b.capture()
    for _ in range(max(3, args.warmup)):
        b.replay()
    t_batch = _time_ms(b.replay, args.steps, stream)
    outs = [(s.unsqueeze(0), a.unsqueeze(0), g.unsqueeze(0)) for (s, a, g) in b.outputs]
    per = lambda: batch.per_tile_launches(rasters, outs=outs)  # noqa: E731
    for _ in range(max(3, args.warmup)):
        per()
    t_per = _time_ms(per, max(3, args.steps // 5), stream)
    hbm, bf16, src = _peaks()
    achieved = 16 * px / (t_batch * 1e-3) / 1e9
    import oracle

    sample = tiles[:8]
    t0 = time.perf_counter()
    spx = 0
    for t in sample:
        z = t.data.cpu().numpy()
        oracle.slope_aspect(z, t.affine, t.nodata, compute_slope=True, compute_aspect=False)
        oracle.slope_aspect(z, t.affine, t.nodata, compute_slope=False, compute_aspect=True)
        oracle.convolve_normalized(z, oracle.gaussian_weights(1.0, 5), t.nodata)
        spx += z.size
    cpu_s = time.perf_counter() - t0
    line = {
        "metric": METRIC, "value": px / (t_batch * 1e-3) / 1e9, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_batch, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "512 f32 fBm tiles, sides log-uniform [256,4096], cell U[1,90] m, nodata -9999/NaN "
                               "on 0-5%; slope+aspect + 5x5 Gaussian (sigma 1)",
                   "pixels": px, "bytes_per_pixel": 16, "batched_ms": t_batch, "per_tile_ms": t_per,
                   "speedup_vs_per_tile": t_per / t_batch, "per_tile_launches": 2 * len(tiles),
                   "autotuned": {"config": batch.BATCH_CONFIGS[tuned["config"]],
                                 "ms_by_config": {str(k): round(v, 4) for k, v in tuned["ms"].items()}},
                   "l2": "3.9 GB in + 11.8 GB out per step exceed L2; no flush"},
        "gpu_launches": args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": None, "peak_source": src, "kernel": "batch_terrain_kernel"},
        "cpu_baseline": {"value": spx / cpu_s / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": "first 8 tiles: reference slope, aspect (2 calls) + float64 5x5 Gaussian, 1 thread"},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_multiband(args, ws, rank, local):
    """12 x 10980^2 uint16 stack: 7x7 focal mean + Gaussian sigma 8 (65x65) per band."""
    import torch

    import vsr_gb300 as vsr
    from vsr_gb300 import algebra, workloads

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    vsr.load_library()
    stack = workloads.gamma_stack(device=dev)
    B, H, W = stack.shape
    r = vsr.from_device(stack, nodata=0)
    stream = torch.cuda.current_stream()
    mean = torch.empty((B, H, W), dtype=torch.float32, device=dev)
    gauss = torch.empty((B, H, W), dtype=torch.float32, device=dev)

    # the Gaussian on "auto": the split-precision tensor-core line passes for
    # this uint16 stack (65 x 65 >= 35)
    def step():
        algebra.focal_mean_bands(r, 3, 3, out_dtype=np.float32, out=mean)
        algebra.gaussian_bands(r, 8.0, 65, precision="auto", out_dtype=np.float32, out=gauss)

    for _ in range(max(3, args.warmup)):
        step()
    t = _time_ms(step, max(1, args.steps // 10), stream)
    t_mean = _time_ms(lambda: algebra.focal_mean_bands(r, 3, 3, out_dtype=np.float32, out=mean), 3, stream)
    t_tc = _time_ms(lambda: algebra.gaussian_bands(r, 8.0, 65, precision="split_bf16", out_dtype=np.float32,
                                                    out=gauss), 3, stream)
    t_fp32 = _time_ms(lambda: algebra.gaussian_bands(r, 8.0, 65, precision="fp32", out_dtype=np.float32,
                                                      out=gauss), 3, stream)
    hbm, bf16, src = _peaks()
    px = B * H * W
    # CPU baseline: the oracle (vectorised float64 restatements of the reference
    # CPU focal mean and of the reference GPU convolution) on crops of band 0
    import oracle  # CPU baseline only

    crop = stack[0, :1024, :1024].cpu().numpy()
    t0 = time.perf_counter()
    oracle.focal_mean(crop, 3, 3, 0)
    cpu_mean_s = (time.perf_counter() - t0) / (1024 * 1024)
    crop = stack[0, :256, :256].cpu().numpy()
    t0 = time.perf_counter()
    ref = oracle.convolve_normalized(crop, oracle.gaussian_weights(8.0, 65), 0)
    cpu_gauss_s = (time.perf_counter() - t0) / (256 * 256)
    # the tensor-core Gaussian's error against the float64 oracle on that crop
    # (relative to max(|ref|, mean |value|), nodata outputs excluded)
    rc = vsr.from_device(stack[0, :256, :256].contiguous(), nodata=0)
    tc_out = algebra.gaussian_bands(rc, 8.0, 65, precision="split_bf16").cpu().numpy()[0]
    m = ref != 0
    tc_err = float(np.max(np.abs(tc_out[m] - ref[m]) / np.maximum(np.abs(ref[m]), float(np.mean(crop)))))
    line = {
        "metric": METRIC, "value": px / (t * 1e-3) / 1e9, "unit": UNIT, "n_gpus": ws, "steps": max(1, args.steps // 10),
        "warmup": args.warmup, "ms_per_step": t, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u16 in, f32 compute/out", "data": "synthetic",
        "config": {"workload": "12 x 10980x10980 uint16 gamma(2,800) clipped 0-10000, 3% nodata 0; focal mean 7x7 "
                               "+ Gaussian sigma 8 (65x65) per band", "focal_mean_ms": t_mean,
                   "focal_mean_gpix_s": px / (t_mean * 1e-3) / 1e9,
                   "focal_mean_hbm_frac": 6 * px / (t_mean * 1e-3) / 1e9 / hbm,
                   "gaussian_path": "auto = split-precision tensor-core line passes (F16 hi/lo, FP32 accumulate)",
                   "gaussian_tensor_core_ms": t_tc, "gaussian_fp32_ms": t_fp32,
                   "gaussian_tensor_core_vs_fp32": t_fp32 / t_tc,
                   "gaussian_tensor_core_max_rel_err_vs_fp64": tc_err},
        # per step: the focal mean (all bands), the band image, two line passes per band
        "gpu_launches": (2 + 2 * B) * max(1, args.steps // 10),
        "roofline": {"bound": "hbm", "achieved": 10 * px / (t * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
                     "frac": 10 * px / (t * 1e-3) / 1e9 / hbm, "traffic": None, "peak_source": src,
                     "kernel": "box_slide_int + gauss_line_kernel"},
        "cpu_baseline": {"value": 1.0 / (cpu_mean_s + cpu_gauss_s) / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": "band 0: 7x7 focal mean on a 1024^2 crop + 65x65 Gaussian (dense float64 "
                                   "correlate, as the reference's dense kernel) on a 256^2 crop, per-pixel times "
                                   "summed, 1 thread"},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_slope2048(args, ws, rank, local):
    """2048^2 fBm DEM (1 % nodata): GPU slope vs the reference's CPU fallback on the whole raster."""
    import torch

    import vsr_gb300 as vsr
    from vsr_gb300 import algebra, workloads

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    vsr.load_library()
    dem = workloads.terrain_2048(device=dev)
    H, W = dem.data.shape
    r = vsr.from_device(dem.data, nodata=dem.nodata, affine=dem.affine)
    out = torch.empty((1, H, W), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()
    fn = lambda: algebra.horn_fused(r, slope=True, aspect=False, hillshade=False, out=(out, None, None))  # noqa: E731
    for _ in range(max(3, args.warmup)):
        fn()
    ms = _time_ms(fn, args.steps, stream)
    hbm, _, src = _peaks()
    import oracle  # CPU baseline only: the reference CPU fallback's algorithm

    host = dem.data.cpu().numpy()
    t0 = time.perf_counter()
    oracle.slope_aspect(host, dem.affine, dem.nodata)
    cpu_s = time.perf_counter() - t0
    px = H * W
    line = {
        "metric": METRIC, "value": px / (ms * 1e-3) / 1e9, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "Horn slope (degrees), 2048x2048 f32 fBm DEM 0-3000 m, 30 m cells, 1 % nodata -9999",
                   "l2": "16 MiB in + 16 MiB out fit in L2: back-to-back launches, no flush (small-raster case)"},
        "gpu_launches": args.steps,
        "roofline": {"bound": "hbm", "achieved": 8 * px / (ms * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
                     "frac": 8 * px / (ms * 1e-3) / 1e9 / hbm, "traffic": None, "peak_source": src,
                     "kernel": "horn_f32_tma (slope only)"},
        "cpu_baseline": {"value": px / cpu_s / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": "the whole 2048^2 DEM, reference float64 slope/aspect algorithm, 1 thread"},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_derivatives(args, ws, rank, local):
    """TRI + TPI + profile curvature in one pass over the 16384^2 fBm DEM (float64 out, the reference dtype)."""
    import torch

    import vsr_gb300 as vsr
    from vsr_gb300 import algebra, workloads

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    vsr.load_library()
    dem = workloads.terrain_16k(device=dev, size=args.dem_size)
    H, W = dem.data.shape
    r = vsr.from_device(dem.data, nodata=dem.nodata, affine=dem.affine)
    outs = tuple(torch.empty((1, H, W), dtype=torch.float64, device=dev) for _ in range(3))
    outs32 = tuple(torch.empty((1, H, W), dtype=torch.float32, device=dev) for _ in range(3))
    stream = torch.cuda.current_stream()
    fn = lambda: algebra.terrain_derivatives(r, out=outs)  # noqa: E731
    for _ in range(max(3, args.warmup)):
        fn()
    steps = max(5, args.steps // 5)
    ms = _time_ms(fn, steps, stream)
    fn32 = lambda: algebra.terrain_derivatives(r, out_dtype=np.float32, out=outs32)  # noqa: E731
    fn32()
    ms32 = _time_ms(fn32, steps, stream)
    hbm, _, src = _peaks()
    import oracle  # CPU baseline only: the reference CPU algorithm, three calls

    strip = dem.data[:512].cpu().numpy()
    t0 = time.perf_counter()
    for k in (oracle.TRI, oracle.TPI, oracle.CURVATURE):
        oracle.terrain_derivative(strip, dem.affine, dem.nodata, k)
    cpu_s = (time.perf_counter() - t0) / strip.size
    px = H * W
    line = {
        "metric": METRIC, "value": px / (ms * 1e-3) / 1e9, "unit": UNIT, "n_gpus": ws, "steps": steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 double-float (f64 out)", "data": "synthetic",
        "config": {"workload": f"TRI + TPI + profile curvature, {H}x{W} f32 fBm DEM 0-4500 m, 10 m cells, "
                               "200 -9999 disc holes; one pass, float64 outputs",
                   "bytes_per_pixel": 28, "f32_outputs_ms": ms32,
                   "l2": "1 GiB in + 6 GiB out per step exceed L2; no flush"},
        "gpu_launches": steps,
        "roofline": {"bound": "hbm", "achieved": 28 * px / (ms * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
                     "frac": 28 * px / (ms * 1e-3) / 1e9 / hbm, "traffic": None, "peak_source": src,
                     "kernel": "terrain_deriv_kernel<float>"},
        "cpu_baseline": {"value": 1.0 / cpu_s / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": "512 x 16384 rows of the same DEM, reference float64 TRI, TPI, curvature "
                                   "(3 calls), 1 thread"},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["vsr", "reference"], default="vsr")
    ap.add_argument("--workload", choices=["terrain", "slope2048", "conv", "batch", "multiband", "derivatives"],
                    default="terrain",
                    help="terrain (default, the headline): fused slope+aspect+hillshade on 16384^2; "
                         "conv: 8192^2 focal convolution, plain FP32 vs split-BF16; batch: 512 uneven tiles, "
                         "one graph-captured persistent launch vs per-tile launches; multiband: 12 x 10980^2 "
                         "uint16 focal mean 7x7 + Gaussian 65x65; slope2048: slope on a 2048^2 DEM vs the "
                         "reference CPU fallback; derivatives: TRI + TPI + curvature on the 16384^2 DEM")
    ap.add_argument("--dem-size", type=int, default=16384,
                    help="DEM side (the benchmark workload is 16384; smaller sizes are for profiling)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local = _dist_env()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    elif args.workload == "conv":
        run_conv(args, ws, rank, local)
    elif args.workload == "batch":
        run_batch(args, ws, rank, local)
    elif args.workload == "multiband":
        run_multiband(args, ws, rank, local)
    elif args.workload == "slope2048":
        run_slope2048(args, ws, rank, local)
    elif args.workload == "derivatives":
        run_derivatives(args, ws, rank, local)
    else:
        run_vsr(args, ws, rank, local)


if __name__ == "__main__":
    main()
