"""Benchmark of the focal-stencil hot path on GB300.

Headline workload (C2): fused slope + aspect + hillshade (azimuth 315, altitude
45) over one 16384 x 16384 float32 fBm DEM (0-4500 m, 10 m cells, -9999 in 200
disc holes).  A step is one fused pass over the whole DEM.  Inputs (1 GiB) and
outputs (2.25 GiB) are far larger than the 129 MB L2, so no flush is needed
between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl vsr|reference]
                    [--workload terrain|slope2048|conv|batch|multiband|derivatives]
                    [--no-secondary]

Prints ONE JSON line (rank 0).  ``value`` is device throughput (Gpixel/s) with
the DEM resident in HBM; ``e2e`` is the same metric through the public API
(from_numpy of a pinned host DEM -> raster_terrain_host into pinned host
buffers: row strips streamed through the GPU with the copies overlapped),
copies included, next to the host link's measured copy rates.  On one GPU the
default run also measures the other benchmark configurations and reports each
under ``config.secondary`` with its own CUDA-event time, roofline, CPU
baseline, error against the float64 oracle and clock sample:

    C1 slope2048  Horn slope on a 2048^2 fBm DEM (1 % nodata)
    C3 conv       8192^2 normalised convolution 15^2 / 31^2 / Gaussian 41^2,
                  plain FP32 vs split-BF16 tensor cores, float64 output
    C4 batch      512 uneven DEM tiles: slope + aspect + 5x5 Gaussian in one
                  graph-replayed persistent launch vs graph-captured per-tile
                  launches
    C5 multiband  12 x 10980^2 uint16 bands: 7x7 focal mean + 65x65 Gaussian

``--workload X`` measures one of them alone (profiling).  ``--impl reference``
times the reference's CPU algorithm (the float64 numpy restatement in oracle/,
the reference being pure Python) on the host cores.  Under torchrun each rank
runs its own replica (the path shards by raster; no collective on the data
path).
"""

from __future__ import annotations

import argparse
import json
import math
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
    """nvidia-smi SM clock / throttle sampler running during a timed region."""

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
        return self

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
        rows = []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]),
                             {n for n, v in zip(names, parts[5:9]) if v.lower() == "active"}))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        # samples under load: power in the upper half of the range seen (all
        # samples when the range is small)
        pw = [r[2] for r in rows]
        cut = (min(pw) + max(pw)) / 2 if max(pw) - min(pw) > 50.0 else -1.0
        load = [r for r in rows if r[2] >= cut]
        reasons = sorted(set().union(*(r[3] for r in load)))
        return {"sm_mhz": statistics.median(r[0] for r in load), "sm_max_mhz": rows[-1][1], "reasons": reasons,
                "samples": len(rows), "samples_under_load": len(load), "power_w_max": max(pw)}


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    return 6800.0, 1900.0, "fallback"


def _events():
    import torch

    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def timed_region(fn, steps: int, gpu: int, *, min_seconds: float = 1.0):
    """CUDA-event milliseconds per call of ``fn`` over one timed region of at
    least ``steps`` calls lasting about ``min_seconds`` or more, with the SM
    clocks sampled during it.  Returns (ms per call, calls, clocks)."""
    import torch

    stream = torch.cuda.current_stream()
    a, b = _events()
    torch.cuda.synchronize()
    a.record(stream)
    fn()
    b.record(stream)
    b.synchronize()
    est = max(a.elapsed_time(b), 1e-3)
    n = max(int(steps), int(math.ceil(min_seconds * 1e3 / est)))
    sampler = ClockSampler(gpu).start()
    time.sleep(0.3)
    torch.cuda.synchronize()
    a.record(stream)
    for _ in range(n):
        fn()
    b.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    return a.elapsed_time(b) / n, n, clocks


def _rel_err_stats(out, ref, scale):
    """max and p99 of |out - ref| / max(|ref|, scale) over finite reference values."""
    out = np.asarray(out, np.float64).ravel()
    ref = np.asarray(ref, np.float64).ravel()
    m = np.isfinite(ref)
    if not m.any():
        return {"max": 0.0, "p99": 0.0, "n": 0}
    e = np.abs(out[m] - ref[m]) / np.maximum(np.abs(ref[m]), scale)
    return {"max": float(e.max()), "p99": float(np.percentile(e, 99)), "n": int(m.sum())}


def _rel_err_samples(samples):
    """max and p99 of |out - ref| / max(|ref|, floor) over the finite reference
    values of (out, ref, floor) samples, each with its own floor (1e-3 of its
    input's mean magnitude: a guard for outputs near zero, which these
    workloads do not produce, so the figure is the plain relative error)."""
    es = []
    for out, ref, floor in samples:
        out = np.asarray(out, np.float64).ravel()
        ref = np.asarray(ref, np.float64).ravel()
        m = np.isfinite(ref)
        es.append(np.abs(out[m] - ref[m]) / np.maximum(np.abs(ref[m]), floor))
    e = np.concatenate(es) if es else np.zeros(0)
    if e.size == 0:
        return {"max": 0.0, "p99": 0.0, "n": 0}
    return {"max": float(e.max()), "p99": float(np.percentile(e, 99)), "n": int(e.size)}


def _abs_err_stats(out, ref, *, circular=False):
    out = np.asarray(out, np.float64).ravel()
    ref = np.asarray(ref, np.float64).ravel()
    m = np.isfinite(ref)
    if not m.any():
        return {"max": 0.0, "p99": 0.0, "n": 0}
    d = np.abs(out[m] - ref[m])
    if circular:
        d = np.minimum(d, 360.0 - d)
    return {"max": float(d.max()), "p99": float(np.percentile(d, 99)), "n": int(m.sum())}


def _strip_starts(H: int, rows: int, n: int, seed: int):
    """n row offsets of ``rows``-row strips: the first and last rows and seeded ones between."""
    rng = np.random.default_rng(seed)
    starts = {0, H - rows}
    while len(starts) < n:
        starts.add(int(rng.integers(1, H - rows)))
    return sorted(starts)


# ----------------------------------------------------------------- CPU legs --
def _oracle_terrain_strip(dem: np.ndarray, y0: int, y1: int, affine, nodata):
    """Reference CPU path (slope, aspect, hillshade: three calls) on rows [y0, y1)."""
    import oracle

    lo, hi = max(0, y0 - 1), min(dem.shape[0], y1 + 1)
    strip = dem[lo:hi]
    s, _ = oracle.slope_aspect(strip, affine, nodata, compute_slope=True, compute_aspect=False)
    _, a = oracle.slope_aspect(strip, affine, nodata, compute_slope=False, compute_aspect=True)
    h, _ = oracle.hillshade(strip, affine, nodata)
    return s[y0 - lo:y1 - lo], a[y0 - lo:y1 - lo], h[y0 - lo:y1 - lo]


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


# --------------------------------------------------------- host link peak --
def host_link_peak(dev, nbytes: int = 1 << 30, reps: int = 3) -> dict:
    """Pinned host <-> device copy rates: one ``nbytes`` copy per direction
    (cudaMemcpyAsync through torch), CUDA events, best of ``reps``; and both
    directions at once on two streams."""
    import torch

    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    h2 = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    d2 = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    out = {}
    for name, fn in (("h2d", lambda: d.copy_(h, non_blocking=True)), ("d2h", lambda: h.copy_(d, non_blocking=True))):
        fn()
        best = None
        for _ in range(reps):
            a, b = _events()
            a.record()
            fn()
            b.record()
            b.synchronize()
            ms = a.elapsed_time(b)
            best = ms if best is None else min(best, ms)
        out[f"{name}_gbs"] = nbytes / (best * 1e-3) / 1e9
    s1, s2 = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    best = None
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with torch.cuda.stream(s1):
            d.copy_(h, non_blocking=True)
        with torch.cuda.stream(s2):
            h2.copy_(d2, non_blocking=True)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    out["duplex_gbs"] = 2 * nbytes / best / 1e9
    out["bytes_per_copy"] = nbytes
    del h, h2, d, d2
    return out


# ----------------------------------------------------------------- GPU leg --
def terrain_errors(dem_t, outs, affine, nodata, *, rows: int = 64, n: int = 4) -> dict:
    """C2 outputs against the float64 oracle on ``n`` row strips (the first, the
    last and seeded ones): slope and aspect in degrees (aspect on the circle),
    hillshade in DN; nodata outputs excluded."""
    H = dem_t.shape[0]
    es, ea, eh = [], [], []
    exact = total = 0
    for y0 in _strip_starts(H, rows, n, seed=7):
        lo, hi = max(0, y0 - 1), min(H, y0 + rows + 1)
        z = dem_t[lo:hi].cpu().numpy()
        rs, ra, rh = _oracle_terrain_strip(z, y0 - lo, y0 - lo + rows, affine, nodata)
        s = outs[0][0, y0:y0 + rows].cpu().numpy()
        a = outs[1][0, y0:y0 + rows].cpu().numpy()
        h = outs[2][0, y0:y0 + rows].cpu().numpy()
        m = rs != nodata
        es.append((s[m], rs[m]))
        m = ra != nodata
        ea.append((a[m], ra[m]))
        d = np.abs(h.astype(int) - rh.astype(int))
        eh.append(int(d.max()))
        exact += int((d == 0).sum())
        total += d.size
    cat = lambda L, i: np.concatenate([x[i] for x in L])  # noqa: E731
    return {"slope_deg": _abs_err_stats(cat(es, 0), cat(es, 1)),
            "aspect_deg": _abs_err_stats(cat(ea, 0), cat(ea, 1), circular=True),
            "hillshade_dn": {"max": max(eh), "exact_share": exact / total},
            "sample": f"{n} strips of {rows} rows x 16384 (first, last, seeded), nodata excluded"}


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
    sampler = ClockSampler(local).start()
    time.sleep(0.3)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = _events()
    # per-launch duration of the dominant kernel (one launch per step): an
    # event pair around every launch of the timed region, read after it ends
    ev = [_events() for _ in range(args.steps)]
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

    phases = []

    def e2e_step(record=None):
        # public API, host in -> host out: row strips streamed through the GPU
        # with host->device, kernel and device->host overlapped on 3 streams
        rr = vsr.from_numpy(in_np, nodata=dem.nodata, affine=dem.affine)
        vstream.raster_terrain_host(rr, out=out_np, phase_events=record)

    e2e_step()
    torch.cuda.synchronize()
    e2e_steps = max(3, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    clocks = sampler.stop()
    e2e_step(record=phases)  # one more step with per-strip phase events (not timed)
    phase_ms = vstream.phase_summary(phases)

    # max over ranks
    from vsr_gb300 import replicas

    t_step, e2e_s = replicas.max_over_ranks([ms / args.steps, e2e_s], device=dev)
    value = ws * px / (t_step * 1e-3) / 1e9
    e2e_value = ws * px / e2e_s / 1e9

    if rank == 0:
        hbm, bf16, peak_kind = _peaks()
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
        link = host_link_peak(dev)
        h2d_b, d2h_b = px * 4, px * 9
        link_ms = max(h2d_b / (link["h2d_gbs"] * 1e9), d2h_b / (link["d2h_gbs"] * 1e9)) * 1e3
        errors = terrain_errors(dem.data, outs, dem.affine, dem.nodata) if H == 16384 else None
        # CPU baseline: the oracle, single thread, on a bounded row sample.
        cpu_rows = 512
        n, dt = cpu_sample(in_np, dem.affine, dem.nodata, cpu_rows, 1)
        n2, dt2 = cpu_sample(in_np, dem.affine, dem.nodata, cpu_rows, 1)
        cpu_val = (n + n2) / (dt + dt2) / 1e9
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD if H == 16384 else WORKLOAD.replace("16384x16384", f"{H}x{W}"),
                       "pixels": px, "bytes_per_pixel": BYTES_PER_PX,
                       "l2": "inputs+outputs (3.5 GB/step) exceed L2; no flush",
                       "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
                       "autotuned": {"rows_per_tile": tuned["shape"][0], "tma_stages": tuned["shape"][1],
                                     "threads_per_cta": tuned["shape"][2], "ctas_per_sm": tuned["shape"][3],
                                     "ms_by_config": {str(k): round(v, 4) for k, v in tuned["ms"].items()}},
                       "error_vs_fp64": errors},
            "gpu_launches": args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": traffic, "peak_source": peak_kind,
                         "kernel": "horn_f32_tma", "launch_ms": lmed},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d_b, "d2h_bytes_per_step": d2h_b,
                    "ms_per_step": e2e_s * 1e3, "host_link": link, "link_bound_ms": link_ms,
                    "frac_of_link": link_ms / (e2e_s * 1e3), "phases_ms": phase_ms},
            "cpu_baseline": {"value": cpu_val, "unit": UNIT, "cores": 1, "kind": "port",
                             "sample": f"2 x {cpu_rows} rows x {W} px (1-row halo) of the same DEM, reference "
                                       "float64 numpy algorithm, 3 calls (slope, aspect, hillshade), 1 thread"},
            "clocks": clocks,
        }
        del outs, r, host_in, host_out, in_np, out_np
        torch.cuda.empty_cache()
        if ws == 1 and not args.no_secondary and H == 16384:
            secondary = {}
            for key, leg in (("C1_slope2048", leg_slope2048), ("C3_conv8192", leg_conv),
                             ("C4_batch512", leg_batch), ("C5_multiband", leg_multiband),
                             ("f1_stream_conv", leg_stream), ("f2_derivatives", leg_derivatives),
                             ("f3_focal_stats", leg_focal_stats), ("f4_decode", leg_decode)):
                try:
                    secondary[key] = leg(args, dev, local)
                except Exception as exc:  # a failed leg is reported, the headline still prints
                    secondary[key] = {"error": f"{type(exc).__name__}: {exc}"}
                torch.cuda.empty_cache()
            line["config"]["secondary"] = secondary
            line["gpu_launches_secondary"] = {k: v.get("gpu_launches") for k, v in secondary.items()}
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


# ------------------------------------------------------- secondary legs --
def leg_slope2048(args, dev, gpu) -> dict:
    """C1: 2048^2 fBm DEM (1 % nodata), GPU slope vs the reference's CPU fallback on the whole raster."""
    import torch

    import oracle  # checker and CPU baseline only
    import vsr_gb300 as vsr
    from vsr_gb300 import algebra, workloads

    dem = workloads.terrain_2048(device=dev)
    H, W = dem.data.shape
    r = vsr.from_device(dem.data, nodata=dem.nodata, affine=dem.affine)
    out = torch.empty((1, H, W), dtype=torch.float32, device=dev)
    fn = lambda: algebra.horn_fused(r, slope=True, aspect=False, hillshade=False, out=(out, None, None))  # noqa: E731
    for _ in range(max(3, args.warmup)):
        fn()
    ms, n, clocks = timed_region(fn, args.steps, gpu)
    hbm, _, src = _peaks()
    host = dem.data.cpu().numpy()
    t0 = time.perf_counter()
    ref, _ = oracle.slope_aspect(host, dem.affine, dem.nodata, compute_slope=True, compute_aspect=False)
    cpu_s = time.perf_counter() - t0
    got = out[0].cpu().numpy()
    m = ref != dem.nodata
    px = H * W
    ach = 8 * px / (ms * 1e-3) / 1e9
    return {
        "workload": "Horn slope (degrees), 2048x2048 f32 fBm DEM 0-3000 m, 30 m cells, 1 % nodata -9999",
        "value": px / (ms * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": ms, "steps": n, "gpu_launches": 1,
        "l2": "16 MiB in + 16 MiB out fit in L2: back-to-back launches, no flush (small-raster case)",
        "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                     "peak_source": src, "kernel": "horn_f32_tma (slope only)", "bytes_per_px": 8},
        "cpu_baseline": {"value": px / cpu_s / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": "the whole 2048^2 DEM, reference float64 slope algorithm, 1 thread"},
        "error_vs_fp64": {"slope_deg": _abs_err_stats(got[m], ref[m]),
                          "nodata_placement_exact": bool(np.array_equal(got == dem.nodata, ref == dem.nodata)),
                          "sample": "whole raster"},
        "clocks": clocks,
    }


def _conv_strip_errors(x_t, out_t, w, rows: int, n: int, seed: int) -> dict:
    """Convolution output vs the float64 oracle on ``n`` row strips (with k//2 halo rows)."""
    import oracle

    H = x_t.shape[0]
    kh = w.shape[0]
    samples = []
    for y0 in _strip_starts(H, rows, n, seed):
        lo, hi = max(0, y0 - kh // 2), min(H, y0 + rows + kh // 2)
        z = x_t[lo:hi].cpu().numpy()
        ref = oracle.convolve_normalized(z, w, None)[y0 - lo:y0 - lo + rows]
        samples.append((out_t[0, y0:y0 + rows].cpu().numpy(), ref, 1e-3 * float(np.mean(np.abs(z)))))
    st = _rel_err_samples(samples)
    st["sample"] = f"{n} strips of {rows} rows (first, last, seeded); |out - ref| / |ref|"
    return st


def leg_conv(args, dev, gpu) -> dict:
    """C3: 8192^2 trend+noise raster, normalised convolution, plain FP32 vs split-BF16, float64 output."""
    import torch

    import oracle  # checker and CPU baseline only
    import vsr_gb300 as vsr
    from vsr_gb300 import algebra, workloads

    H = W = 8192
    x = workloads.trend_noise(H, W, device=dev)
    r = vsr.from_device(x)
    kernels = {"k15": workloads.random_weights(15, 215), "k31": workloads.random_weights(31, 231),
               "gauss41": oracle.gaussian_weights(5.0, 41)}
    out64 = torch.empty((1, H, W), dtype=torch.float64, device=dev)
    out32 = torch.empty((1, H, W), dtype=torch.float32, device=dev)
    hbm, bf16, src = _peaks()
    res = {}
    clocks = None
    for name, w in kernels.items():
        k = w.shape[0]
        t = {}
        for prec in ("fp32", "split"):
            for odt, o in ((np.float64, out64), (np.float32, out32)):
                fn = lambda: algebra.convolve_bands(r, w, precision=prec, out_dtype=odt, out=o)  # noqa: E731
                for _ in range(max(3, args.warmup)):
                    fn()
                ms, n, ck = timed_region(fn, max(5, args.steps // 5), gpu, min_seconds=0.6)
                t[(prec, np.dtype(odt).name)] = ms
                if name == "k31" and prec == "split" and o is out64:
                    clocks = ck
            # error of the float64-output form against the float64 oracle
            algebra.convolve_bands(r, w, precision=prec, out_dtype=np.float64, out=out64)
            torch.cuda.synchronize()
            t[(prec, "err")] = _conv_strip_errors(x, out64, w, rows=32, n=3, seed=k)
        kp = ((64 + k - 1) + 15) // 16 * 16
        # 3 split products per kernel row; a 128 x 64 output tile multiplies
        # K = kp (window width rounded to 16): 2 * kp flops per output per row
        issued = 3 * 2 * H * W * k * kp
        ms_tc = t[("split", "float64")]
        res[name] = {"k": k, "fp32_ms": t[("fp32", "float64")], "split_ms": ms_tc,
                     "speedup_split_vs_fp32": t[("fp32", "float64")] / ms_tc,
                     "fp32_gpix_s": H * W / t[("fp32", "float64")] / 1e6, "split_gpix_s": H * W / ms_tc / 1e6,
                     "f32_output": {"fp32_ms": t[("fp32", "float32")], "split_ms": t[("split", "float32")]},
                     "useful_tflops_split": 2 * k * k * H * W / ms_tc / 1e9,
                     "issued_tensor_tflops": issued / ms_tc / 1e9,
                     "error_vs_fp64": {"split": t[("split", "err")], "fp32": t[("fp32", "err")]}}
    crop = x[:1024, :1024].cpu().numpy()
    t0 = time.perf_counter()
    oracle.convolve_normalized(crop, kernels["k31"], None)
    cpu_s = time.perf_counter() - t0
    main = res["k31"]
    ach = main["issued_tensor_tflops"]
    return {
        "workload": "normalised focal convolution, 8192x8192 f32 U[0,1)+0-100 trend, no nodata, float64 output "
                    "(the reference's dtype); headline kernel 31x31 split precision (BF16 high parts, F16 low part)",
        # per call: band images + summed-area table + largest-value scan + the tensor-core kernel
        "value": main["split_gpix_s"], "unit": UNIT, "ms_per_step": main["split_ms"], "gpu_launches": 4,
        "kernels": res, "l2": "256 MiB in + 512 MiB out per step exceed L2; no flush",
        "roofline": {"bound": "tensor", "achieved": ach, "peak": bf16, "unit": "TFLOP/s", "frac": ach / bf16,
                     "peak_source": src, "kernel": "conv_tc_kernel",
                     "flops": "issued MMA flops: 3 split products x 2 x Kp per output per kernel row"},
        "cpu_baseline": {"value": 1024 * 1024 / cpu_s / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": "1024x1024 crop, 31x31 kernel, float64 scipy correlate restatement, 1 thread"},
        "clocks": clocks,
    }


def leg_batch(args, dev, gpu) -> dict:
    """C4: 512 uneven DEM tiles, slope + aspect + 5x5 Gaussian: one graph-replayed
    persistent launch vs the same per-tile launches captured in a graph."""
    import torch

    import oracle  # checker and CPU baseline only
    import vsr_gb300 as vsr
    from vsr_gb300 import batch, workloads

    tiles = workloads.tile_batch(device=dev)
    rasters = [vsr.from_device(t.data, nodata=t.nodata, affine=t.affine) for t in tiles]
    px = sum(int(t.data.numel()) for t in tiles)
    b = batch.TerrainBatch(rasters, sigma=1.0, kernel_size=5)
    tuned = batch.autotune_batch(b)
    b.capture()
    for _ in range(max(3, args.warmup)):
        b.replay()
    t_batch, n, clocks = timed_region(b.replay, args.steps, gpu)
    per = batch.PerTileGraph(rasters, sigma=1.0, kernel_size=5)
    for _ in range(max(3, args.warmup)):
        per.replay()
    t_per, n_per, _ = timed_region(per.replay, max(3, args.steps // 5), gpu, min_seconds=0.6)
    # errors on sampled tiles (the batched outputs of the last replay)
    b.replay()
    torch.cuda.synchronize()
    es, ea, eg = [], [], []
    for i in range(0, len(tiles), 64):
        t = tiles[i]
        z = t.data.cpu().numpy()
        rs, ra = oracle.slope_aspect(z, t.affine, t.nodata)
        rg = oracle.convolve_normalized(z, oracle.gaussian_weights(1.0, 5), t.nodata)
        s, a, g = (o.cpu().numpy() for o in b.outputs[i])
        nd_s = np.isnan(rs) if np.isnan(t.nodata) else rs == t.nodata
        es.append((s[~nd_s], rs[~nd_s]))
        ea.append((a[~nd_s], ra[~nd_s]))
        nd_g = np.isnan(rg) if np.isnan(t.nodata) else rg == t.nodata
        eg.append((g[~nd_g], rg[~nd_g], 1e-3 * float(np.nanmean(np.abs(np.where(z == t.nodata, np.nan, z))))))
    cat = lambda L, i: np.concatenate([x[i] for x in L])  # noqa: E731
    hbm, _, src = _peaks()
    ach = 16 * px / (t_batch * 1e-3) / 1e9
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
    return {
        "workload": "512 f32 fBm tiles, sides log-uniform [256,4096], cell U[1,90] m, nodata -9999/NaN on 0-5%; "
                    "slope+aspect + 5x5 Gaussian (sigma 1)",
        "value": px / (t_batch * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": t_batch, "steps": n, "gpu_launches": 1,
        "pixels": px, "bytes_per_pixel": 16, "batched_ms": t_batch, "per_tile_graph_ms": t_per,
        "speedup_vs_per_tile_graph": t_per / t_batch, "per_tile_launches": per.launches,
        "autotuned": {"config": batch.BATCH_CONFIGS[tuned["config"]],
                      "ms_by_config": {str(k): round(v, 4) for k, v in tuned["ms"].items()}},
        "l2": "3.9 GB in + 11.8 GB out per step exceed L2; no flush",
        "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                     "peak_source": src, "kernel": "batch_terrain_kernel"},
        "cpu_baseline": {"value": spx / cpu_s / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": "first 8 tiles: reference slope, aspect (2 calls) + float64 5x5 Gaussian, 1 thread"},
        "error_vs_fp64": {"slope_deg": _abs_err_stats(cat(es, 0), cat(es, 1)),
                          "aspect_deg": _abs_err_stats(cat(ea, 0), cat(ea, 1), circular=True),
                          "gaussian_rel": _rel_err_samples(eg),
                          "sample": "every 64th tile (8 tiles), nodata excluded; Gaussian |out - ref| / |ref|"},
        "clocks": clocks,
    }


def leg_multiband(args, dev, gpu) -> dict:
    """C5: 12 x 10980^2 uint16 stack, 7x7 focal mean + Gaussian sigma 8 (65x65), all bands per launch."""
    import torch

    import oracle  # checker and CPU baseline only
    import vsr_gb300 as vsr
    from vsr_gb300 import algebra, workloads

    stack = workloads.gamma_stack(device=dev)
    B, H, W = stack.shape
    r = vsr.from_device(stack, nodata=0)
    mean = torch.empty((B, H, W), dtype=torch.float32, device=dev)
    gauss = torch.empty((B, H, W), dtype=torch.float32, device=dev)

    # the Gaussian on "auto": the split-precision tensor-core line passes for
    # this uint16 stack (65 x 65 >= 35)
    def step():
        algebra.focal_mean_bands(r, 3, 3, out_dtype=np.float32, out=mean)
        algebra.gaussian_bands(r, 8.0, 65, precision="auto", out_dtype=np.float32, out=gauss)

    for _ in range(max(3, args.warmup)):
        step()
    t, n, clocks = timed_region(step, 3, gpu)
    t_mean, _, _ = timed_region(lambda: algebra.focal_mean_bands(r, 3, 3, out_dtype=np.float32, out=mean), 3, gpu,
                                min_seconds=0.3)
    t_tc, _, _ = timed_region(lambda: algebra.gaussian_bands(r, 8.0, 65, precision="split",
                                                             out_dtype=np.float32, out=gauss), 3, gpu, min_seconds=0.3)
    t_fp32, _, _ = timed_region(lambda: algebra.gaussian_bands(r, 8.0, 65, precision="fp32", out_dtype=np.float32,
                                                               out=gauss), 3, gpu, min_seconds=0.3)
    step()
    torch.cuda.synchronize()
    hbm, bf16, src = _peaks()
    px = B * H * W
    # errors on crops of the first, a middle and the last band (with halo), nodata outputs excluded
    em, eg = [], []
    w65 = oracle.gaussian_weights(8.0, 65)
    for b_, (y0, x0) in ((0, (0, 0)), (B - 1, (H - 256, W - 256)), (B // 2, (H // 2, W // 3))):
        lo_y, lo_x = max(0, y0 - 32), max(0, x0 - 32)
        hi_y, hi_x = min(H, y0 + 256 + 32), min(W, x0 + 256 + 32)
        z = stack[b_, lo_y:hi_y, lo_x:hi_x].cpu().numpy()
        sl = (slice(y0 - lo_y, y0 - lo_y + 256), slice(x0 - lo_x, x0 - lo_x + 256))
        rm = oracle.focal_mean(z, 3, 3, 0)[sl]
        rg = oracle.convolve_normalized(z, w65, 0)[sl]
        gm = mean[b_, y0:y0 + 256, x0:x0 + 256].cpu().numpy()
        gg = gauss[b_, y0:y0 + 256, x0:x0 + 256].cpu().numpy()
        em.append((gm[rm != 0], rm[rm != 0]))
        eg.append((gg[rg != 0], rg[rg != 0], 1e-3 * float(np.mean(z))))
    cat = lambda L, i: np.concatenate([x[i] for x in L])  # noqa: E731
    crop = stack[0, :1024, :1024].cpu().numpy()
    t0 = time.perf_counter()
    oracle.focal_mean(crop, 3, 3, 0)
    cpu_mean_s = (time.perf_counter() - t0) / (1024 * 1024)
    crop = stack[0, :256, :256].cpu().numpy()
    t0 = time.perf_counter()
    oracle.convolve_normalized(crop, w65, 0)
    cpu_gauss_s = (time.perf_counter() - t0) / (256 * 256)
    ach = 10 * px / (t * 1e-3) / 1e9
    return {
        "workload": "12 x 10980x10980 uint16 gamma(2,800) clipped 0-10000, 3% nodata 0; focal mean 7x7 + Gaussian "
                    "sigma 8 (65x65), all bands per launch, float32 outputs",
        "value": px / (t * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": t, "steps": n, "dtype": "u16 in, f32 out",
        # per step: the focal mean (all bands), the Gaussian band image, the two
        # line passes over all bands
        "gpu_launches": 4,
        "focal_mean_ms": t_mean, "focal_mean_gpix_s": px / (t_mean * 1e-3) / 1e9,
        "focal_mean_hbm_frac": 6 * px / (t_mean * 1e-3) / 1e9 / hbm,
        "gaussian_path": "auto = split-precision tensor-core line passes (row pass: exact byte planes x F16 hi/lo weights; column pass: F16 hi/lo row sums; FP32 accumulate)",
        "gaussian_tensor_core_ms": t_tc, "gaussian_fp32_ms": t_fp32, "gaussian_tensor_core_vs_fp32": t_fp32 / t_tc,
        "l2": "2.9 GB in + 11.6 GB out per step exceed L2; no flush",
        "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                     "peak_source": src, "kernel": "box_warp_int + gauss_row_kernel + gauss_col_kernel", "bytes_per_px": 10},
        "cpu_baseline": {"value": 1.0 / (cpu_mean_s + cpu_gauss_s) / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": "band 0: 7x7 focal mean on a 1024^2 crop + 65x65 Gaussian (dense float64 "
                                   "correlate, as the reference's dense kernel) on a 256^2 crop, per-pixel times "
                                   "summed, 1 thread"},
        "error_vs_fp64": {"focal_mean_rel": _rel_err_stats(cat(em, 0), cat(em, 1), 1.0),
                          "gaussian_rel": _rel_err_samples(eg),
                          "sample": "256^2 crops of bands 0, 6 and 11 (with a 32-px halo), nodata excluded; "
                                    "|out - ref| / |ref|"},
        "clocks": clocks,
    }


def leg_derivatives(args, dev, gpu) -> dict:
    """TRI + TPI + profile curvature in one pass over the 16384^2 fBm DEM (float64 out, the reference dtype)."""
    import torch

    import oracle  # checker and CPU baseline only
    import vsr_gb300 as vsr
    from vsr_gb300 import algebra, workloads

    dem = workloads.terrain_16k(device=dev, size=args.dem_size)
    H, W = dem.data.shape
    r = vsr.from_device(dem.data, nodata=dem.nodata, affine=dem.affine)
    outs = tuple(torch.empty((1, H, W), dtype=torch.float64, device=dev) for _ in range(3))
    fn = lambda: algebra.terrain_derivatives(r, out=outs)  # noqa: E731
    for _ in range(max(3, args.warmup)):
        fn()
    ms, n, clocks = timed_region(fn, max(5, args.steps // 5), gpu)
    hbm, _, src = _peaks()
    strip = dem.data[:512].cpu().numpy()
    t0 = time.perf_counter()
    for k in (oracle.TRI, oracle.TPI, oracle.CURVATURE):
        oracle.terrain_derivative(strip, dem.affine, dem.nodata, k)
    cpu_s = (time.perf_counter() - t0) / strip.size
    px = H * W
    ach = 28 * px / (ms * 1e-3) / 1e9
    return {
        "workload": f"TRI + TPI + profile curvature, {H}x{W} f32 fBm DEM 0-4500 m, 10 m cells, 200 -9999 disc "
                    "holes; one pass, float64 outputs",
        "value": px / (ms * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": ms, "steps": n, "gpu_launches": 1,
        "l2": "1 GiB in + 6 GiB out per step exceed L2; no flush",
        "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                     "peak_source": src, "kernel": "terrain_deriv_kernel<float>", "bytes_per_px": 28},
        "cpu_baseline": {"value": 1.0 / cpu_s / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": "512 x 16384 rows of the same DEM, reference float64 TRI, TPI, curvature "
                                   "(3 calls), 1 thread"},
        "clocks": clocks,
    }


def leg_focal_stats(args, dev, gpu) -> dict:
    """Focal min / max / std / range / variety (7 x 7) on one 10980^2 uint16 band of the multiband workload."""
    import torch

    import oracle  # checker and CPU baseline only
    import vsr_gb300 as vsr
    from vsr_gb300 import algebra, workloads

    band = workloads.gamma_stack(bands=1, device=dev)
    _, H, W = band.shape
    r = vsr.from_device(band, nodata=0)
    out = torch.empty((1, H, W), dtype=torch.float32, device=dev)
    hbm, _, src = _peaks()
    px = H * W
    per, clocks = {}, None
    crop = band[0, 2000:2256 + 6, 3000:3256 + 6].cpu().numpy()
    for stat in ("min", "max", "std", "range", "variety"):
        fn = lambda: algebra.focal_stat_bands(r, stat, 3, 3, out_dtype=np.float32, out=out)  # noqa: E731
        for _ in range(3):
            fn()
        ms, n, ck = timed_region(fn, 3, gpu, min_seconds=0.3)
        if stat == "std":
            clocks = ck
        got = out[0, 2003:2259, 3003:3259].cpu().numpy().astype(np.float64)
        t0 = time.perf_counter()
        ref = oracle.focal_stat(crop, 3, 3, 0, stat)[3:-3, 3:-3]
        cpu_s = (time.perf_counter() - t0) / ref.size
        m = np.isfinite(ref)
        err = np.abs(got[m] - ref[m]) / np.maximum(np.abs(ref[m]), 1.0)
        per[stat] = {"ms": ms, "gpix_s": px / (ms * 1e-3) / 1e9, "hbm_frac": 6 * px / (ms * 1e-3) / 1e9 / hbm,
                     "cpu_gpix_s": 1.0 / cpu_s / 1e9, "max_rel_err_vs_fp64": float(err.max()),
                     "exact": bool(np.array_equal(got[m], ref[m].astype(np.float32).astype(np.float64)))}
    ms = per["std"]["ms"]
    return {
        "workload": f"focal min/max/std/range/variety, 7x7 window, one {H}x{W} uint16 band (gamma(2,800) clipped "
                    "0-10000, 3% nodata 0), float32 outputs; headline figure: std",
        "value": px / (ms * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": ms, "gpu_launches": 1, "stats": per,
        "l2": "241 MB in + 482 MB out per call exceed L2; no flush",
        "roofline": {"bound": "hbm", "achieved": 6 * px / (ms * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
                     "frac": 6 * px / (ms * 1e-3) / 1e9 / hbm, "peak_source": src,
                     "kernel": "focal_stat_kernel<int, std>", "bytes_per_px": 6},
        "cpu_baseline": {"value": per["std"]["cpu_gpix_s"], "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": "256^2 crop (3-px halo), reference CPU focal statistic (the oracle's "
                                   "sliding-window restatement), 1 thread, per statistic in 'stats'"},
        "clocks": clocks,
    }


def leg_decode(args, dev, gpu) -> dict:
    """GeoTIFF decode onto the GPU: an 8192^2 float32 DEM, 512^2 DEFLATE tiles, floating-point predictor."""
    import tempfile
    import zlib as _zlib

    import torch

    import vsr_gb300 as vsr
    from vsr_gb300 import io, workloads

    dem = workloads.terrain_16k(device=dev, size=8192)
    host = dem.data.cpu().numpy()
    H, W = host.shape
    px = H * W
    with tempfile.TemporaryDirectory() as tmp:
        path = Path(tmp) / "dem.tif"
        io.write_raster(path, vsr.from_numpy(host, nodata=dem.nodata, affine=dem.affine), blockxsize=512,
                        blockysize=512, level=1)
        size = path.stat().st_size
        fn = lambda: io.read_raster(path, residency=vsr.Residency.DEVICE)  # noqa: E731
        r = fn()
        ok = bool(torch.equal(r.device_data(), dem.data))
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        sampler = ClockSampler(gpu).start()
        reps = 5
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        e2e_s = (time.perf_counter() - t0) / reps
        clocks = sampler.stop()
        # the device half alone (byte planes undone and tiles assembled): time the
        # kernel through the C ABI on already inflated chunks
        with open(path, "rb") as f:
            t = io._read_ifds(f)[0].tags
        offs, cnts, geo = io._chunk_layout(t, H, W, 1, False)
        with open(path, "rb") as f:
            raw = []
            for o, c in zip(offs, cnts):
                f.seek(int(o))
                raw.append(f.read(int(c)))
        t0 = time.perf_counter()
        parts = [_zlib.decompress(b) for b in raw[:16]]
        cpu_inflate_s = (time.perf_counter() - t0) / (16 * 512 * 512)
        parts = [_zlib.decompress(b) for b in raw]
    offsets = np.cumsum([0] + [len(p) for p in parts])
    staged0 = torch.from_numpy(np.frombuffer(b"".join(parts), np.uint8).copy()).to(dev)
    table = np.zeros(len(parts), dtype=[("offset", "<i8"), ("x0", "<i4"), ("y0", "<i4"), ("width", "<i4"),
                                        ("height", "<i4"), ("band", "<i4"), ("pad", "<i4")])
    for k, g in enumerate(geo):
        table[k] = (offsets[k], g[0], g[1], g[2], g[3], 0, 0)
    chunks = torch.from_numpy(table.view(np.uint8).copy()).to(dev)
    staged = torch.empty_like(staged0)
    outt = torch.empty((H, W), dtype=torch.int32, device=dev)
    from vsr_gb300 import _lib

    lib = _lib.load()

    def kern():
        staged.copy_(staged0)  # predictor 3 works in place
        _lib.check(lib.vsr_tiff_assemble(staged.data_ptr(), chunks.data_ptr(), len(parts), 512, 4, 1, 0, 3, 0, H, W,
                                         outt.data_ptr(), H * W, W, torch.cuda.current_stream().cuda_stream),
                   "vsr_tiff_assemble")

    kern()
    ms_copy, _, _ = timed_region(lambda: staged.copy_(staged0), 3, gpu, min_seconds=0.2)
    ms_all, n, _ = timed_region(kern, 3, gpu, min_seconds=0.3)
    ms_k = max(ms_all - ms_copy, 1e-6)
    hbm, _, src = _peaks()
    ach = 12 * px / (ms_k * 1e-3) / 1e9
    # CPU baseline: the host decode of the same tiles (inflate + byte planes undone + tiles placed), numpy, 1 thread
    t0 = time.perf_counter()
    for k in range(4):
        b = np.frombuffer(parts[k], np.uint8).reshape(512, -1)
        d = np.cumsum(b, axis=1, dtype=np.uint8)
        np.ascontiguousarray(d.reshape(512, 4, 512).transpose(0, 2, 1)).view(">f4")
    cpu_s = (time.perf_counter() - t0) / (4 * 512 * 512) + cpu_inflate_s
    return {
        "workload": f"read_raster of a {H}x{W} float32 fBm DEM GeoTIFF ({size / 1e6:.0f} MB), 512x512 DEFLATE tiles, "
                    "floating-point predictor, into device memory; headline: the device half (byte planes undone, "
                    "tiles assembled), e2e: the whole call (host directory + inflate on 8 threads + one H2D copy)",
        "value": px / (ms_k * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": ms_k, "steps": n, "gpu_launches": 1,
        "kernel_ms_note": "time of (restore the staged bytes + assemble) minus the restore copy alone",
        "decoded_equals_source": ok,
        "e2e": {"value": px / e2e_s / 1e9, "unit": UNIT, "ms_per_call": e2e_s * 1e3, "h2d_bytes_per_call": size},
        "l2": "268 MB in place + 268 MB out per call exceed L2; no flush",
        "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                     "peak_source": src, "kernel": "tiff_assemble_kernel (one warp per chunk row)",
                     "bytes_per_px": 12},
        "cpu_baseline": {"value": 1.0 / cpu_s / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": "16 tiles inflated (zlib) + 4 tiles' byte planes undone (numpy), per-pixel "
                                   "times summed, 1 thread"},
        "clocks": clocks,
    }


def leg_stream(args, dev, gpu) -> dict:
    """Streamed host-to-host 31 x 31 convolution of the 8192^2 raster (row strips with the kernel's halo)."""
    import torch

    import vsr_gb300 as vsr
    from vsr_gb300 import stream, workloads

    x = workloads.trend_noise(8192, 8192, device=dev).cpu()
    host = torch.empty(x.shape, dtype=torch.float32, pin_memory=True)
    host.copy_(x)
    r = vsr.from_numpy(host.numpy())
    w = workloads.random_weights(31, 231)
    fn = lambda: stream.raster_convolve_host(r, w, precision="split", out_dtype=np.float32, strip_rows=1024)  # noqa: E731
    fn()
    torch.cuda.synchronize()
    sampler = ClockSampler(gpu).start()
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        fn()
    dt = (time.perf_counter() - t0) / reps
    clocks = sampler.stop()
    px = 8192 * 8192
    link = host_link_peak(dev)
    link_ms = max(px * 4 / (link["h2d_gbs"] * 1e9), px * 4 / (link["d2h_gbs"] * 1e9)) * 1e3
    return {
        "workload": "raster_convolve_host: 8192x8192 f32 U[0,1)+trend from pinned host memory, 31x31 split "
                    "precision, float32 result in (pageable) host memory, 1024-row strips + 30 halo rows, 3 streams",
        "value": px / dt / 1e9, "unit": UNIT, "ms_per_step": dt * 1e3, "gpu_launches": 4 * 8,
        "host_link": link, "link_bound_ms": link_ms, "frac_of_link": link_ms / (dt * 1e3),
        "roofline": {"bound": "host link", "achieved": 8 * px / dt / 1e9, "peak": link["duplex_gbs"], "unit": "GB/s",
                     "frac": 8 * px / dt / 1e9 / link["duplex_gbs"], "peak_source": "measured (this run)",
                     "kernel": "copies + conv_tc_kernel per strip", "bytes_per_px": 8},
        "cpu_baseline": None,
        "clocks": clocks,
    }


LEGS = {"slope2048": leg_slope2048, "conv": leg_conv, "batch": leg_batch, "multiband": leg_multiband,
        "derivatives": leg_derivatives, "focal_stats": leg_focal_stats, "decode": leg_decode, "stream": leg_stream}


def run_leg(args, ws, rank, local):
    """One workload alone, printed as its own JSON line (profiling runs)."""
    import torch

    import vsr_gb300 as vsr

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    vsr.load_library()
    d = LEGS[args.workload](args, dev, local)
    if rank != 0:
        return
    line = {"metric": METRIC, "value": d.pop("value"), "unit": d.pop("unit"), "n_gpus": ws, "steps": d.get("steps"),
            "warmup": args.warmup, "ms_per_step": d.pop("ms_per_step"), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": d.pop("dtype", "f32"), "data": "synthetic",
            "gpu_launches": d.pop("gpu_launches"), "roofline": d.pop("roofline"),
            "cpu_baseline": d.pop("cpu_baseline"), "clocks": d.pop("clocks"), "config": d}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["vsr", "reference"], default="vsr")
    ap.add_argument("--workload", choices=["terrain", *LEGS], default="terrain",
                    help="terrain (default, the headline, with the others as secondary legs): fused "
                         "slope+aspect+hillshade on 16384^2; conv: 8192^2 focal convolution, plain FP32 vs "
                         "split-BF16; batch: 512 uneven tiles, one graph-replayed persistent launch vs per-tile "
                         "launches; multiband: 12 x 10980^2 uint16 focal mean 7x7 + Gaussian 65x65; slope2048: "
                         "slope on a 2048^2 DEM vs the reference CPU fallback; derivatives: TRI + TPI + curvature "
                         "on the 16384^2 DEM; focal_stats: min/max/std/range/variety 7x7 on a 10980^2 uint16 "
                         "band; decode: GeoTIFF read onto the GPU; stream: host-to-host streamed convolution")
    ap.add_argument("--no-secondary", action="store_true", help="headline only (skip the other configurations)")
    ap.add_argument("--dem-size", type=int, default=16384,
                    help="DEM side (the benchmark workload is 16384; smaller sizes are for profiling)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local = _dist_env()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    elif args.workload == "terrain":
        run_vsr(args, ws, rank, local)
    else:
        run_leg(args, ws, rank, local)


if __name__ == "__main__":
    main()
