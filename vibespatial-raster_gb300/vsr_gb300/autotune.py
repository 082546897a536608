"""Launch-configuration autotuner for the tunable libvsr kernels.

libvsr keeps, per tunable operation, a small table of launch configurations
(for the fused Horn kernel: output rows per tile, TMA pipeline stages,
threads per CTA and the CTAs per SM its register budget is sized for).  ``autotune_horn`` times every configuration on the
caller's own raster with CUDA events, selects the fastest through
``vsr_tuning_set`` and records the choice in an on-disk cache keyed by
(operation, raster size class, dtype, SM count) so later processes apply it
without re-timing (``apply_cached``).  The reference has no tuning: its
launches use one fixed 16 x 16 block (algebra.py:2323-2338).
"""

from __future__ import annotations

import json
import os
from pathlib import Path

from vsr_gb300 import _lib

HORN_CONFIGS = [  # mirrors kHornConfigs in csrc/horn.cu:
    # (rows per tile, TMA stages, threads per CTA, CTAs per SM the registers are sized for)
    (64, 2, 128, 4), (48, 2, 128, 4), (32, 2, 128, 4), (32, 2, 128, 5), (64, 2, 256, 2),
]


def cache_path() -> Path:
    base = os.environ.get("VSR_GB300_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "vsr_gb300")
    return Path(base) / "tuning.json"


def _load_cache() -> dict:
    p = cache_path()
    try:
        return json.loads(p.read_text())
    except (OSError, ValueError):
        return {}


def _store_cache(d: dict) -> None:
    p = cache_path()
    try:
        p.parent.mkdir(parents=True, exist_ok=True)
        tmp = p.with_suffix(".tmp")
        tmp.write_text(json.dumps(d, indent=1, sort_keys=True))
        os.replace(tmp, p)
    except OSError:
        pass  # a read-only home only costs re-tuning


def _size_class(h: int, w: int) -> str:
    def c(n):
        return 1 << max(0, (int(n) - 1).bit_length())

    return f"{c(h)}x{c(w)}"


def _sm_count() -> int:
    import ctypes

    lib = _lib.load()
    n = ctypes.c_int(0)
    _lib.check(lib.vsr_device_info(ctypes.byref(n), None, None), "vsr_device_info")
    return n.value


def cache_key(op: str, h: int, w: int, dtype: str) -> str:
    return f"{op}|{_size_class(h, w)}|{dtype}|sm{_sm_count()}"


def apply_cached(op: str, h: int, w: int, dtype: str = "float32") -> int | None:
    """Apply a cached choice for this problem class; returns it or None."""
    key = cache_key(op, h, w, dtype)
    hit = _load_cache().get(key)
    if hit is None:
        return None
    lib = _lib.load()
    _lib.check(lib.vsr_tuning_set(_lib.VSR_OP_HORN if op == "horn" else _lib.VSR_OP_BATCH, int(hit["config"])),
               "vsr_tuning_set")
    return int(hit["config"])


def autotune_horn(dem, *, repeats: int = 8, rounds: int = 3, outputs=None) -> dict:
    """Time every Horn launch configuration on ``dem`` and keep the fastest.

    Each configuration runs ``repeats`` launches back to back between one
    pair of CUDA events (the steady state a pipeline of launches sees, not
    an isolated launch); the configurations take turns for ``rounds`` rounds
    and each keeps its best round, so clock and neighbour drift during the
    tuning does not decide the choice.  ``dem`` is an OwnedRasterArray;
    ``outputs`` optional preallocated output tensors (as for
    ``algebra.horn_fused(out=...)``).  Returns {"config": i, "shape": (rows,
    stages, threads, CTAs per SM), "ms": {i: best mean ms per launch}}.
    """
    import torch

    from vsr_gb300 import algebra

    lib = _lib.load()
    n = lib.vsr_tuning_count(_lib.VSR_OP_HORN)
    stream = torch.cuda.current_stream()
    times = {cfg: float("inf") for cfg in range(n)}
    for cfg in range(n):  # warm-up: the first launch of each shape sets its attributes
        _lib.check(lib.vsr_tuning_set(_lib.VSR_OP_HORN, cfg), "vsr_tuning_set")
        algebra.horn_fused(dem, out=outputs)
    for _ in range(rounds):
        for cfg in range(n):
            _lib.check(lib.vsr_tuning_set(_lib.VSR_OP_HORN, cfg), "vsr_tuning_set")
            algebra.horn_fused(dem, out=outputs)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(repeats):
                algebra.horn_fused(dem, out=outputs)
            b.record(stream)
            b.synchronize()
            times[cfg] = min(times[cfg], a.elapsed_time(b) / repeats)
    best = min(times, key=times.get)
    _lib.check(lib.vsr_tuning_set(_lib.VSR_OP_HORN, best), "vsr_tuning_set")
    key = cache_key("horn", dem.height, dem.width, str(dem.dtype))
    cache = _load_cache()
    cache[key] = {"config": best, "shape": list(HORN_CONFIGS[best]), "ms": times[best]}
    _store_cache(cache)
    return {"config": best, "shape": HORN_CONFIGS[best], "ms": times}
