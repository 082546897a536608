"""Generate golden input/output vectors from the reference's own CPU code.

Run in a container where the reference source tree is present:

    python tests/golden/make_golden.py --reference <path to the reference source tree>

The reference package (vibespatial-raster 0.1.7) imports two modules from its
external core runtime (``vibespatial.residency`` and ``vibespatial.runtime``)
that are not installed.  The small stand-ins below provide only the names the
CPU code paths touch; nothing numeric is stubbed.  The reference's CPU
functions then run unmodified:

* ``raster_slope`` / ``raster_aspect`` with ``use_gpu=False``
  -> ``_cpu_slope_aspect``        (src/vibespatial/raster/algebra.py:2162-2249)
* ``raster_hillshade`` with ``use_gpu=False``
  -> ``_hillshade_cpu``           (algebra.py:2543-2629)
* ``raster_focal_mean`` with ``use_gpu=False``
  -> ``_focal_mean_cpu``          (algebra.py:3083-3101)
* ``raster_tri`` / ``raster_tpi`` / ``raster_curvature`` with ``use_gpu=False``
  -> ``_terrain_derivative_cpu``  (algebra.py:3352-3445)
* ``raster_focal_min`` / ``_max`` / ``_std`` / ``_range`` / ``_variety`` with
  ``use_gpu=False`` -> ``_focal_*_cpu``  (algebra.py:3041-3164)
* ``raster_gaussian_filter`` / ``raster_convolve`` weight handling
  (algebra.py:2101-2154): the reference has no CPU convolution, so the
  weights it hands to ``_gpu_convolve`` are captured by replacing that one
  function with a recorder.

Every case is written to ``focal_golden.npz`` next to this script together
with a JSON manifest of the case parameters and the numpy/scipy versions.
The GPU machine does not have the reference tree; tests there read only the
committed ``.npz``.
"""

from __future__ import annotations

import argparse
import enum
import json
import sys
import types
import warnings
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def _install_core_stubs() -> None:
    """Register minimal ``vibespatial.residency`` / ``vibespatial.runtime``."""

    residency = types.ModuleType("vibespatial.residency")

    class Residency(enum.StrEnum):
        HOST = "host"
        DEVICE = "device"

    class TransferTrigger(enum.StrEnum):
        EXPLICIT_RUNTIME_REQUEST = "explicit_runtime_request"
        USER_MATERIALIZATION = "user_materialization"

    class _Plan:
        def __init__(self, transfer_required: bool) -> None:
            self.transfer_required = transfer_required

    def select_residency_plan(*, current, target, trigger):  # noqa: ARG001
        return _Plan(current is not target)

    residency.Residency = Residency
    residency.TransferTrigger = TransferTrigger
    residency.select_residency_plan = select_residency_plan

    runtime = types.ModuleType("vibespatial.runtime")

    class RuntimeSelection:  # only referenced as a type annotation
        pass

    runtime.RuntimeSelection = RuntimeSelection

    sys.modules["vibespatial.residency"] = residency
    sys.modules["vibespatial.runtime"] = runtime


def _fbm(h: int, w: int, seed: int, lo: float, hi: float) -> np.ndarray:
    """Small smooth random surface (sum of bilinear-upsampled noise octaves)."""
    rng = np.random.default_rng(seed)
    z = np.zeros((h, w), np.float64)
    for o in range(5):
        gh, gw = 2 + 2**o, 2 + 2**o
        g = rng.random((gh, gw))
        yi = np.linspace(0, gh - 1, h)
        xi = np.linspace(0, gw - 1, w)
        y0 = np.floor(yi).astype(int).clip(0, gh - 2)
        x0 = np.floor(xi).astype(int).clip(0, gw - 2)
        fy = (yi - y0)[:, None]
        fx = (xi - x0)[None, :]
        v = (
            g[y0][:, x0] * (1 - fy) * (1 - fx)
            + g[y0 + 1][:, x0] * fy * (1 - fx)
            + g[y0][:, x0 + 1] * (1 - fy) * fx
            + g[y0 + 1][:, x0 + 1] * fy * fx
        )
        z += v * 2.0 ** (-0.8 * o)
    z = (z - z.min()) / (z.max() - z.min())
    return lo + (hi - lo) * z


def _terrain_cases() -> list[dict]:
    cases = []
    aff1 = (1.0, 0.0, 0.0, 0.0, -1.0, 0.0)
    cases.append(dict(name="flat8", data=np.full((8, 8), 500.0, np.float32), nodata=None, affine=aff1))
    cases.append(
        dict(name="ramp_east", data=np.tile(np.arange(12, dtype=np.float64), (10, 1)), nodata=None, affine=aff1)
    )
    np.random.seed(42)
    cases.append(
        dict(name="seed42_u100_1000", data=np.random.uniform(100, 1000, (10, 10)), nodata=None, affine=aff1)
    )
    d = _fbm(37, 53, 7, 0.0, 3000.0).astype(np.float32)
    rng = np.random.default_rng(11)
    idx = rng.choice(d.size, size=int(0.04 * d.size), replace=False)
    d.flat[idx] = -9999.0
    d[0, 0] = -9999.0
    d[-1, 5] = -9999.0
    d[9, -1] = -9999.0
    cases.append(dict(name="fbm_nodata_f32", data=d, nodata=-9999.0, affine=(30.0, 0.0, 5e5, 0.0, -30.0, 4.5e6)))
    d = _fbm(23, 31, 8, 100.0, 900.0).astype(np.float32)
    d[5, 7] = np.nan
    d[0, 12] = np.nan
    d[22, 30] = np.nan
    cases.append(dict(name="fbm_nan_f32", data=d, nodata=float("nan"), affine=(10.0, 0.0, 0.0, 0.0, -10.0, 0.0)))
    d = (_fbm(17, 19, 9, -200.0, 2500.0)).astype(np.int16)
    d[3, 4] = -32768
    d[16, 0] = -32768
    cases.append(dict(name="int16_nodata", data=d, nodata=-32768, affine=(25.0, 0.0, 0.0, 0.0, -25.0, 0.0)))
    cases.append(
        dict(name="row_1xN", data=_fbm(2, 29, 3, 0.0, 50.0)[:1].astype(np.float32), nodata=None, affine=aff1)
    )
    cases.append(
        dict(name="col_Nx1", data=_fbm(29, 2, 4, 0.0, 50.0)[:, :1].astype(np.float32), nodata=None, affine=aff1)
    )
    cases.append(dict(name="one_1x1", data=np.array([[7.5]], np.float32), nodata=None, affine=aff1))
    cases.append(
        dict(
            name="rotated_affine",
            data=_fbm(13, 21, 5, 0.0, 80.0).astype(np.float32),
            nodata=None,
            affine=(-2.0, 0.5, 0.0, 0.3, 3.0, 0.0),
        )
    )
    cases.append(
        dict(
            name="zero_affine",
            data=_fbm(11, 9, 6, 0.0, 20.0).astype(np.float64),
            nodata=None,
            affine=(0.0, 0.0, 0.0, 0.0, 0.0, 0.0),
        )
    )
    d = _fbm(33, 65, 12, 0.0, 4500.0).astype(np.float32)
    yy, xx = np.mgrid[0:33, 0:65]
    d[(yy - 16) ** 2 + (xx - 40) ** 2 <= 25] = -9999.0
    cases.append(dict(name="disc_hole_f32", data=d, nodata=-9999.0, affine=(10.0, 0.0, 0.0, 0.0, -10.0, 0.0)))
    d = _fbm(19, 24, 13, 0.0, 300.0).astype(np.float64)
    d[4, 4] = -9999.0
    cases.append(dict(name="nodata_f64", data=d, nodata=-9999.0, affine=(5.0, 0.0, 0.0, 0.0, -5.0, 0.0)))
    return cases


HILLSHADE_PARAMS = [
    dict(azimuth=315.0, altitude=45.0, z_factor=1.0),
    dict(azimuth=90.0, altitude=30.0, z_factor=2.0),
    dict(azimuth=200.0, altitude=90.0, z_factor=0.5),
]


def _focal_cases() -> list[dict]:
    cases = []
    cases.append(
        dict(
            name="seq_5x5",
            data=np.arange(1, 26, dtype=np.float64).reshape(5, 5),
            nodata=None,
            radius=(1, 1),
        )
    )
    rng = np.random.default_rng(21)
    d = rng.uniform(0, 100, (13, 17)).astype(np.float32)
    d[rng.random((13, 17)) < 0.1] = -9999.0
    cases.append(dict(name="rand_nodata_r12", data=d, nodata=-9999.0, radius=(1, 2)))
    cases.append(dict(name="rand_nodata_r3", data=d, nodata=-9999.0, radius=(3, 3)))
    u = np.clip(rng.gamma(2.0, 800.0, (21, 18)), 0, 10000).astype(np.uint16)
    u[rng.random((21, 18)) < 0.03] = 0
    u[0:2, 0:2] = 0
    cases.append(dict(name="u16_gamma_r3", data=u, nodata=0, radius=(3, 3)))
    d = rng.uniform(-5, 5, (9, 11)).astype(np.float32)
    d[4, 5] = np.nan
    d[0, 0] = np.nan
    cases.append(dict(name="nan_r1", data=d, nodata=float("nan"), radius=(1, 1)))
    cases.append(dict(name="nonodata_r2", data=rng.uniform(0, 1, (12, 7)).astype(np.float32), nodata=None, radius=(2, 2)))
    return cases


FOCAL_STATS = ("min", "max", "std", "range", "variety")

GAUSS_PARAMS = [(1.0, None), (1.0, 5), (0.7, None), (2.5, 8), (5.0, 41), (8.0, 65), (3.0, None)]


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="root of the reference source tree (holds src/vibespatial)")
    ap.add_argument("--out", default=str(HERE / "focal_golden.npz"))
    args = ap.parse_args()

    sys.path.insert(0, str(Path(args.reference) / "src"))
    _install_core_stubs()
    import scipy

    from vibespatial.raster import algebra as ref_alg
    from vibespatial.raster.buffers import from_numpy

    arrays: dict[str, np.ndarray] = {}
    manifest: dict = {
        "numpy": np.__version__,
        "scipy": scipy.__version__,
        "reference": "vibespatial-raster 0.1.7",
        "terrain": [],
        "hillshade_params": HILLSHADE_PARAMS,
        "focal_mean": [],
        "focal_stats": list(FOCAL_STATS),
        "gaussian": [],
    }

    for c in _terrain_cases():
        name = c["name"]
        dem = from_numpy(c["data"], nodata=c["nodata"], affine=c["affine"])
        arrays[f"terrain/{name}/input"] = c["data"]
        s = ref_alg.raster_slope(dem, use_gpu=False).to_numpy()
        a = ref_alg.raster_aspect(dem, use_gpu=False).to_numpy()
        arrays[f"terrain/{name}/slope"] = s
        arrays[f"terrain/{name}/aspect"] = a
        for k, hp in enumerate(HILLSHADE_PARAMS):
            with np.errstate(invalid="ignore"):
                hs = ref_alg.raster_hillshade(dem, use_gpu=False, **hp)
            arrays[f"terrain/{name}/hillshade{k}"] = hs.to_numpy()
            if k == 0:
                hs_nodata = hs.nodata
        deriv_nodata = None
        for key, fn in (("tri", ref_alg.raster_tri), ("tpi", ref_alg.raster_tpi),
                        ("curvature", ref_alg.raster_curvature)):
            with np.errstate(invalid="ignore"):
                dv = fn(dem, use_gpu=False)
            arrays[f"terrain/{name}/{key}"] = dv.to_numpy()
            deriv_nodata = dv.nodata
        manifest["terrain"].append(
            {
                "name": name,
                "nodata": None if c["nodata"] is None else float(c["nodata"]),
                "affine": list(c["affine"]),
                "in_dtype": str(c["data"].dtype),
                "slope_dtype": str(s.dtype),
                "hillshade_nodata": hs_nodata,
                "deriv_nodata": deriv_nodata,
            }
        )

    for c in _focal_cases():
        name = c["name"]
        r = from_numpy(c["data"], nodata=c["nodata"])
        out = ref_alg.raster_focal_mean(r, c["radius"], use_gpu=False).to_numpy()
        arrays[f"focal_mean/{name}/input"] = c["data"]
        arrays[f"focal_mean/{name}/output"] = out
        for stat in FOCAL_STATS:
            fn = getattr(ref_alg, f"raster_focal_{stat}")
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                arrays[f"focal_{stat}/{name}/output"] = fn(r, c["radius"], use_gpu=False).to_numpy()
        manifest["focal_mean"].append(
            {
                "name": name,
                "nodata": None if c["nodata"] is None else float(c["nodata"]),
                "radius": list(c["radius"]),
                "out_dtype": str(out.dtype),
            }
        )

    captured: list[np.ndarray] = []

    def _recorder(raster, kernel_weights):  # replaces the GPU launch only
        captured.append(np.array(kernel_weights, copy=True))
        return raster

    real = ref_alg._gpu_convolve
    ref_alg._gpu_convolve = _recorder
    try:
        dummy = from_numpy(np.zeros((4, 4), np.float32))
        for sigma, ks in GAUSS_PARAMS:
            captured.clear()
            ref_alg.raster_gaussian_filter(dummy, sigma, kernel_size=ks)
            w = captured[0]
            key = f"gaussian/s{sigma}_k{ks}"
            arrays[key] = w
            manifest["gaussian"].append({"key": key, "sigma": sigma, "kernel_size": ks, "shape": list(w.shape)})
        for bad_sigma in (0.0, -1.0):
            try:
                ref_alg.raster_gaussian_filter(dummy, bad_sigma)
            except ValueError as e:
                manifest.setdefault("gaussian_errors", []).append([bad_sigma, str(e)])
        try:
            ref_alg.raster_convolve(dummy, np.ones(3))
        except ValueError as e:
            manifest["convolve_1d_error"] = str(e)
        captured.clear()
        ref_alg.raster_convolve(dummy, [[1, 2], [3, 4]])
        arrays["convolve/int_list_weights"] = captured[0]
    finally:
        ref_alg._gpu_convolve = real

    np.savez_compressed(args.out, **arrays)
    Path(args.out).with_suffix(".json").write_text(json.dumps(manifest, indent=1, default=str) + "\n")
    print(f"wrote {len(arrays)} arrays to {args.out}")


if __name__ == "__main__":
    main()
