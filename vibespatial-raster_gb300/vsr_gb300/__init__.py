"""vsr_gb300 -- GB300-native focal stencils behind vibespatial-raster's API.

Public names mirror ``vibespatial.raster`` for the focal path
(src/vibespatial/raster/__init__.py:143-187 resolves them lazily there).
"""

from __future__ import annotations

__version__ = "0.1.0"

from vsr_gb300._lib import load as load_library  # noqa: F401
from vsr_gb300.algebra import (  # noqa: F401
    raster_aspect,
    raster_convolve,
    raster_curvature,
    raster_focal_max,
    raster_focal_mean,
    raster_focal_min,
    raster_focal_range,
    raster_focal_std,
    raster_focal_variety,
    raster_gaussian_filter,
    raster_hillshade,
    raster_slope,
    raster_terrain,
    raster_terrain_derivatives,
    raster_tpi,
    raster_tri,
)
from vsr_gb300.buffers import (  # noqa: F401
    OwnedRasterArray,
    RasterDeviceState,
    RasterDiagnosticEvent,
    RasterDiagnosticKind,
    from_device,
    from_numpy,
)
from vsr_gb300.io import RasterMetadata, RasterWindow, read_raster, read_raster_metadata, write_raster  # noqa: F401
from vsr_gb300.residency import Residency, TransferTrigger  # noqa: F401

__all__ = [
    "OwnedRasterArray",
    "RasterMetadata",
    "RasterWindow",
    "RasterDeviceState",
    "RasterDiagnosticEvent",
    "RasterDiagnosticKind",
    "Residency",
    "TransferTrigger",
    "from_device",
    "from_numpy",
    "load_library",
    "raster_aspect",
    "raster_convolve",
    "raster_curvature",
    "raster_focal_max",
    "raster_focal_mean",
    "raster_focal_min",
    "raster_focal_range",
    "raster_focal_std",
    "raster_focal_variety",
    "raster_gaussian_filter",
    "raster_hillshade",
    "raster_slope",
    "raster_terrain",
    "raster_terrain_derivatives",
    "raster_tpi",
    "raster_tri",
    "read_raster",
    "read_raster_metadata",
    "write_raster",
]
