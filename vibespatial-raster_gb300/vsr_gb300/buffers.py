"""OwnedRasterArray: the raster buffer type the focal operations take and return.

Keeps the contract of the reference type (src/vibespatial/raster/buffers.py:
258-700): band-first ``(B, H, W)`` or ``(H, W)`` C-contiguous pixel data, a
``nodata`` sentinel, a 6-tuple GDAL ``affine``, a ``crs``, HOST/DEVICE
residency and a diagnostics list of ``RasterDiagnosticEvent``.  The device
mirror is a ``torch.Tensor`` on the current CUDA device instead of a CuPy
array (CuPy is not a dependency); ``from_device`` accepts torch tensors and
any object exposing ``__dlpack__`` or ``__cuda_array_interface__``.
"""

from __future__ import annotations

import time
import warnings
from collections.abc import Sequence
from dataclasses import dataclass, field
from enum import StrEnum

import numpy as np

from vsr_gb300.residency import Residency, TransferTrigger


class RasterDiagnosticKind(StrEnum):
    CREATED = "created"
    TRANSFER = "transfer"
    MATERIALIZATION = "materialization"
    RUNTIME = "runtime"


@dataclass(frozen=True)
class RasterDiagnosticEvent:
    kind: RasterDiagnosticKind
    detail: str
    residency: Residency
    visible_to_user: bool = False
    elapsed_seconds: float = 0.0
    bytes_transferred: int = 0


@dataclass(frozen=True)
class RasterDeviceState:
    """Device mirror: pixel data and a lazily built boolean nodata mask."""

    data: object  # torch.Tensor on a CUDA device
    nodata_mask: object | None = None


_TORCH_TO_NP = None


def _torch():
    import torch

    return torch


def torch_dtype(np_dtype):
    torch = _torch()
    return {
        np.dtype(np.uint8): torch.uint8,
        np.dtype(np.int8): torch.int8,
        np.dtype(np.int16): torch.int16,
        np.dtype(np.uint16): torch.uint16,
        np.dtype(np.int32): torch.int32,
        np.dtype(np.uint32): torch.uint32,
        np.dtype(np.int64): torch.int64,
        np.dtype(np.float16): torch.float16,
        np.dtype(np.float32): torch.float32,
        np.dtype(np.float64): torch.float64,
        np.dtype(np.bool_): torch.bool,
    }[np.dtype(np_dtype)]


def numpy_dtype(t_dtype) -> np.dtype:
    torch = _torch()
    table = {
        torch.uint8: np.uint8,
        torch.int8: np.int8,
        torch.int16: np.int16,
        torch.uint16: np.uint16,
        torch.int32: np.int32,
        torch.uint32: np.uint32,
        torch.int64: np.int64,
        torch.float16: np.float16,
        torch.float32: np.float32,
        torch.float64: np.float64,
        torch.bool: np.bool_,
    }
    return np.dtype(table[t_dtype])


def _host_to_device(host: np.ndarray):
    torch = _torch()
    if not torch.cuda.is_available():
        raise RuntimeError("a CUDA device is required for device-resident raster operations")
    t = torch.from_numpy(np.ascontiguousarray(host))
    return t.to("cuda", non_blocking=t.is_pinned())


@dataclass
class OwnedRasterArray:
    """Owned raster buffer with HOST/DEVICE residency and diagnostics."""

    data: np.ndarray
    nodata: float | int | None
    dtype: np.dtype
    affine: tuple[float, float, float, float, float, float]
    crs: object | None = None
    residency: Residency = Residency.HOST
    diagnostics: list[RasterDiagnosticEvent] = field(default_factory=list)
    runtime_history: list = field(default_factory=list)
    device_state: RasterDeviceState | None = None
    _host_materialized: bool = True

    # -- shape ---------------------------------------------------------------
    @property
    def band_count(self) -> int:
        return self.data.shape[0] if self.data.ndim == 3 else 1

    @property
    def height(self) -> int:
        return self.data.shape[-2]

    @property
    def width(self) -> int:
        return self.data.shape[-1]

    @property
    def pixel_count(self) -> int:
        return self.height * self.width

    @property
    def shape(self) -> tuple[int, ...]:
        return self.data.shape

    # -- nodata --------------------------------------------------------------
    @property
    def nodata_mask(self) -> np.ndarray:
        """Host boolean mask, True = nodata (buffers.py:304-328 rules)."""
        self._ensure_host_state()
        if self.nodata is None:
            return np.zeros(self.data.shape, dtype=bool)
        if np.isnan(self.nodata):
            if not np.issubdtype(self.data.dtype, np.floating):
                warnings.warn(
                    f"nodata is NaN but data dtype is {self.data.dtype}; "
                    "NaN cannot exist in integer arrays so mask is all-False",
                    stacklevel=2,
                )
                return np.zeros(self.data.shape, dtype=bool)
            return np.isnan(self.data)
        return self.data == self.nodata

    @property
    def valid_mask(self) -> np.ndarray:
        return ~self.nodata_mask

    @property
    def bounds(self) -> tuple[float, float, float, float]:
        a, b, c, d, e, f = self.affine
        xs = [c, c + a * self.width, c + b * self.height, c + a * self.width + b * self.height]
        ys = [f, f + d * self.width, f + e * self.height, f + d * self.width + e * self.height]
        return (min(xs), min(ys), max(xs), max(ys))

    # -- residency -----------------------------------------------------------
    def move_to(self, target: Residency, *, trigger: TransferTrigger = TransferTrigger.EXPLICIT_RUNTIME_REQUEST,
                reason: str = "") -> None:
        if target is self.residency:
            return
        if target is Residency.DEVICE:
            self._ensure_device_state()
        else:
            self._ensure_host_state()
        self.residency = target

    def _ensure_device_state(self) -> RasterDeviceState:
        if self.device_state is not None:
            return self.device_state
        t0 = time.perf_counter()
        dev = _host_to_device(self.data)
        elapsed = time.perf_counter() - t0
        nbytes = int(self.data.nbytes)
        self.device_state = RasterDeviceState(data=dev)
        self.residency = Residency.DEVICE
        self.diagnostics.append(
            RasterDiagnosticEvent(
                kind=RasterDiagnosticKind.TRANSFER,
                detail=f"host->device {nbytes:,} bytes ({self.height}x{self.width}x{self.band_count} {self.dtype})",
                residency=Residency.DEVICE,
                visible_to_user=True,
                elapsed_seconds=elapsed,
                bytes_transferred=nbytes,
            )
        )
        return self.device_state

    def _ensure_host_state(self, out: np.ndarray | None = None) -> None:
        if self._host_materialized or self.device_state is None:
            return
        torch = _torch()
        t0 = time.perf_counter()
        src = self.device_state.data
        if out is not None:
            if out.shape != tuple(src.shape) or out.dtype != numpy_dtype(src.dtype):
                raise ValueError("out buffer shape/dtype does not match the raster")
            dst = torch.from_numpy(out)
            dst.copy_(src, non_blocking=dst.is_pinned())
            if dst.is_pinned():
                torch.cuda.current_stream().synchronize()
            self.data = out
        else:
            self.data = src.cpu().numpy()
        elapsed = time.perf_counter() - t0
        self._host_materialized = True
        self.diagnostics.append(
            RasterDiagnosticEvent(
                kind=RasterDiagnosticKind.TRANSFER,
                detail=f"device->host {self.data.nbytes:,} bytes",
                residency=Residency.HOST,
                visible_to_user=True,
                elapsed_seconds=elapsed,
                bytes_transferred=int(self.data.nbytes),
            )
        )

    def to_numpy(self, out: np.ndarray | None = None) -> np.ndarray:
        """Host array, copying from the device if needed.

        ``out`` (an extension over the reference signature) receives the copy
        when given, e.g. a page-locked buffer for a fast device->host read.
        """
        if self.residency is Residency.DEVICE:
            self._ensure_host_state(out)
        return self.data

    def device_data(self):
        """Device-resident ``torch.Tensor`` of the pixels."""
        return self._ensure_device_state().data

    def device_nodata_mask(self):
        """Device boolean mask (True = nodata), computed once and cached."""
        torch = _torch()
        state = self._ensure_device_state()
        if state.nodata_mask is not None:
            return state.nodata_mask
        d = state.data
        if self.nodata is None:
            mask = torch.zeros(d.shape, dtype=torch.bool, device=d.device)
        elif np.isnan(self.nodata):
            if not np.issubdtype(self.dtype, np.floating):
                warnings.warn(f"nodata is NaN but data dtype is {self.dtype}; mask is all-False", stacklevel=2)
                mask = torch.zeros(d.shape, dtype=torch.bool, device=d.device)
            else:
                mask = torch.isnan(d)
        else:
            mask = d == self.nodata
        self.device_state = RasterDeviceState(data=d, nodata_mask=mask)
        return mask

    def device_band(self, band_index: int):
        d = self.device_data()
        if d.ndim == 2:
            if band_index != 0:
                raise IndexError(f"single-band raster, got band_index={band_index}")
            return d
        if band_index < 0 or band_index >= d.shape[0]:
            raise IndexError(f"band_index={band_index} out of range for {d.shape[0]}-band raster")
        return d[band_index]

    @staticmethod
    def from_band_stack(band_results: Sequence[OwnedRasterArray], *, source: OwnedRasterArray) -> OwnedRasterArray:
        """Assemble per-band results into one (B, H, W) raster (buffers.py:544-659)."""
        if not band_results:
            raise ValueError("band_results must not be empty")
        if len(band_results) == 1:
            r = band_results[0]
            r.affine, r.crs, r.nodata = source.affine, source.crs, source.nodata
            return r
        ref = band_results[0]
        for i, br in enumerate(band_results[1:], start=1):
            if br.dtype != ref.dtype:
                raise ValueError(f"dtype mismatch: band 0 has {ref.dtype}, band {i} has {br.dtype}")
            if (ref.nodata is None) != (br.nodata is None):
                raise ValueError(f"nodata mismatch: band 0 has {ref.nodata}, band {i} has {br.nodata}")
            if ref.nodata is not None:
                both_nan = isinstance(ref.nodata, float) and isinstance(br.nodata, float) and np.isnan(ref.nodata) and np.isnan(br.nodata)
                if not both_nan and ref.nodata != br.nodata:
                    raise ValueError(f"nodata mismatch: band 0 has {ref.nodata}, band {i} has {br.nodata}")
            if br.height != ref.height or br.width != ref.width:
                raise ValueError(
                    f"shape mismatch: band 0 is ({ref.height}, {ref.width}), band {i} is ({br.height}, {br.width})"
                )
        merged = [e for br in band_results for e in br.diagnostics]
        if any(br.residency is Residency.DEVICE for br in band_results):
            torch = _torch()
            bands = [br.device_data().reshape(br.height, br.width) for br in band_results]
            result = from_device(torch.stack(bands, 0), nodata=source.nodata, affine=source.affine, crs=source.crs)
        else:
            bands = [br.to_numpy().reshape(br.height, br.width) for br in band_results]
            result = from_numpy(np.stack(bands, 0), nodata=source.nodata, affine=source.affine, crs=source.crs)
        result.diagnostics = merged + result.diagnostics
        return result

    def diagnostics_report(self) -> dict:
        return {
            "shape": self.shape,
            "dtype": str(self.dtype),
            "band_count": self.band_count,
            "pixel_count": self.pixel_count,
            "nodata": self.nodata,
            "residency": str(self.residency),
            "device_allocated": self.device_state is not None,
            "events": [
                {
                    "kind": str(e.kind),
                    "detail": e.detail,
                    "residency": str(e.residency),
                    "elapsed_seconds": e.elapsed_seconds,
                    "bytes_transferred": e.bytes_transferred,
                }
                for e in self.diagnostics
            ],
        }

    def __repr__(self) -> str:
        return (
            f"OwnedRasterArray(shape={self.shape}, dtype={self.dtype}, nodata={self.nodata}, "
            f"residency={self.residency}, crs={self.crs})"
        )


def from_numpy(data: np.ndarray, *, nodata=None, affine=(1.0, 0.0, 0.0, 0.0, -1.0, 0.0), crs=None,
               residency: Residency = Residency.HOST) -> OwnedRasterArray:
    """Host-resident raster from a numpy array (buffers.py:708-760)."""
    if data.ndim not in (2, 3):
        raise ValueError(f"raster data must be 2D or 3D, got {data.ndim}D")
    if nodata is not None and np.isnan(nodata) and not np.issubdtype(data.dtype, np.floating):
        raise ValueError(
            f"nodata=NaN is incompatible with integer dtype {data.dtype}; "
            "use a finite sentinel value or cast to a floating-point dtype"
        )
    arr = OwnedRasterArray(
        data=np.ascontiguousarray(data),
        nodata=nodata,
        dtype=data.dtype,
        affine=tuple(affine),
        crs=crs,
        residency=Residency.HOST,
        diagnostics=[],
    )
    if residency is Residency.DEVICE:
        arr.move_to(Residency.DEVICE)
    arr.diagnostics.append(
        RasterDiagnosticEvent(
            kind=RasterDiagnosticKind.CREATED,
            detail=f"from_numpy shape={data.shape} dtype={data.dtype}",
            residency=residency,
        )
    )
    return arr


def as_device_tensor(device_data):
    """torch.Tensor view of a device array (torch, DLPack or CUDA array interface)."""
    torch = _torch()
    if isinstance(device_data, torch.Tensor):
        t = device_data
    elif hasattr(device_data, "__dlpack__"):
        t = torch.from_dlpack(device_data)
    elif hasattr(device_data, "__cuda_array_interface__"):
        t = torch.as_tensor(device_data, device="cuda")
    else:
        raise TypeError("device_data must be a CUDA torch.Tensor or expose __dlpack__ / __cuda_array_interface__")
    if not t.is_cuda:
        raise ValueError("device_data must live on a CUDA device")
    return t


def from_device(device_data, *, nodata=None, affine=(1.0, 0.0, 0.0, 0.0, -1.0, 0.0), crs=None) -> OwnedRasterArray:
    """Device-resident raster wrapping a device array without a copy (buffers.py:763-814)."""
    t = as_device_tensor(device_data)
    if t.ndim not in (2, 3):
        raise ValueError(f"raster data must be 2D or 3D, got {t.ndim}D")
    np_dt = numpy_dtype(t.dtype)
    return OwnedRasterArray(
        data=np.empty(tuple(t.shape), dtype=np_dt),
        nodata=nodata,
        dtype=np_dt,
        affine=tuple(affine),
        crs=crs,
        residency=Residency.DEVICE,
        device_state=RasterDeviceState(data=t),
        _host_materialized=False,
        diagnostics=[
            RasterDiagnosticEvent(
                kind=RasterDiagnosticKind.CREATED,
                detail=f"from_device shape={tuple(t.shape)} dtype={np_dt}",
                residency=Residency.DEVICE,
            )
        ],
    )
