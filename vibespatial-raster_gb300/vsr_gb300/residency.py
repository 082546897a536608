"""Residency vocabulary of the raster buffers.

Mirrors the names the reference's ``OwnedRasterArray`` uses from its core
runtime (``vibespatial.residency``: ``Residency.HOST/DEVICE``,
``TransferTrigger``), so that code written against the reference reads the
same here.
"""

from __future__ import annotations

from enum import StrEnum


class Residency(StrEnum):
    HOST = "host"
    DEVICE = "device"


class TransferTrigger(StrEnum):
    EXPLICIT_RUNTIME_REQUEST = "explicit_runtime_request"
    USER_MATERIALIZATION = "user_materialization"
