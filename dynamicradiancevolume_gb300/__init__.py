"""GB300 dynamic-radiance-volume indirect lighting (a from-scratch sm_103a
implementation of Wumpf/DynamicRadianceVolume's per-frame cache pipeline).

The product is the C-ABI library `libdrv_gb300.so` (include/drv.h); this
package loads it through ctypes and offers the workload helpers the tests and
the benchmark use. There is no CPU fallback: without the built library every
entry point raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import abi

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libdrv_gb300.so"
HEADER = PKG.parent / "include" / "drv.h"

_lib: C.CDLL | None = None


class DrvError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def load(build_if_missing: bool = False) -> C.CDLL:
    """Loads and binds libdrv_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        if not build_if_missing:
            raise DrvError(abi.ERR_NOT_SUPPORTED,
                           f"{LIB_PATH.name} is not built; run `python -m dynamicradiancevolume_gb300.build`")
        from .build import build
        build()
    _lib = abi.bind(C.CDLL(str(LIB_PATH)))
    return _lib


def check(status: int, ctx=None) -> None:
    if status != abi.OK:
        lib = load()
        msg = lib.drv_last_error_string(ctx).decode() if ctx else ""
        raise DrvError(status, msg)


__all__ = ["abi", "load", "check", "DrvError", "LIB_PATH", "HEADER"]
