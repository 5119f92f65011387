"""GB300-native engine for FMD's per-timestep hot path.

The product is the shared library `fmd_gb300/lib/libfmd.so`: FMD's public
C API (include/fmd.h) implemented in host C over hand-written sm_103a CUDA
kernels (include/fmdg.h).  This package only builds and loads it.
"""
from __future__ import annotations

import os

from .build import LIBFMD, build  # noqa: F401

__all__ = ["build", "load", "lib_path"]


def lib_path() -> str:
    return LIBFMD


def load():
    """Load libfmd.so through the fmd.h ctypes binding.  Raises if the
    library has not been built: there is no CPU fallback."""
    from .api import Lib
    if not os.path.exists(LIBFMD):
        raise RuntimeError("libfmd.so is not built; run `python -m fmd_gb300.build` (nvcc, sm_103a)")
    return Lib(LIBFMD, prefix="fmdx_")
