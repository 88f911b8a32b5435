"""GB300 SOAPsnp/GSNP consensus caller.

The calling path runs in libgsnp_gb300.so (hand-written sm_103a kernels behind
the C ABI of include/gsnp_gb300.h).  This package is a thin ctypes binding over
that library plus helpers that turn SOAPsnp command-line flags and in-memory
alignments into its arguments.  There is no Python or CPU fallback for the
calling work: importing `native()` raises when the library is not built.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libgsnp_gb300.so")

_lib = None


def native() -> ctypes.CDLL:
    """Load libgsnp_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                "libgsnp_gb300.so is not built (run __graft_entry__.build() or python gsnp_gb300/build.py)")
        lib = ctypes.CDLL(LIB_PATH)
        from . import api
        api.declare(lib)
        _lib = lib
    return _lib


__all__ = ["native", "LIB_PATH"]
