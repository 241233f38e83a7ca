"""GB300-native SunlightLB: the SunlightLB lattice Boltzmann C API on one GPU.

The product is the shared library ``lib/libsunlightlb.so`` (C API of
``include/sunlightlb.h``, CUDA kernels for sm_103a).  This package builds it
in tree and exposes it to Python with the calling conventions of the
reference's SWIG module (``from sunlightlb_gb300.SunlightLB import *``).
There is no CPU code path: device calls fail loudly without a CUDA GPU.
"""

import os

from . import build as _build
from .binding import Library

LIB_PATH = _build.LIB

_lib = None


def library(rebuild=False):
    """The loaded GB300 library (built first if needed)."""
    global _lib
    if _lib is None or rebuild:
        if rebuild or not os.path.exists(LIB_PATH):
            _build.build(force=rebuild)
        _lib = Library(LIB_PATH, extended=True)
    return _lib
