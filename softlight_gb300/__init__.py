"""GB300-native implementation of SoftLight's triangle draw path.

The product is the CUDA library softlight_gb300/libslg.so (C ABI in
include/slg.h); this package holds its sources (csrc/), the build step,
a ctypes binding shaped like SL_Context and the seeded procedural workloads.
"""
from .api import Context, SLContext, SLError, open_library, exported_symbols, LIB_PATH  # noqa: F401


def build(verbose=False, force=False):
    from .buildlib import build as _build
    return _build(verbose=verbose, force=force)
