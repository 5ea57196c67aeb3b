"""CPU oracle of the draw path: test infrastructure, not product code.

Context() returns an SLContext bound to oracle/build/libslo.so (symbol prefix
"slo_"), so a workload can be built on it with the same calls as on the GPU
library and the two results compared.
"""
from .build import build_oracle, LIB  # noqa: F401


def Context(num_threads=1):
    from softlight_gb300.api import SLContext, open_library
    lib = open_library(build_oracle(), "slo_", gpu=False)
    import ctypes as C
    fn = lib.slo_last_stats
    fn.restype = None
    fn.argtypes = [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
    ctx = SLContext(lib, "slo_", gpu=False)
    ctx.num_threads(num_threads)
    return ctx


def last_stats(ctx):
    """(triangles binned, fragments passing the depth test) of the last draw."""
    import ctypes as C
    b, f = C.c_uint64(), C.c_uint64()
    ctx._lib.slo_last_stats(ctx._h, C.byref(b), C.byref(f))
    return b.value, f.value
