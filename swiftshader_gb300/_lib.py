"""ctypes binding of libswgb.so (the C-ABI of include/swgb.h).

There is no fallback: if the library is missing or fails to load, every entry
point raises.  The library is built in-tree by ``swiftshader_gb300.build``.
"""
import ctypes as C
import os

from . import abi
from .build import LIB

_lib = None

EXPORTS = ["swgb_abi_version", "swgb_last_error", "swgb_ctx_create", "swgb_ctx_destroy",
           "swgb_ctx_set_stream", "swgb_draw", "swgb_draw_batch", "swgb_sync", "swgb_get_counters",
           "swgb_reset_counters", "swgb_launch_count", "swgb_set_kernel_timing", "swgb_get_kernel_times",
           "swgb_draw_noalloc", "swgb_draw_adjoint", "swgb_draw_adjoint_batch", "swgb_plan_batch",
           "swgb_ctx_set_raster_config", "swgb_ctx_get_raster_config", "swgb_autotune", "swgb_clear",
           "swgb_resolve", "swgb_blit"]


class SwgbError(RuntimeError):
    def __init__(self, status, where, msg=""):
        self.status = status
        super().__init__("%s failed: %s%s" % (where, abi.STATUS_NAMES.get(status, status), (" (%s)" % msg) if msg else ""))


def load(path=None):
    """Loads the native library (raises OSError when it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB
    if not os.path.exists(p):
        raise OSError("libswgb.so not built (%s); run swiftshader_gb300.build.build()" % p)
    L = C.CDLL(p)
    L.swgb_abi_version.restype = C.c_int
    L.swgb_last_error.restype = C.c_char_p
    L.swgb_ctx_create.argtypes = [C.c_int, C.c_void_p, C.POINTER(C.c_void_p)]
    L.swgb_ctx_create.restype = C.c_int
    L.swgb_ctx_destroy.argtypes = [C.c_void_p]
    L.swgb_ctx_destroy.restype = C.c_int
    L.swgb_ctx_set_stream.argtypes = [C.c_void_p, C.c_void_p]
    L.swgb_ctx_set_stream.restype = C.c_int
    L.swgb_draw.argtypes = [C.c_void_p, C.POINTER(abi.PipelineState), C.POINTER(abi.DrawArgs)]
    L.swgb_draw.restype = C.c_int
    L.swgb_draw_batch.argtypes = [C.c_void_p, C.POINTER(abi.PipelineState), C.POINTER(abi.DrawArgs), C.c_uint32]
    L.swgb_draw_batch.restype = C.c_int
    L.swgb_sync.argtypes = [C.c_void_p]
    L.swgb_sync.restype = C.c_int
    L.swgb_get_counters.argtypes = [C.c_void_p, C.POINTER(abi.Counters)]
    L.swgb_get_counters.restype = C.c_int
    L.swgb_reset_counters.argtypes = [C.c_void_p]
    L.swgb_reset_counters.restype = C.c_int
    L.swgb_launch_count.argtypes = [C.c_void_p]
    L.swgb_launch_count.restype = C.c_uint64
    L.swgb_set_kernel_timing.argtypes = [C.c_void_p, C.c_int]
    L.swgb_set_kernel_timing.restype = C.c_int
    L.swgb_get_kernel_times.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_uint32)]
    L.swgb_get_kernel_times.restype = C.c_int
    L.swgb_draw_noalloc.argtypes = [C.POINTER(abi.PipelineState), C.POINTER(abi.DrawArgs), C.c_void_p]
    L.swgb_draw_noalloc.restype = C.c_int
    L.swgb_draw_adjoint.argtypes = [C.c_void_p, C.POINTER(abi.PipelineState), C.POINTER(abi.DrawArgs),
                                    C.POINTER(abi.AdjointArgs)]
    L.swgb_draw_adjoint.restype = C.c_int
    L.swgb_draw_adjoint_batch.argtypes = [C.c_void_p, C.POINTER(abi.PipelineState), C.POINTER(abi.DrawArgs),
                                          C.POINTER(abi.AdjointArgs), C.c_uint32]
    L.swgb_draw_adjoint_batch.restype = C.c_int
    L.swgb_plan_batch.argtypes = [C.POINTER(abi.PipelineState), C.POINTER(abi.DrawArgs), C.c_uint32,
                                  C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
    L.swgb_plan_batch.restype = C.c_int
    L.swgb_ctx_set_raster_config.argtypes = [C.c_void_p, C.POINTER(abi.RasterConfig)]
    L.swgb_ctx_set_raster_config.restype = C.c_int
    L.swgb_ctx_get_raster_config.argtypes = [C.c_void_p, C.POINTER(abi.RasterConfig)]
    L.swgb_ctx_get_raster_config.restype = C.c_int
    L.swgb_autotune.argtypes = [C.c_void_p, C.POINTER(abi.PipelineState), C.POINTER(abi.DrawArgs), C.c_uint32, C.c_int,
                                C.c_uint32, C.POINTER(abi.RasterConfig), C.POINTER(abi.RasterConfig),
                                C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.swgb_autotune.restype = C.c_int
    L.swgb_clear.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(abi.Image), C.POINTER(abi.Rect)]
    L.swgb_clear.restype = C.c_int
    L.swgb_resolve.argtypes = [C.c_void_p, C.POINTER(abi.Image), C.POINTER(abi.Image), C.POINTER(abi.ResolveRegion)]
    L.swgb_resolve.restype = C.c_int
    L.swgb_blit.argtypes = [C.c_void_p, C.POINTER(abi.Image), C.POINTER(abi.Image), C.POINTER(abi.BlitRegion), C.c_uint32]
    L.swgb_blit.restype = C.c_int
    if L.swgb_abi_version() != 7:
        raise OSError("libswgb ABI version mismatch")
    _lib = L
    return L


def check(status, where):
    if status != abi.OK:
        msg = load().swgb_last_error()
        raise SwgbError(status, where, msg.decode() if msg else "")
