"""TEST INFRASTRUCTURE ONLY: Python driver of SwiftShader's own draw routines.

Loads ``oracle/_ref/librefjit.so`` (built by ``oracle/refjit/build_refjit.py``
from the reference sources) and runs the reference's SetupRoutine, SamplerCore
and QuadRasterizer + PixelRoutine on scene inputs, with the vertex stage and
draw constants taken from the oracle (``oracle_triangle_inputs``).  Only
``tests/golden/make_refjit_fixtures.py`` uses it: the fixtures it writes are
what the CPU tests compare the oracle with.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(os.path.dirname(HERE), "_ref", "librefjit.so")
VF = 14  # floats per vertex record (clip xyzw, projected z w, 8 varyings)
VI = 3   # ints per vertex record (X, Y, clip flags)

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise FileNotFoundError("%s is missing: run python oracle/refjit/build_refjit.py" % LIB)
        import sys
        sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
        from swiftshader_gb300 import abi
        # lazy binding: the SPIR-V emitter paths a shaderless pipeline never
        # reaches stay unresolved
        L = C.CDLL(LIB, mode=os.RTLD_LAZY)
        L.refjit_setup.argtypes = [C.POINTER(abi.PipelineState), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        L.refjit_setup.restype = C.c_int
        L.refjit_sample_quad.argtypes = [C.POINTER(abi.Texture), C.c_void_p, C.c_void_p, C.c_void_p]
        L.refjit_sample_quad.restype = C.c_int
        L.refjit_raster.argtypes = [C.POINTER(abi.PipelineState), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_int, C.c_int, C.c_void_p]
        L.refjit_raster.restype = C.c_int
        _lib = L
    return _lib


def triangle_inputs(olib, st, args, tri):
    """The oracle's vertex records and draw constants for triangle tri."""
    vf = np.zeros(3 * VF, np.float32)
    vi = np.zeros(3 * VI, np.int32)
    consts = np.zeros(6, np.float32)
    scissor = np.zeros(4, np.int32)
    nv = olib.oracle_triangle_inputs(C.byref(st), C.byref(args), tri, vf.ctypes.data, vi.ctypes.data,
                                     consts.ctypes.data, scissor.ctypes.data)
    if nv < 0:
        raise RuntimeError("oracle_triangle_inputs failed")
    return vf, vi, consts, scissor, nv


def setup(st, vf, vi, consts, scissor, nv, max_rows):
    """Reference setup of one triangle: (out_i[4], spans[4, max_rows, 2], out_f[8 + 3 nv + 1])."""
    out_i = np.zeros(4, np.int32)
    spans = np.zeros((4, max_rows, 2), np.uint16)
    out_f = np.zeros(8 + 3 * 8 + 1, np.float32)
    r = lib().refjit_setup(C.byref(st), consts.ctypes.data, scissor.ctypes.data, vf.ctypes.data, vi.ctypes.data, nv,
                           out_i.ctypes.data, spans.ctypes.data, max_rows, out_f.ctypes.data)
    if r != 0:
        raise RuntimeError("refjit_setup failed")
    return out_i, spans, out_f[:8 + 3 * nv + 1]


def sample_quad(tex, u, v):
    """Reference SamplerCore on one quad: [4 components, 4 lanes] float32."""
    u = np.ascontiguousarray(u, np.float32)
    v = np.ascontiguousarray(v, np.float32)
    out = np.zeros(16, np.float32)
    r = lib().refjit_sample_quad(C.byref(tex), u.ctypes.data, v.ctypes.data, out.ctypes.data)
    if r != 0:
        raise RuntimeError("refjit_sample_quad failed")
    return out.reshape(4, 4)


def raster(st, vf, vi, consts, scissor, ntri, nv):
    """Reference rasteriser + shaderless pixel routine over all triangles of a
    draw (the depth / stencil attachments of st are host arrays updated in
    place); returns (visible, clipped, occlusion samples)."""
    return raster_timed(st, vf, vi, consts, scissor, ntri, nv)[:3]


def raster_timed(st, vf, vi, consts, scissor, ntri, nv):
    """raster() plus the nanoseconds of its setup loop and of the pixel routine."""
    counts = np.zeros(5, np.uint64)
    r = lib().refjit_raster(C.byref(st), consts.ctypes.data, scissor.ctypes.data, vf.ctypes.data, vi.ctypes.data,
                            ntri, nv, counts.ctypes.data)
    if r != 0:
        raise RuntimeError("refjit_raster failed")
    return tuple(int(c) for c in counts)
