"""TEST INFRASTRUCTURE ONLY: Python loader for the CPU oracle.

Only tests/, __graft_entry__.smoke() and bench.py (cpu_baseline leg and
--impl reference) import this module.  The swiftshader_gb300 package never
does.  ``build()`` compiles swgb_oracle.c with gcc; ``render()`` runs one draw
of a scene on host buffers and returns the attachments and counters.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libswgb_oracle.so")
# the timing build: FPU flush-to-zero mode instead of the software flush, -O3;
# used only to time the CPU baseline, after its frame is compared with LIB's
LIB_TIMING = os.path.join(BUILD, "libswgb_oracle_timing.so")
SRC = os.path.join(HERE, "swgb_oracle.c")
SRC_BLIT = os.path.join(HERE, "swgb_oracle_blit.c")
CFLAGS = ["-O2", "-fPIC", "-shared", "-std=c11", "-fwrapv", "-ffp-contract=off", "-fno-fast-math",
          "-Wall", "-Wextra"]

_lib = None
_lib_timing = None


def build(force=False, timing=False):
    os.makedirs(BUILD, exist_ok=True)
    out = LIB_TIMING if timing else LIB
    if not force and os.path.exists(out) and os.path.getmtime(out) >= max(
            os.path.getmtime(SRC), os.path.getmtime(SRC_BLIT), os.path.getmtime(os.path.join(HERE, "swgb_oracle.h")),
            os.path.getmtime(os.path.join(os.path.dirname(HERE), "include", "swgb.h"))):
        return out
    tmp = out + ".tmp%d" % os.getpid()
    flags = [f if f != "-O2" else "-O3" for f in CFLAGS] + ["-DSWGB_ORACLE_HW_FLUSH"] if timing else CFLAGS
    subprocess.check_call(["gcc"] + flags + ["-o", tmp, SRC, SRC_BLIT, "-lm", "-lpthread"])
    os.replace(tmp, out)
    return out


def lib(timing=False):
    """The checker build, or with timing=True the timing build."""
    global _lib, _lib_timing
    if timing:
        if _lib_timing is None:
            from swiftshader_gb300 import abi
            L = C.CDLL(build(timing=True))
            L.oracle_draw.argtypes = [C.POINTER(abi.PipelineState), C.POINTER(abi.DrawArgs), C.c_int,
                                      C.POINTER(abi.Counters)]
            L.oracle_draw.restype = C.c_int
            L.oracle_timing_build.restype = C.c_int
            _lib_timing = L
        return _lib_timing
    if _lib is None:
        import sys
        sys.path.insert(0, os.path.dirname(HERE))
        from swiftshader_gb300 import abi
        build()
        L = C.CDLL(LIB)
        L.oracle_draw.argtypes = [C.POINTER(abi.PipelineState), C.POINTER(abi.DrawArgs), C.c_int,
                                  C.POINTER(abi.Counters)]
        L.oracle_draw.restype = C.c_int
        L.oracle_draw_visibility.argtypes = [C.POINTER(abi.PipelineState), C.POINTER(abi.DrawArgs), C.c_int,
                                             C.POINTER(abi.Counters), C.c_void_p, C.c_void_p, C.c_int]
        L.oracle_draw_visibility.restype = C.c_int
        L.oracle_round_int.argtypes = [C.c_float]
        L.oracle_round_int.restype = C.c_int32
        L.oracle_round_int_clamped.argtypes = [C.c_float]
        L.oracle_round_int_clamped.restype = C.c_int32
        L.oracle_trunc_int.argtypes = [C.c_float]
        L.oracle_trunc_int.restype = C.c_int32
        L.oracle_mulhigh_u16.argtypes = [C.c_uint16, C.c_uint16]
        L.oracle_mulhigh_u16.restype = C.c_uint16
        L.oracle_mulhigh_s16.argtypes = [C.c_int16, C.c_int16]
        L.oracle_mulhigh_s16.restype = C.c_int16
        L.oracle_fmuladd.argtypes = [C.c_float, C.c_float, C.c_float]
        L.oracle_fmuladd.restype = C.c_float
        L.oracle_log2sqrt.argtypes = [C.c_float]
        L.oracle_log2sqrt.restype = C.c_float
        L.oracle_ftz.argtypes = [C.c_float]
        L.oracle_ftz.restype = C.c_float
        for f in (L.oracle_linear_to_srgb, L.oracle_srgb_to_linear):
            f.argtypes = [C.c_float]
            f.restype = C.c_float
        L.oracle_transcendental_n.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_size_t]
        L.oracle_transcendental_n.restype = None
        L.oracle_clear.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(abi.Image), C.POINTER(abi.Rect)]
        L.oracle_clear.restype = C.c_int
        L.oracle_resolve.argtypes = [C.POINTER(abi.Image), C.POINTER(abi.Image), C.POINTER(abi.ResolveRegion)]
        L.oracle_resolve.restype = C.c_int
        L.oracle_blit.argtypes = [C.POINTER(abi.Image), C.POINTER(abi.Image), C.POINTER(abi.BlitRegion), C.c_uint32]
        L.oracle_blit.restype = C.c_int
        L.oracle_vertex.argtypes = [C.POINTER(abi.PipelineState), C.POINTER(abi.DrawArgs), C.c_uint32,
                                    C.POINTER(C.c_float), C.POINTER(C.c_int32)]
        L.oracle_vertex.restype = C.c_int
        L.oracle_triangle_inputs.argtypes = [C.POINTER(abi.PipelineState), C.POINTER(abi.DrawArgs), C.c_uint32,
                                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_triangle_inputs.restype = C.c_int
        L.oracle_setup_samples.argtypes = [C.POINTER(abi.PipelineState), C.POINTER(abi.DrawArgs), C.c_uint32,
                                           C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        L.oracle_setup_samples.restype = C.c_int
        L.oracle_set_interpolation_muladd.argtypes = [C.c_int]
        L.oracle_set_interpolation_muladd.restype = None
        L.oracle_setup.argtypes = [C.POINTER(abi.PipelineState), C.POINTER(abi.DrawArgs), C.c_uint32,
                                   C.POINTER(C.c_int32), C.POINTER(C.c_uint16), C.c_int, C.POINTER(C.c_float)]
        L.oracle_setup.restype = C.c_int
        L.oracle_sample_quad.argtypes = [C.POINTER(abi.Texture), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                         C.POINTER(C.c_float)]
        L.oracle_sample_quad.restype = C.c_int
        _lib = L
    return _lib


TRANSCENDENTAL = {"log2_mediump": 0, "exp2_mediump": 1, "linear_to_srgb": 2, "srgb_to_linear": 3}


def transcendental(name, x):
    """Element-wise Log2 / Exp2 (mediump) or the sRGB transfer functions of the
    oracle over a float32 array."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.empty_like(x)
    lib().oracle_transcendental_n(TRANSCENDENTAL[name], x.ctypes.data, out.ctypes.data, x.size)
    return out


def image(arr, format, samples=1):
    """abi.Image over a C-contiguous numpy array [H, W, ...] or
    [samples, H, W, ...] (host memory, for the oracle's Blitter)."""
    from swiftshader_gb300 import abi
    assert arr.flags["C_CONTIGUOUS"]
    h, w = (arr.shape[1], arr.shape[2]) if samples > 1 else (arr.shape[0], arr.shape[1])
    bpp = abi.TEXEL_BYTES[format]
    return abi.Image(arr.ctypes.data, format, w, h, samples, w * bpp, w * bpp * h)


def clear(arr, format, value, samples=1, area=None):
    """Blitter::clear of a host image in place (value as Renderer.clear_area takes it)."""
    from swiftshader_gb300 import abi
    img = image(arr, format, samples)
    if format == abi.FORMAT_S8_UINT:
        v, vf = (C.c_uint32 * 4)(int(value), 0, 0, 0), abi.FORMAT_S8_UINT
    elif format in (abi.FORMAT_D32_SFLOAT, abi.FORMAT_D16_UNORM):
        v, vf = (C.c_float * 4)(float(value), 0, 0, 0), abi.FORMAT_D32_SFLOAT
    else:
        v, vf = (C.c_float * 4)(*[float(x) for x in value]), abi.FORMAT_R32G32B32A32_SFLOAT
    r = C.byref(abi.Rect(*area)) if area is not None else None
    st = lib().oracle_clear(v, vf, C.byref(img), r)
    assert st == 0, st


def resolve(src, dst, format, region=None):
    """Blitter::resolve of a host [4, H, W, C] image into [H', W', C]."""
    from swiftshader_gb300 import abi
    r = C.byref(abi.ResolveRegion(*region)) if region is not None else None
    st = lib().oracle_resolve(C.byref(image(src, format, 4)), C.byref(image(dst, format)), r)
    assert st == 0, st


def blit(src, src_format, dst, dst_format, src_box, dst_box, filter):
    """Blitter::blit between host images."""
    from swiftshader_gb300 import abi
    reg = abi.BlitRegion((C.c_int32 * 4)(*src_box), (C.c_int32 * 4)(*dst_box))
    st = lib().oracle_blit(C.byref(image(src, src_format)), C.byref(image(dst, dst_format)), C.byref(reg), int(filter))
    assert st == 0, st


def _ptr(a):
    return a.ctypes.data if a is not None else None


def host_state(scene, color, depth, stencil=None):
    """PipelineState + DrawArgs whose pointers address host numpy arrays."""
    from swiftshader_gb300 import scenes
    verts = np.ascontiguousarray(scene.vertices, np.float32)
    levels = [np.ascontiguousarray(l) for l in scene.texture_levels]
    st = scenes.build_state(scene, _ptr(color), _ptr(depth), _ptr(verts), [_ptr(l) for l in levels],
                            stencil_ptr=None if stencil is None else _ptr(stencil))
    idx = None if scene.indices is None else np.ascontiguousarray(scene.indices)
    args = scenes.build_args(scene, _ptr(idx))
    keep = (verts, levels, idx)
    return st, args, keep


def render(scene, nthreads=1, color=None, depth=None, stencil=None, timing=False):
    """Runs one draw of 'scene' on the CPU oracle; returns (color, depth, counters dict).
    A scene with a stencil state draws into 'stencil' (a fresh cleared one when
    None; render_stencil returns it).  timing=True runs the timing build."""
    from swiftshader_gb300 import abi, scenes
    if color is None or depth is None:
        color, depth = scenes.clear_buffers(scene)
    if stencil is None:
        stencil = scenes.stencil_buffer(scene)
    st, args, keep = host_state(scene, color, depth, stencil)
    cnt = abi.Counters()
    s = lib(timing).oracle_draw(C.byref(st), C.byref(args), nthreads, C.byref(cnt))
    if s != 0:
        raise RuntimeError("oracle_draw failed: %s" % abi.STATUS_NAMES.get(s, s))
    del keep
    return color, depth, cnt.as_dict()


def render_stencil(scene, nthreads=1):
    """render() of a scene with a stencil state; returns (color, depth, stencil, counters)."""
    from swiftshader_gb300 import scenes
    stencil = scenes.stencil_buffer(scene)
    color, depth, cnt = render(scene, nthreads, stencil=stencil)
    return color, depth, stencil, cnt


def render_visibility(scene, nthreads=1, cap=8):
    """render() that also returns the fixed visibility: vis [S, H, W, cap]
    primitive ids passing the depth test per sample in primitive order, and
    vis_len [S, H, W] (counts every entry, even past cap)."""
    from swiftshader_gb300 import abi, scenes
    color, depth = scenes.clear_buffers(scene)
    st, args, keep = host_state(scene, color, depth)
    S = scene.samples
    vis = np.zeros((S, scene.height, scene.width, cap), np.uint32)
    vis_len = np.zeros((S, scene.height, scene.width), np.uint32)
    cnt = abi.Counters()
    s = lib().oracle_draw_visibility(C.byref(st), C.byref(args), nthreads, C.byref(cnt), vis.ctypes.data,
                                     vis_len.ctypes.data, cap)
    if s != 0:
        raise RuntimeError("oracle_draw_visibility failed: %s" % abi.STATUS_NAMES.get(s, s))
    del keep
    return color, depth, cnt.as_dict(), vis, vis_len
