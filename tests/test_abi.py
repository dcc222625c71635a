"""The C-ABI on the CPU: struct layouts of the ctypes mirror against the
header (compiled with gcc), the exported symbols of libswgb.so, and host-side
error handling that needs no device."""
import ctypes as C

import numpy as np
import os
import subprocess
import sys

import pytest

from swiftshader_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "swgb.h")

STRUCTS = {
    "swgb_vertex_attrib": abi.VertexAttrib,
    "swgb_vertex_binding": abi.VertexBinding,
    "swgb_texture_level": abi.TextureLevel,
    "swgb_texture": abi.Texture,
    "swgb_pipeline_state": abi.PipelineState,
    "swgb_draw_args": abi.DrawArgs,
    "swgb_counters": abi.Counters,
    "swgb_adjoint_args": abi.AdjointArgs,
    "swgb_raster_config": abi.RasterConfig,
    "swgb_stencil_op_state": abi.StencilOpState,
    "swgb_image": abi.Image,
    "swgb_rect": abi.Rect,
    "swgb_resolve_region": abi.ResolveRegion,
    "swgb_blit_region": abi.BlitRegion,
}


def header_layout(tmp_path):
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "%s"' % HEADER, "int main(void) {"]
    for cname, py in STRUCTS.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-std=c11", "-Wall", "-Werror", "-o", str(exe), str(src)])
    out = subprocess.check_output([str(exe)], text=True)
    return dict((k, int(v)) for k, v in (ln.split() for ln in out.splitlines()))


def test_ctypes_mirror_matches_header(tmp_path):
    lay = header_layout(tmp_path)
    for cname, py in STRUCTS.items():
        assert lay[cname] == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert lay["%s.%s" % (cname, f)] == getattr(py, f).offset, (cname, f)


def test_header_declares_every_export():
    text = open(HEADER).read()
    from swiftshader_gb300 import _lib
    for name in _lib.EXPORTS:
        assert name + "(" in text, name


@pytest.fixture(scope="module")
def built_lib():
    from swiftshader_gb300 import build
    path = build.build()
    return path


def test_library_loads_and_exports_all_symbols(built_lib):
    """Loading needs no GPU; every symbol the header declares is exported."""
    out = subprocess.check_output(["nm", "-D", "--defined-only", built_lib], text=True)
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    from swiftshader_gb300 import _lib
    for name in _lib.EXPORTS:
        assert name in exported, name
    L = _lib.load(built_lib)
    assert L.swgb_abi_version() == 7


def test_host_side_errors_without_device(built_lib):
    """Argument validation happens on the host and returns a status (never
    aborts); context creation without a GPU reports NO_DEVICE."""
    import torch
    from swiftshader_gb300 import _lib, scenes
    L = _lib.load(built_lib)
    ctx = C.c_void_p()
    status = L.swgb_ctx_create(0, None, C.byref(ctx))
    if torch.cuda.is_available():
        assert status == abi.OK
        L.swgb_ctx_destroy(ctx)
    else:
        assert status == abi.NO_DEVICE
    assert L.swgb_draw(None, None, None) == abi.INVALID_ARG
    assert L.swgb_sync(None) == abi.INVALID_ARG
    # the allocation-free draw validates sizes before touching any device;
    # every buffer pointer is null, which the host's state validation rejects
    # as well, so no kernel can launch on these states
    sc = scenes.scene_small(n_tris=4, width=16, height=16)
    st = scenes.build_state(sc, None, None, None)
    a = scenes.build_args(sc)
    a.count = 40000
    assert L.swgb_draw_noalloc(C.byref(st), C.byref(a), None) == abi.INVALID_ARG
    assert b"32768" in L.swgb_last_error()
    # primitive restart runs only through swgb_draw: the batched and
    # allocation-free paths refuse it on the host
    rs = scenes.restart_scene(abi.TOPOLOGY_TRIANGLE_STRIP, n_indices=64)
    rst = scenes.build_state(rs, None, None, None)
    ra = scenes.build_args(rs, None)
    assert L.swgb_draw_noalloc(C.byref(rst), C.byref(ra), None) == abi.UNSUPPORTED_STATE
    # swgb_plan_batch never launches anything (it only compares the byte
    # ranges draws touch), so it gets real host buffers of the right sizes
    cbuf, dbuf = scenes.clear_buffers(rs)
    vbuf = np.ascontiguousarray(rs.vertices, np.float32)
    ibuf = np.ascontiguousarray(rs.indices)
    pst = scenes.build_state(rs, cbuf.ctypes.data, dbuf.ctypes.data, vbuf.ctypes.data)
    pa = scenes.build_args(rs, ibuf.ctypes.data)
    segs = C.c_uint32()
    assert L.swgb_plan_batch(C.byref(pst), C.byref(pa), 1, None, C.byref(segs)) == abi.UNSUPPORTED_STATE
    # an out-of-range provoking-vertex mode fails the state validation every
    # entry point shares (checked through the host-only planner)
    pa.restart_index_count = 0
    pa.count = 4
    pst.provoking_vertex = 2
    assert L.swgb_plan_batch(C.byref(pst), C.byref(pa), 1, None, C.byref(segs)) == abi.INVALID_ARG
    assert b"provoking" in L.swgb_last_error()
    # raster configuration: validated on the host
    assert L.swgb_ctx_set_raster_config(None, None) == abi.INVALID_ARG
    assert L.swgb_autotune(None, None, None, 0, 1, 0, None, None, None, None, None) == abi.INVALID_ARG
    # Blitter entry points: null context / arguments rejected on the host
    img = abi.Image(None, abi.FORMAT_R8G8B8A8_UNORM, 4, 4, 1, 16, 64)
    assert L.swgb_clear(None, None, 0, C.byref(img), None) == abi.INVALID_ARG
    assert L.swgb_resolve(None, C.byref(img), C.byref(img), None) == abi.INVALID_ARG
    assert L.swgb_blit(None, C.byref(img), C.byref(img), None, 0) == abi.INVALID_ARG


def test_header_lists_the_bin_shapes():
    """The shapes the header documents are the ones the Python mirror offers."""
    text = open(HEADER).read()
    for w, h in abi.BIN_SHAPES:
        assert "%dx%d" % (w, h) in text
    assert "#define SWGB_AUTOTUNE_CANDIDATES %d" % abi.AUTOTUNE_CANDIDATES in text
    assert "#define SWGB_AUTOTUNE_DEFAULT_RUNS %d" % abi.AUTOTUNE_DEFAULT_RUNS in text
    assert "#define SWGB_AUTOTUNE_MAX_RUNS %d" % abi.AUTOTUNE_MAX_RUNS in text
    assert abi.AUTOTUNE_CANDIDATES == 2 * len(abi.BIN_SHAPES)
