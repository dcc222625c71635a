"""swgb_draw_noalloc: the allocation-free draw, for callers that cannot
allocate device memory while they draw (code recording a CUDA stream capture,
hosts whose device memory belongs to another allocator, real-time loops).

It must produce exactly the bits of swgb_draw, call after call, although every
call reuses the same fixed scratch array.  This file is collected last so a
failure here never hides the other tests' results."""
import ctypes as C

import numpy as np
import pytest

from swiftshader_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def _noalloc_render(L, scene):
    import torch
    from swiftshader_gb300 import DeviceScene
    ds = DeviceScene(scene)
    torch.cuda.synchronize()
    st, a = ds.state(), ds.args()
    status = L.swgb_draw_noalloc(C.byref(st), C.byref(a), None)
    assert status == abi.OK, L.swgb_last_error()
    torch.cuda.synchronize()
    return ds.color.cpu().numpy(), ds.depth.cpu().numpy()


def _ctx_render(scene):
    from gpu_helpers import render_gpu
    c, d, _ = render_gpu(scene)
    return c, d


def test_noalloc_matches_draw_twice(gpu_lib):
    L = gpu_lib
    first = scenes.scene_heightfield(quads_x=120, quads_y=60, width=320, height=180, tex_size=256)
    second = scenes.scene_textured_small(n_tris=300, width=150, height=90)
    for sc in (first, second):
        c_ref, d_ref = _ctx_render(sc)
        c, d = _noalloc_render(L, sc)
        assert np.array_equal(c, c_ref)
        assert np.array_equal(d.view(np.uint32), d_ref.view(np.uint32))
    # and the first scene again, after the array holds the second's leftovers
    c_ref, d_ref = _ctx_render(first)
    c, d = _noalloc_render(L, first)
    assert np.array_equal(c, c_ref)
    assert np.array_equal(d.view(np.uint32), d_ref.view(np.uint32))


def test_noalloc_full_pipeline_draw(gpu_lib):
    """A draw that runs the full-pipeline raster variant through the fixed
    scratch: D16_UNORM depth with depth bias, a B8G8R8A8_UNORM attachment,
    a CLAMP_TO_BORDER texture with a custom border colour."""
    L = gpu_lib
    sc = scenes.scene_textured_small(n_tris=250, width=96, height=64, mip=True, address=abi.ADDRESS_CLAMP_TO_BORDER,
                                     blend=True, seed_index=69)
    sc.depth_format = abi.FORMAT_D16_UNORM
    sc.depth_bias = (3.0, 1.0, 0.0)
    sc.color_format = abi.FORMAT_B8G8R8A8_UNORM
    sc.sampler = dict(sc.sampler, border_color=abi.BORDER_COLOR_FLOAT_CUSTOM_EXT, custom_border_color=(0.2, 0.4, 0.6, 0.8))
    c_ref, d_ref = _ctx_render(sc)
    c, d = _noalloc_render(L, sc)
    assert np.array_equal(c, c_ref)
    assert np.array_equal(np.ascontiguousarray(d).view(np.uint8), np.ascontiguousarray(d_ref).view(np.uint8))


def test_noalloc_allocates_nothing(gpu_lib):
    """After a first call (module loading and the one-time lookups), further
    calls leave the device's free memory exactly as it was."""
    import torch
    from swiftshader_gb300 import DeviceScene
    L = gpu_lib
    sc = scenes.scene_heightfield(quads_x=120, quads_y=60, width=320, height=180, tex_size=256)
    ds = DeviceScene(sc)
    st, a = ds.state(), ds.args()
    assert L.swgb_draw_noalloc(C.byref(st), C.byref(a), None) == abi.OK, L.swgb_last_error()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        ds.clear()
        assert L.swgb_draw_noalloc(C.byref(st), C.byref(a), None) == abi.OK, L.swgb_last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_oversized_draws(gpu_lib):
    L = gpu_lib
    sc = scenes.scene_small(n_tris=8, width=32, height=32)
    st = scenes.build_state(sc, None, None, None)  # null buffers: the host rejects the state too
    a = scenes.build_args(sc)
    a.count = 32769
    assert L.swgb_draw_noalloc(C.byref(st), C.byref(a), None) == abi.INVALID_ARG
    assert b"32768" in L.swgb_last_error()
