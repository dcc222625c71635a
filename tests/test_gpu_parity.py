"""GPU parity: the C-ABI draw path on the device against the CPU oracle, on the
same seeded inputs.  Coverage, depth and RGBA8 colour are compared bit for bit,
and the device counters (triangles in / rejected / clipped / visible, quads,
fragments tested / passed) must equal the oracle's."""
import numpy as np
import pytest

from swiftshader_gb300 import abi, scenes

from gpu_helpers import assert_bit_exact, render_gpu, render_oracle

pytestmark = pytest.mark.gpu


def check_scene(scene, gpu_lib):
    c_gpu, d_gpu, cnt_gpu = render_gpu(scene)
    c_ref, d_ref, cnt_ref = render_oracle(scene)
    assert_bit_exact(d_gpu, d_ref, "depth")
    assert_bit_exact(c_gpu, c_ref, "color")
    assert_counters(cnt_gpu, cnt_ref)
    return cnt_ref


def assert_counters(gpu, ref):
    """Every counter equal, except the mip-level mask: the oracle records the
    levels the reference filters for all four lanes of every shaded quad, the
    device only those of lanes it actually writes, a subset."""
    g = dict(gpu)
    r = dict(ref)
    gm, rm = g.pop("texture_levels_mask"), r.pop("texture_levels_mask")
    assert g == r
    assert gm & ~rm == 0


def test_small_untextured_full_size(gpu_lib):
    """1000 Gouraud triangles at 256x256, RGBA8 + D32F, depth LESS."""
    cnt = check_scene(scenes.scene_small(), gpu_lib)
    assert cnt["triangles_visible"] > 900 and cnt["fragments_passed"] > 0


@pytest.mark.parametrize("n,w,h,seed", [(1, 64, 64, 11), (7, 50, 33, 12), (300, 256, 200, 13), (2000, 96, 96, 14)])
def test_small_untextured_shapes(gpu_lib, n, w, h, seed):
    """Ragged framebuffer sizes (not multiples of the 32-pixel bin) and dense overlap."""
    check_scene(scenes.scene_small(n_tris=n, width=w, height=h, seed_index=seed), gpu_lib)


@pytest.mark.parametrize("mip,address,blend", [
    (True, abi.ADDRESS_REPEAT, True),
    (True, abi.ADDRESS_CLAMP_TO_EDGE, True),
    (False, abi.ADDRESS_REPEAT, False),
    (True, abi.ADDRESS_MIRRORED_REPEAT, False),
    (False, abi.ADDRESS_CLAMP_TO_EDGE, True),
    (True, abi.ADDRESS_MIRROR_CLAMP_TO_EDGE, True),
    (False, abi.ADDRESS_MIRROR_CLAMP_TO_EDGE, False),
])
def test_textured_small(gpu_lib, mip, address, blend):
    """16-bit UNORM8 filtering: trilinear / bilinear, REPEAT / CLAMP / MIRROR /
    MIRROR_CLAMP_TO_EDGE, blend on / off."""
    s = scenes.scene_textured_small(mip=mip, address=address, blend=blend)
    check_scene(s, gpu_lib)


def test_heightfield_reduced(gpu_lib):
    """The 1M-triangle textured height field at reduced size (same generator,
    perspective, clipping at the screen edges, trilinear, alpha blend)."""
    s = scenes.scene_heightfield(quads_x=160, quads_y=80, width=320, height=180, tex_size=256)
    cnt = check_scene(s, gpu_lib)
    assert cnt["triangles_clipped"] > 0


def test_culling_and_winding(gpu_lib):
    for cull in (abi.CULL_BACK, abi.CULL_FRONT, abi.CULL_FRONT_AND_BACK):
        for ff in (abi.FRONT_FACE_CCW, abi.FRONT_FACE_CW):
            s = scenes.scene_small(n_tris=200, width=96, height=80, seed_index=21)
            s.cull_mode, s.front_face = cull, ff
            check_scene(s, gpu_lib)


def test_clipping_near_far_and_sides(gpu_lib):
    """Triangles crossing every frustum plane, some behind the eye (w < 0)."""
    s = scenes.scene_small(n_tris=400, width=128, height=128, seed_index=22)
    rng = np.random.Generator(np.random.PCG64(99))
    v = s.vertices
    v[:, 0:2] = rng.uniform(-3.0, 3.0, (v.shape[0], 2))
    v[:, 2] = rng.uniform(-1.0, 2.0, v.shape[0])
    v[:, 3] = rng.uniform(-0.5, 2.0, v.shape[0])
    cnt = check_scene(s, gpu_lib)
    assert cnt["triangles_clipped"] > 100


def test_scissor_and_viewport_offset(gpu_lib):
    s = scenes.scene_small(n_tris=300, width=160, height=120, seed_index=23)
    s.viewport = (10, -5, 130, 110)
    s.scissor = (7, 9, 101, 77)
    check_scene(s, gpu_lib)


def test_blend_ops(gpu_lib):
    for bl in [(abi.BLEND_ONE, abi.BLEND_ONE, abi.BLEND_OP_ADD, abi.BLEND_ONE, abi.BLEND_ZERO, abi.BLEND_OP_ADD),
               (abi.BLEND_SRC_COLOR, abi.BLEND_DST_COLOR, abi.BLEND_OP_SUBTRACT, abi.BLEND_ONE, abi.BLEND_ONE, abi.BLEND_OP_MAX),
               (abi.BLEND_ONE_MINUS_DST_ALPHA, abi.BLEND_SRC_ALPHA, abi.BLEND_OP_REVERSE_SUBTRACT,
                abi.BLEND_DST_ALPHA, abi.BLEND_ONE_MINUS_SRC_COLOR, abi.BLEND_OP_MIN)]:
        s = scenes.scene_small(n_tris=150, width=64, height=64, seed_index=24)
        s.blend = bl
        s.clear_color = (40, 80, 120, 160)
        check_scene(s, gpu_lib)


def test_depth_compare_ops(gpu_lib):
    for op in range(8):
        s = scenes.scene_small(n_tris=120, width=64, height=48, seed_index=25)
        s.depth_compare = op
        s.clear_depth = 0.5
        check_scene(s, gpu_lib)


def test_degenerate_and_empty(gpu_lib):
    """Zero-area, sub-pixel and collinear triangles, plus non-finite positions."""
    s = scenes.scene_small(n_tris=64, width=64, height=64, seed_index=26)
    v = s.vertices
    v[3:6, 0:2] = v[3, 0:2]                      # all three vertices equal
    v[6:9, 0] = np.array([0.1, 0.2, 0.3]); v[6:9, 1] = np.array([0.1, 0.2, 0.3])  # collinear
    v[9:12, 0:2] = v[9, 0:2] + np.array([[0, 0], [1e-4, 0], [0, 1e-4]], np.float32)  # sub-pixel
    v[12, 0] = np.inf                             # non-finite -> trivially rejected
    v[15, 1] = np.nan
    check_scene(s, gpu_lib)


def test_heightfield_full_size_bit_exact(gpu_lib):
    """The full 1M-triangle 1080p textured frame, bit for bit against the oracle."""
    cnt = check_scene(scenes.scene_heightfield(), gpu_lib)
    assert cnt["triangles_in"] == 1_000_000 and cnt["triangles_clipped"] > 0


def test_heightfield_full_size_properties(gpu_lib):
    """Full 1M-triangle 1080p frame: deterministic run to run (bit-identical),
    and counters consistent with the frame."""
    s = scenes.scene_heightfield()
    c1, d1, cnt1 = render_gpu(s)
    c2, d2, cnt2 = render_gpu(s)
    assert_bit_exact(c1, c2, "color run-to-run")
    assert_bit_exact(d1, d2, "depth run-to-run")
    assert cnt1 == cnt2
    assert cnt1["triangles_in"] == 1_000_000
    assert cnt1["triangles_visible"] + cnt1["triangles_rejected"] == cnt1["triangles_in"]
    assert cnt1["fragments_passed"] <= cnt1["fragments_tested"] <= 4 * cnt1["quads"]
    # every pixel of the frame is covered by the grid
    assert (d1 < 1.0).mean() > 0.99


@pytest.mark.parametrize("rows", ["0", "700"])
def test_span_scratch_fallback(gpu_lib, monkeypatch, rows):
    """When the span scratch runs out (forced small here), the remaining
    triangles walk their edges inside the raster kernel: same bits."""
    monkeypatch.setenv("SWGB_SPAN_ROWS", rows if rows != "0" else "1")
    check_scene(scenes.scene_textured_small(n_tris=150, width=96, height=72), gpu_lib)
    check_scene(scenes.scene_heightfield(quads_x=60, quads_y=30, width=160, height=96, tex_size=64), gpu_lib)
    # 4x MSAA outlines (never trimmed) and clipped polygons take the same fallback
    s = scenes.scene_small(n_tris=300, width=72, height=56, seed_index=42)
    s.samples = 4
    check_scene(s, gpu_lib)
    s = scenes.scene_small(n_tris=300, width=96, height=96, seed_index=22)
    rng = np.random.Generator(np.random.PCG64(99))
    v = s.vertices
    v[:, 0:2] = rng.uniform(-3.0, 3.0, (v.shape[0], 2))
    v[:, 2] = rng.uniform(-1.0, 2.0, v.shape[0])
    v[:, 3] = rng.uniform(-0.5, 2.0, v.shape[0])
    check_scene(s, gpu_lib)
    s.samples = 4
    check_scene(s, gpu_lib)


@pytest.mark.parametrize("per_bin", ["32", "4096", "0"])
def test_bin_list_paths(gpu_lib, monkeypatch, per_bin):
    """Bins rasterised from k_bin_list's candidate lists, by their own walk
    (lists off, or more candidates than a list holds), or a mix of both: same
    bits.  Lists are forced on for these small draws (32 entries per bin
    overflows some of their bins)."""
    monkeypatch.setenv("SWGB_BIN_LIST_MIN", "1")
    monkeypatch.setenv("SWGB_BIN_LIST", per_bin)
    check_scene(scenes.scene_textured_small(n_tris=400, width=96, height=72), gpu_lib)
    check_scene(scenes.scene_heightfield(quads_x=60, quads_y=30, width=160, height=96, tex_size=64), gpu_lib)
    s = scenes.scene_small(n_tris=600, width=72, height=56, seed_index=42)
    s.samples = 4
    check_scene(s, gpu_lib)


def _float_variant(tex_fmt, color_fmt, blend, address, mip, seed=31):
    """Random textured triangles with float textures / float attachments."""
    s = scenes.scene_textured_small(n_tris=180, width=80, height=64, tex_size=32, mip=mip, address=address,
                                    blend=False, seed_index=seed)
    rng = np.random.Generator(np.random.PCG64(seed))
    dt = np.float16 if tex_fmt == abi.FORMAT_R16G16B16A16_SFLOAT else np.float32
    if tex_fmt != abi.FORMAT_R8G8B8A8_UNORM:
        base = rng.uniform(-0.25, 1.5, (32, 32, 4))
        s.texture_levels = scenes.float_mip_chain(base, dt) if mip else [base.astype(dt)]
        s.texture_format = tex_fmt
    s.color_format = color_fmt
    s.clear_color = (0.1, 0.2, 0.3, 0.4) if color_fmt != abi.FORMAT_R8G8B8A8_UNORM else (10, 20, 30, 40)
    if blend:
        s.blend = (abi.BLEND_ONE, abi.BLEND_ONE_MINUS_SRC_ALPHA, abi.BLEND_OP_ADD,
                   abi.BLEND_ONE, abi.BLEND_ONE_MINUS_SRC_ALPHA, abi.BLEND_OP_ADD)
    return s


@pytest.mark.parametrize("tex_fmt", [abi.FORMAT_R8G8B8A8_UNORM, abi.FORMAT_B8G8R8A8_SRGB, abi.FORMAT_R16G16B16A16_SFLOAT,
                                     abi.FORMAT_R32G32B32A32_SFLOAT])
@pytest.mark.parametrize("border,linear,mixed", [
    (abi.BORDER_COLOR_FLOAT_OPAQUE_WHITE, True, False),
    (abi.BORDER_COLOR_FLOAT_TRANSPARENT_BLACK, False, False),
    (abi.BORDER_COLOR_FLOAT_OPAQUE_BLACK, True, True),
    (abi.BORDER_COLOR_FLOAT_CUSTOM_EXT, True, False),
])
def test_clamp_to_border(gpu_lib, tex_fmt, border, linear, mixed):
    """CLAMP_TO_BORDER: every texture format takes the 32-bit filter path
    (8-bit texels as their 16-bit-path values, normalized after filtering);
    texels outside the image read the border colour scaled to that path's
    units; trilinear / point; border on one axis and REPEAT on the other."""
    s = _float_variant(tex_fmt, abi.FORMAT_R8G8B8A8_UNORM, True, abi.ADDRESS_CLAMP_TO_BORDER, linear) \
        if tex_fmt in (abi.FORMAT_R16G16B16A16_SFLOAT, abi.FORMAT_R32G32B32A32_SFLOAT) else \
        scenes.scene_textured_small(n_tris=200, width=96, height=72, mip=linear, address=abi.ADDRESS_CLAMP_TO_BORDER,
                                    blend=True, seed_index=68)
    s.texture_format = tex_fmt
    s.sampler = dict(s.sampler, border_color=border, custom_border_color=(0.25, 0.5, 1.5, 0.75))
    if not linear:
        s.sampler.update(mag_filter=abi.FILTER_NEAREST, min_filter=abi.FILTER_NEAREST)
    if mixed:
        s.sampler["address_v"] = abi.ADDRESS_REPEAT
    check_scene(s, gpu_lib)


def test_mirror_clamp_nan_coordinates(gpu_lib):
    """MIRROR_CLAMP_TO_EDGE maps a NaN coordinate to the last texel, as
    ADDRESSING_MIRRORONCE's integer arithmetic does; some vertices carry NaN
    texture coordinates."""
    s = scenes.scene_textured_small(n_tris=120, width=64, height=48, mip=False, address=abi.ADDRESS_MIRROR_CLAMP_TO_EDGE,
                                    seed_index=67)
    s.vertices[::7, 8] = np.nan
    s.vertices[3::11, 9] = np.nan
    check_scene(s, gpu_lib)


@pytest.mark.parametrize("tex_fmt,color_fmt,blend,address,mip", [
    (abi.FORMAT_R32G32B32A32_SFLOAT, abi.FORMAT_R32G32B32A32_SFLOAT, False, abi.ADDRESS_CLAMP_TO_EDGE, False),
    (abi.FORMAT_R32G32B32A32_SFLOAT, abi.FORMAT_R32G32B32A32_SFLOAT, True, abi.ADDRESS_REPEAT, True),
    (abi.FORMAT_R16G16B16A16_SFLOAT, abi.FORMAT_R16G16B16A16_SFLOAT, True, abi.ADDRESS_REPEAT, True),
    (abi.FORMAT_R16G16B16A16_SFLOAT, abi.FORMAT_R32G32B32A32_SFLOAT, False, abi.ADDRESS_MIRRORED_REPEAT, True),
    (abi.FORMAT_R32G32B32A32_SFLOAT, abi.FORMAT_R8G8B8A8_UNORM, True, abi.ADDRESS_CLAMP_TO_EDGE, True),
    (abi.FORMAT_R8G8B8A8_UNORM, abi.FORMAT_R16G16B16A16_SFLOAT, True, abi.ADDRESS_REPEAT, True),
    (abi.FORMAT_R32G32B32A32_SFLOAT, abi.FORMAT_R32G32B32A32_SFLOAT, True, abi.ADDRESS_MIRROR_CLAMP_TO_EDGE, True),
    (abi.FORMAT_R16G16B16A16_SFLOAT, abi.FORMAT_R16G16B16A16_SFLOAT, False, abi.ADDRESS_MIRROR_CLAMP_TO_EDGE, False),
])
def test_float_texture_and_attachment_formats(gpu_lib, tex_fmt, color_fmt, blend, address, mip):
    """fp32 SamplerCore path (RGBA16F / RGBA32F textures) and float colour
    attachments (Reactor's Half/Float conversions), bit for bit."""
    check_scene(_float_variant(tex_fmt, color_fmt, blend, address, mip), gpu_lib)


def test_sphere_fp32_full_size(gpu_lib):
    """The adjoint workload's forward frame: 20k-triangle uv-sphere, 1024^2
    RGBA32F texture bilinear CLAMP, RGBA32F attachment at 512^2."""
    cnt = check_scene(scenes.scene_sphere_fp32(), gpu_lib)
    assert cnt["triangles_visible"] > 10000


def test_sphere_views_rgba16f_reduced(gpu_lib):
    """The batched-adjoint workload's views (noisy sphere, RGBA16F mipmapped
    trilinear, premultiplied OVER into RGBA16F) at reduced size, three views."""
    rng = np.random.Generator(np.random.PCG64(4))
    mesh = scenes.uv_sphere(rng, 60, 40, noise_sigma=0.02)
    levels = scenes.float_mip_chain(rng.uniform(0.0, 1.0, (128, 128, 4)), np.float16)
    for view in (0, 7, 200):
        s = scenes.scene_sphere_views(view, width=96, height=96, mesh=mesh, levels=levels)
        check_scene(s, gpu_lib)


@pytest.mark.parametrize("color_fmt,blend,textured", [
    (abi.FORMAT_R8G8B8A8_UNORM, False, False),
    (abi.FORMAT_R8G8B8A8_UNORM, True, True),
    (abi.FORMAT_R16G16B16A16_SFLOAT, True, True),
    (abi.FORMAT_R32G32B32A32_SFLOAT, False, True),
])
def test_msaa4(gpu_lib, color_fmt, blend, textured):
    """4x MSAA: per-sample spans, coverage, depth and colour planes; shading
    once per pixel at its centre."""
    if textured:
        s = _float_variant(abi.FORMAT_R16G16B16A16_SFLOAT, color_fmt, blend, abi.ADDRESS_REPEAT, True, seed=41)
    else:
        s = scenes.scene_small(n_tris=300, width=72, height=56, seed_index=42)
    s.samples = 4
    cnt = check_scene(s, gpu_lib)
    assert cnt["fragments_tested"] > 0


def test_msaa4_clipped_and_scissored(gpu_lib):
    s = scenes.scene_small(n_tris=300, width=96, height=80, seed_index=43)
    rng = np.random.Generator(np.random.PCG64(43))
    v = s.vertices
    v[:, 0:2] = rng.uniform(-2.0, 2.0, (v.shape[0], 2))
    v[:, 3] = rng.uniform(0.3, 1.5, v.shape[0])
    s.scissor = (5, 7, 81, 60)
    s.samples = 4
    check_scene(s, gpu_lib)


def test_sphere_views_msaa_reduced(gpu_lib):
    """The batched-adjoint view at reduced size with its 4x MSAA attachment."""
    rng = np.random.Generator(np.random.PCG64(4))
    mesh = scenes.uv_sphere(rng, 60, 40, noise_sigma=0.02)
    levels = scenes.float_mip_chain(rng.uniform(0.0, 1.0, (128, 128, 4)), np.float16)
    s = scenes.scene_sphere_views(3, width=96, height=96, mesh=mesh, levels=levels)
    s.samples = 4
    check_scene(s, gpu_lib)


@pytest.mark.parametrize("topology", [abi.TOPOLOGY_TRIANGLE_STRIP, abi.TOPOLOGY_TRIANGLE_FAN])
@pytest.mark.parametrize("index_dtype", [None, np.uint8, np.uint16, np.uint32])
def test_strips_and_fans(gpu_lib, topology, index_dtype):
    """Triangle strips and fans (setBatchIndices, first vertex provoking) with
    every index type, back faces culled."""
    check_scene(scenes.strip_fan_scene(topology, n_tris=240, indexed=index_dtype), gpu_lib)


def test_strip_with_first_and_base_vertex(gpu_lib):
    sc = scenes.strip_fan_scene(abi.TOPOLOGY_TRIANGLE_STRIP, n_tris=150, indexed=np.uint16)
    sc.vertices = np.concatenate([np.zeros((5, scenes.VERTEX_FLOATS), np.float32), sc.vertices])
    sc.base_vertex = 5
    check_scene(sc, gpu_lib)
    nd = scenes.strip_fan_scene(abi.TOPOLOGY_TRIANGLE_FAN, n_tris=150)
    nd.vertices = np.concatenate([np.zeros((9, scenes.VERTEX_FLOATS), np.float32), nd.vertices])
    nd.first_vertex = 9
    check_scene(nd, gpu_lib)


@pytest.mark.parametrize("topology", [abi.TOPOLOGY_TRIANGLE_LIST, abi.TOPOLOGY_TRIANGLE_STRIP, abi.TOPOLOGY_TRIANGLE_FAN])
@pytest.mark.parametrize("indexed", [None, np.uint16])
def test_provoking_vertex_last(gpu_lib, topology, indexed):
    """VK_EXT_provoking_vertex LAST: setBatchIndices' rotated vertex order
    (the setup's tie-breaks and clipping see it), textured and blended."""
    if topology == abi.TOPOLOGY_TRIANGLE_LIST:
        s = scenes.scene_textured_small(n_tris=200, width=96, height=72, seed_index=61)
        if indexed is not None:
            s.indices = np.arange(s.vertex_count, dtype=indexed)[::-1].copy()
            s.vertices = s.vertices[::-1].copy()
    else:
        s = scenes.strip_fan_scene(topology, n_tris=240, indexed=indexed, seed_index=62)
    s.provoking_vertex = 1
    check_scene(s, gpu_lib)


@pytest.mark.parametrize("topology", [abi.TOPOLOGY_TRIANGLE_LIST, abi.TOPOLOGY_TRIANGLE_STRIP, abi.TOPOLOGY_TRIANGLE_FAN])
@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.uint32])
def test_primitive_restart(gpu_lib, topology, dtype):
    """Primitive restart split on the device into the sub-draws
    vk::IndexBuffer::getIndexBuffers makes (leading, back-to-back and trailing
    restarts, segments too short for a triangle), both provoking modes."""
    for last in (0, 1):
        s = scenes.restart_scene(topology, n_indices=200 if dtype == np.uint8 else 700, dtype=dtype, seed_index=63 + last)
        s.provoking_vertex = last
        cnt = check_scene(s, gpu_lib)
        assert cnt["triangles_in"] > 0


def test_primitive_restart_many_blocks(gpu_lib):
    """1.5M indices: the segment scan crosses 1465 blocks of 1024 positions and
    the carry pass's chunk loop."""
    s = scenes.restart_scene(abi.TOPOLOGY_TRIANGLE_STRIP, n_indices=1_500_000, width=128, height=96, dtype=np.uint32,
                             restart_every=(50, 3000), seed_index=65)
    cnt = check_scene(s, gpu_lib)
    assert cnt["triangles_in"] > 1_000_000


@pytest.mark.parametrize("tex_fmt", [abi.FORMAT_B8G8R8A8_UNORM, abi.FORMAT_R8G8B8A8_SRGB, abi.FORMAT_B8G8R8A8_SRGB])
@pytest.mark.parametrize("mip,address", [(True, abi.ADDRESS_REPEAT), (False, abi.ADDRESS_CLAMP_TO_EDGE)])
def test_texture_formats_8bit(gpu_lib, tex_fmt, mip, address):
    """B8G8R8A8 and sRGB 8-bit textures on the 16-bit filtering path (sRGB
    texels decoded through sRGBtoLinearFF_FF00 before filtering)."""
    s = scenes.scene_textured_small(mip=mip, address=address, blend=True, seed_index=71)
    s.texture_format = tex_fmt
    check_scene(s, gpu_lib)


@pytest.mark.parametrize("write_mask", [0xF, 0b0101, 0b1010])
def test_bgra_attachment(gpu_lib, write_mask):
    """B8G8R8A8_UNORM colour attachment: R and B bytes swapped on read (blend)
    and write, write-mask bits with them."""
    s = scenes.scene_textured_small(n_tris=150, width=80, height=64, blend=True, seed_index=72)
    s.color_format = abi.FORMAT_B8G8R8A8_UNORM
    s.clear_color = (200, 100, 50, 25)
    s.color_write_mask = write_mask
    check_scene(s, gpu_lib)


@pytest.mark.parametrize("color_fmt", [abi.FORMAT_R8G8B8A8_SRGB, abi.FORMAT_B8G8R8A8_SRGB])
@pytest.mark.parametrize("blend,write_mask", [(True, 0xF), (False, 0xF), (True, 0b1011)])
def test_srgb_attachment(gpu_lib, color_fmt, blend, write_mask):
    """sRGB colour attachments: the blend decodes the destination's R, G, B with
    sRGBtoLinear and the write encodes with linearToSRGB, both through
    Pow<Mediump> (Reactor's relaxed Log2/Exp2 polynomials); 4x MSAA too."""
    s = scenes.scene_textured_small(n_tris=400, width=96, height=72, blend=blend, seed_index=76)
    s.color_format = color_fmt
    s.clear_color = (3, 60, 181, 77)
    s.color_write_mask = write_mask
    check_scene(s, gpu_lib)
    # additive blend: sums above 1 reach the encode before its clamp
    s = scenes.scene_small(n_tris=200, width=64, height=48, seed_index=77)
    s.color_format = color_fmt
    s.samples = 4
    if blend:
        s.blend = (abi.BLEND_ONE, abi.BLEND_ONE, abi.BLEND_OP_ADD, abi.BLEND_ONE, abi.BLEND_ONE, abi.BLEND_OP_ADD)
    check_scene(s, gpu_lib)


def test_d16_depth(gpu_lib):
    """D16_UNORM depth: fragments quantized to Round(z * 0xFFFF) and compared
    against the stored integers, every compare op; 4x MSAA; dense overlap."""
    for op in range(8):
        s = scenes.scene_small(n_tris=120, width=64, height=48, seed_index=25)
        s.depth_format = abi.FORMAT_D16_UNORM
        s.depth_compare = op
        s.clear_depth = 0.5
        check_scene(s, gpu_lib)
    s = scenes.scene_small(n_tris=2000, width=96, height=96, seed_index=14)
    s.depth_format = abi.FORMAT_D16_UNORM
    check_scene(s, gpu_lib)
    s = scenes.scene_small(n_tris=300, width=72, height=56, seed_index=42)
    s.depth_format = abi.FORMAT_D16_UNORM
    s.samples = 4
    check_scene(s, gpu_lib)
    s = scenes.scene_heightfield(quads_x=160, quads_y=80, width=320, height=180, tex_size=256)
    s.depth_format = abi.FORMAT_D16_UNORM
    s.color_format = abi.FORMAT_B8G8R8A8_UNORM
    s.texture_format = abi.FORMAT_B8G8R8A8_SRGB
    check_scene(s, gpu_lib)


@pytest.mark.parametrize("bias", [(3.0, 0.0, 0.0), (0.0, 1.5, 0.0), (-200.0, -2.0, -0.001), (1e5, 4.0, 0.002)])
@pytest.mark.parametrize("d16", [False, True])
def test_depth_bias(gpu_lib, bias, d16):
    """Depth bias: constant (minimum resolvable difference per polygon for
    D32F, 1.01/0xFFFF for D16), slope, and clamp, over dense overlap where the
    bias decides the order; GREATER as well as LESS."""
    for op in (abi.COMPARE_LESS, abi.COMPARE_GREATER_OR_EQUAL):
        s = scenes.scene_small(n_tris=800, width=96, height=80, seed_index=74)
        s.depth_bias = bias
        s.depth_compare = op
        s.clear_depth = 1.0 if op == abi.COMPARE_LESS else 0.0
        if d16:
            s.depth_format = abi.FORMAT_D16_UNORM
        check_scene(s, gpu_lib)


@pytest.mark.parametrize("bounds", [(0.0, 1.0), (0.3, 0.7), (0.5, 0.5), (0.9, 0.2)])
@pytest.mark.parametrize("depth_test", [True, False])
def test_depth_bounds(gpu_lib, bounds, depth_test):
    """Depth bounds test on the stored depth after the depth test (or masking
    the coverage without one), D32F and D16, with 4x MSAA."""
    for d16, samples in ((False, 1), (True, 1), (False, 4)):
        s = scenes.scene_small(n_tris=600, width=72, height=64, seed_index=75)
        s.depth_bounds = bounds
        s.depth_test = depth_test
        s.clear_depth = 0.6
        s.samples = samples
        if d16:
            s.depth_format = abi.FORMAT_D16_UNORM
        check_scene(s, gpu_lib)


def check_stencil_scene(scene):
    import torch
    import oracle
    from swiftshader_gb300 import DeviceScene, Renderer
    r = Renderer(0)
    ds = DeviceScene(scene)
    torch.cuda.synchronize()
    r.reset_counters()
    r.draw(ds.state(), ds.args())
    r.synchronize()
    c_ref, d_ref, s_ref, cnt_ref = oracle.render_stencil(scene, 4)
    assert_bit_exact(ds.stencil.cpu().numpy(), s_ref, "stencil")
    assert_bit_exact(ds.depth_numpy(), d_ref, "depth")
    assert_bit_exact(ds.color.cpu().numpy(), c_ref, "color")
    assert_counters(r.counters(), cnt_ref)
    return cnt_ref


K, Z, R, IC, DC, INV, IW, DW = range(8)
STENCIL_CASES = [
    # front: (fail, pass, depth_fail, compare, compare_mask, write_mask, ref), back likewise, clear
    ((K, IW, K, abi.COMPARE_ALWAYS, 0xFF, 0xFF, 0), (K, DW, K, abi.COMPARE_ALWAYS, 0xFF, 0xFF, 0), 7),
    ((INV, R, IC, abi.COMPARE_LESS, 0x0F, 0xF0, 5), (DC, Z, INV, abi.COMPARE_GREATER_OR_EQUAL, 0xFF, 0x3F, 9), 6),
    ((R, K, K, abi.COMPARE_EQUAL, 0xFF, 0xFF, 4), (R, K, K, abi.COMPARE_NOT_EQUAL, 0xFF, 0xFF, 4), 4),
    ((K, IC, K, abi.COMPARE_LESS_OR_EQUAL, 0xFF, 0x00, 200), (K, DC, K, abi.COMPARE_GREATER, 0xFF, 0xFF, 3), 250),
    ((K, K, K, abi.COMPARE_NEVER, 0xFF, 0xFF, 0), (K, K, K, abi.COMPARE_ALWAYS, 0xFF, 0xFF, 0), 0),
]


@pytest.mark.parametrize("case", range(len(STENCIL_CASES)))
@pytest.mark.parametrize("depth_test,samples", [(True, 1), (False, 1), (True, 4)])
def test_stencil(gpu_lib, case, depth_test, samples):
    """Stencil test and ops (front / back by facing, compare and write masks,
    every op and compare), with and without a depth test, 4x MSAA; cases whose
    ops act on failing fragments run without early depth rejection."""
    front, back, clear = STENCIL_CASES[case]
    s = scenes.scene_small(n_tris=700, width=88, height=72, seed_index=77 + case)
    s.stencil = {"front": front, "back": back, "clear": clear}
    s.depth_test = depth_test
    s.samples = samples
    cnt = check_stencil_scene(s)
    assert cnt["fragments_tested"] > 0 or not depth_test


def test_stencil_with_bounds_and_d16(gpu_lib):
    s = scenes.scene_small(n_tris=700, width=88, height=72, seed_index=83)
    s.stencil = {"front": STENCIL_CASES[1][0], "back": STENCIL_CASES[1][1], "clear": 6}
    s.depth_bounds = (0.2, 0.8)
    s.clear_depth = 0.7
    s.depth_format = abi.FORMAT_D16_UNORM
    check_stencil_scene(s)


def test_raster_waits_for_texture_event(gpu_lib):
    """swgb_draw_args.raster_wait_event: textures uploaded on another stream
    that is kept busy first; the draw's raster stage waits for the event, so
    the frame equals the one drawn with the textures already in place (a
    raster that ran early would read the zeroed texture levels)."""
    import torch
    from swiftshader_gb300 import DeviceScene, Renderer
    s = scenes.scene_textured_small(n_tris=300, width=96, height=72)
    c_ref, d_ref, _ = render_gpu(s)
    r = Renderer(0)
    ds = DeviceScene(s)
    host_tex = ds.texture_region.cpu().pin_memory()
    ds.texture_region.zero_()
    busy = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    ev = torch.cuda.Event()
    with torch.cuda.stream(side):
        for i in range(20):
            busy.fill_(i)
        ds.texture_region.copy_(host_tex, non_blocking=True)
        ev.record(side)
    a = ds.args()
    a.raster_wait_event = ev.cuda_event
    ds.clear(r)
    r.draw(ds.state(), a)
    r.synchronize()
    torch.cuda.synchronize()
    assert_bit_exact(ds.color.cpu().numpy(), c_ref, "color")
    assert_bit_exact(ds.depth_numpy(), d_ref, "depth")
