"""Triangle strips and fans in the oracle (setBatchIndices with the first
vertex provoking, src/Device/Renderer.cpp:97-134): every triangle of a regular
strip or a convex fan has the winding of the first one, and the index types
(uint8 / uint16 / uint32, or none) give the same frame."""
import numpy as np
import pytest

from swiftshader_gb300 import abi, scenes


def regular(topology, n, reverse=False):
    if topology == abi.TOPOLOGY_TRIANGLE_STRIP:
        xs = np.linspace(-0.9, 0.9, n // 2 + 2)
        pts = [(x, y) for x in xs for y in (-0.5, 0.5)][:n + 2]
    else:
        ang = np.linspace(0.0, 2.0 * np.pi, n + 1)
        pts = [(0.0, 0.0)] + [(0.8 * np.cos(a), 0.8 * np.sin(a)) for a in ang]
    if reverse:
        pts = [(x, -y) for x, y in pts]
    v = np.zeros((len(pts), scenes.VERTEX_FLOATS), np.float32)
    v[:, 0:2] = pts
    v[:, 2] = 0.5
    v[:, 3] = 1.0
    v[:, 4:8] = 1.0
    return scenes.Scene(name="regular", width=64, height=64, vertices=v, tri_count=n, topology=topology,
                        cull_mode=abi.CULL_BACK)


@pytest.mark.parametrize("topology", [abi.TOPOLOGY_TRIANGLE_STRIP, abi.TOPOLOGY_TRIANGLE_FAN])
def test_regular_strip_and_fan_keep_one_winding(oracle_mod, topology):
    _, _, a = oracle_mod.render(regular(topology, 20))
    _, _, b = oracle_mod.render(regular(topology, 20, reverse=True))
    # one orientation is entirely front-facing, the mirrored one entirely back-facing
    assert sorted([a["triangles_visible"], b["triangles_visible"]]) == [0, 20]


@pytest.mark.parametrize("topology", [abi.TOPOLOGY_TRIANGLE_STRIP, abi.TOPOLOGY_TRIANGLE_FAN])
def test_index_types_give_the_same_frame(oracle_mod, topology):
    ref = oracle_mod.render(scenes.strip_fan_scene(topology, n_tris=200))
    for dt in (np.uint8, np.uint16, np.uint32):
        got = oracle_mod.render(scenes.strip_fan_scene(topology, n_tris=200, indexed=dt))
        assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1]) and got[2] == ref[2]


def test_first_and_base_vertex(oracle_mod):
    """first_vertex (non-indexed) and base_vertex shift the vertices read."""
    sc = scenes.strip_fan_scene(abi.TOPOLOGY_TRIANGLE_STRIP, n_tris=100)
    ref = oracle_mod.render(sc)
    pad = np.zeros((7, scenes.VERTEX_FLOATS), np.float32)
    shifted = scenes.strip_fan_scene(abi.TOPOLOGY_TRIANGLE_STRIP, n_tris=100)
    shifted.vertices = np.concatenate([pad, sc.vertices])
    shifted.first_vertex = 7
    got = oracle_mod.render(shifted)
    assert np.array_equal(got[0], ref[0]) and got[2] == ref[2]


def split_restart(indices, topology, restart):
    """vk::IndexBuffer's ProcessPrimitiveRestart restated in numpy: the
    (first index, primitive count) of every sub-draw."""
    out, start, n = [], 0, 0
    for i, v in enumerate(list(indices) + [restart]):
        if v == restart:
            prims = (n // 3) if topology == abi.TOPOLOGY_TRIANGLE_LIST else max(n, 2) - 2
            if n and prims:
                out.append((start, prims))
            n = 0
        else:
            if n == 0:
                start = i
            n += 1
    return out


@pytest.mark.parametrize("topology", [abi.TOPOLOGY_TRIANGLE_LIST, abi.TOPOLOGY_TRIANGLE_STRIP, abi.TOPOLOGY_TRIANGLE_FAN])
@pytest.mark.parametrize("last", [0, 1])
def test_primitive_restart_equals_sub_draws(oracle_mod, topology, last):
    """A restart draw renders as its sub-draws drawn one after another, each
    from its own first index (the reference's Renderer::draw per sub-draw)."""
    sc = scenes.restart_scene(topology, n_indices=500, dtype=np.uint16, seed_index=66)
    sc.provoking_vertex = last
    got = oracle_mod.render(sc)
    color, depth = scenes.clear_buffers(sc)
    total = {}
    for start, prims in split_restart(sc.indices, topology, 0xFFFF):
        sub = scenes.restart_scene(topology, n_indices=500, dtype=np.uint16, seed_index=66)
        sub.provoking_vertex = last
        sub.restart_index_count = 0
        sub.indices = sc.indices[start:].copy()
        sub.tri_count = prims
        _, _, cnt = oracle_mod.render(sub, color=color, depth=depth)
        for k, v in cnt.items():
            total[k] = (total.get(k, 0) | v) if k == "texture_levels_mask" else total.get(k, 0) + v
    assert np.array_equal(got[0], color) and np.array_equal(got[1], depth)
    assert got[2] == total and total["triangles_in"] > 50


def test_provoking_vertex_last_rotates_vertices(oracle_mod):
    """LAST draws each triangle from its rotated vertex list: the same as a
    FIRST draw of a list whose triangles were rotated by hand."""
    sc = scenes.scene_small(n_tris=150, width=64, height=48, seed_index=67)
    sc.provoking_vertex = 1
    got = oracle_mod.render(sc)
    rot = scenes.scene_small(n_tris=150, width=64, height=48, seed_index=67)
    v = rot.vertices.reshape(150, 3, -1)
    rot.vertices = np.ascontiguousarray(v[:, [2, 0, 1], :].reshape(450, -1))
    ref = oracle_mod.render(rot)
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1]) and got[2] == ref[2]


def test_bgra_attachment_and_texture_are_swizzles(oracle_mod):
    """B8G8R8A8 attachments and textures hold R and B swapped: a BGRA draw of a
    BGRA copy of the texture equals the RGBA draw with R and B bytes swapped,
    write-mask bits included."""
    base = scenes.scene_textured_small(n_tris=120, width=64, height=48, tex_size=32, seed_index=68)
    base.clear_color = (10, 20, 30, 40)
    base.color_write_mask = 0b1011  # R, G, A
    ref = oracle_mod.render(base)
    sw = scenes.scene_textured_small(n_tris=120, width=64, height=48, tex_size=32, seed_index=68)
    sw.clear_color = (30, 20, 10, 40)
    sw.color_write_mask = 0b1011
    sw.color_format = abi.FORMAT_B8G8R8A8_UNORM
    sw.texture_format = abi.FORMAT_B8G8R8A8_UNORM
    sw.texture_levels = [np.ascontiguousarray(lv[..., [2, 1, 0, 3]]) for lv in sw.texture_levels]
    got = oracle_mod.render(sw)
    assert np.array_equal(got[0][..., [2, 1, 0, 3]], ref[0]) and np.array_equal(got[1], ref[1]) and got[2] == ref[2]


def test_srgb_table_and_d16_quantization(oracle_mod):
    """sRGB textures decode through sRGBtoLinearFF_FF00 (0 -> 0, 255 -> 0xFF00,
    monotonic); a D16_UNORM draw stores every depth a D32F draw of the same
    scene stores, rounded to 16 bits, where the two keep the same fragments."""
    s = scenes.scene_textured_small(n_tris=60, width=48, height=40, tex_size=16, mip=False, blend=False, seed_index=69)
    s.texture_levels = [np.full_like(s.texture_levels[0], 255)]
    s.texture_format = abi.FORMAT_R8G8B8A8_SRGB
    a = oracle_mod.render(s)
    s.texture_format = abi.FORMAT_R8G8B8A8_UNORM
    b = oracle_mod.render(s)
    assert np.array_equal(a[0], b[0])  # sRGB 255 decodes to exactly 1.0, like UNORM 255
    d32 = scenes.scene_small(n_tris=1, width=64, height=64, seed_index=70)
    d16 = scenes.scene_small(n_tris=1, width=64, height=64, seed_index=70)
    d16.depth_format = abi.FORMAT_D16_UNORM
    z32 = oracle_mod.render(d32)[1]
    z16 = oracle_mod.render(d16)[1]
    covered = z32 < 1.0
    assert covered.any()
    assert np.array_equal(z16[covered], np.rint(z32[covered].astype(np.float64) * 65535.0).astype(np.uint16))


def test_depth_bias_constant_known_answer(oracle_mod):
    """A constant-depth triangle at z = 0.5 with constant bias 2^20: r =
    2^(e - 23) with e the exponent of 0.5, so every covered depth becomes
    0.5 + 2^20 * 2^-24 = 0.5625 (SetupRoutine.cpp:417-476); a clamp of 0.03
    limits it to 0.53."""
    s = scenes.scene_small(n_tris=1, width=32, height=32, seed_index=73)
    s.vertices[:, 0:2] = np.array([[-0.9, -0.9], [0.9, -0.9], [0.0, 0.9]], np.float32)
    s.vertices[:, 2] = 0.5
    s.depth_bias = (float(2 ** 20), 0.0, 0.0)
    d = oracle_mod.render(s)[1]
    assert (d[d < 1.0] == np.float32(0.5625)).all() and (d < 1.0).sum() > 100
    s.depth_bias = (float(2 ** 20), 0.0, 0.03)
    d = oracle_mod.render(s)[1]
    assert (d[d < 1.0] == np.float32(0.5) + np.float32(0.03)).all()


def test_stencil_counts_fragments(oracle_mod):
    """Stencil INCREMENT_AND_WRAP on pass with compare ALWAYS and depth ALWAYS:
    the stencil attachment ends holding, per pixel, how many fragments
    passed; their sum is the fragments_passed counter."""
    s = scenes.scene_small(n_tris=300, width=64, height=48, seed_index=76)
    s.depth_compare = abi.COMPARE_ALWAYS
    op = (abi.STENCIL_OP_KEEP, abi.STENCIL_OP_INCREMENT_AND_WRAP, abi.STENCIL_OP_KEEP, abi.COMPARE_ALWAYS, 0xFF, 0xFF, 0)
    s.stencil = {"front": op, "back": op, "clear": 0}
    _, _, st, cnt = oracle_mod.render_stencil(s)
    assert int(st.astype(np.int64).sum()) == cnt["fragments_passed"] > 1000


def test_mirror_clamp_to_edge_is_clamp_of_abs(oracle_mod):
    """MIRROR_CLAMP_TO_EDGE (ADDRESSING_MIRRORONCE, SamplerCore.cpp:2418-2428,
    2554-2558) addresses |u| with CLAMP_TO_EDGE's result: a draw whose texture
    coordinates are negated renders under MIRROR_CLAMP_TO_EDGE exactly what
    the original renders under CLAMP_TO_EDGE (negation is exact through the
    plane equations and the interpolation), on the 16-bit and fp32 paths."""
    from swiftshader_gb300 import abi, scenes
    for fmt in (abi.FORMAT_R8G8B8A8_UNORM, abi.FORMAT_R32G32B32A32_SFLOAT):
        a = scenes.scene_textured_small(n_tris=60, width=48, height=40, mip=True, address=abi.ADDRESS_CLAMP_TO_EDGE,
                                        seed_index=66)
        if fmt != abi.FORMAT_R8G8B8A8_UNORM:
            a.texture_format = fmt
            a.texture_levels = [lv.astype(np.float32) / 255.0 for lv in a.texture_levels]
        b = scenes.scene_textured_small(n_tris=60, width=48, height=40, mip=True, address=abi.ADDRESS_MIRROR_CLAMP_TO_EDGE,
                                        seed_index=66)
        b.texture_format, b.texture_levels = a.texture_format, a.texture_levels
        a.vertices[:, 8:10] = np.abs(a.vertices[:, 8:10])  # u, v >= 0: CLAMP_TO_EDGE of u is that of |-u|
        b.vertices = a.vertices.copy()
        b.vertices[:, 8:10] = -b.vertices[:, 8:10]
        ca, da, _ = oracle_mod.render(a)
        cb, db, _ = oracle_mod.render(b)
        assert np.array_equal(da, db)
        assert np.array_equal(ca, cb)
        # and it differs from plain CLAMP_TO_EDGE of the negated coordinates
        b.sampler = dict(b.sampler, address_u=abi.ADDRESS_CLAMP_TO_EDGE, address_v=abi.ADDRESS_CLAMP_TO_EDGE)
        cc, _, _ = oracle_mod.render(b)
        assert not np.array_equal(cc, ca)


def test_clamp_to_border_sampling(oracle_mod):
    """CLAMP_TO_BORDER on the oracle's 32-bit path: point samples inside the
    image return the texel (8-bit: b << 8 normalized by 1 / 0xFF00), outside
    it the border colour (custom colours scaled by 0xFF00 and back)."""
    import ctypes as C
    from swiftshader_gb300 import abi
    tex = np.arange(4 * 4 * 4, dtype=np.uint8).reshape(4, 4, 4) * 3
    t = abi.Texture()
    t.format = abi.FORMAT_R8G8B8A8_UNORM
    t.level_count = 1
    t.levels[0] = abi.TextureLevel(tex.ctypes.data, 4, 4, 4, 0)
    t.mag_filter = t.min_filter = abi.FILTER_NEAREST
    t.mipmap_mode = abi.MIPMAP_MODE_NEAREST
    t.address_u = t.address_v = abi.ADDRESS_CLAMP_TO_BORDER
    t.max_lod = 0.0
    t.border_color = abi.BORDER_COLOR_FLOAT_CUSTOM_EXT
    t.custom_border_color = (C.c_float * 4)(0.25, 0.5, 1.5, 0.75)
    u = (C.c_float * 4)(0.125, 0.625, -0.1, 1.2)
    v = (C.c_float * 4)(0.375, 0.875, 0.5, 0.5)
    out = (C.c_float * 16)()
    assert oracle_mod.lib().oracle_sample_quad(C.byref(t), u, v, out) == 0
    o = np.array(out, np.float32).reshape(4, 4)
    inv = np.float32(1.0) / np.float32(65280.0)
    for lane, (x, y) in enumerate([(0, 1), (2, 3)]):
        assert np.array_equal(o[lane], (tex[y, x].astype(np.float32) * np.float32(256)) * inv)
    border = (np.float32(65280.0) * np.array([0.25, 0.5, 1.5, 0.75], np.float32)) * inv
    assert np.array_equal(o[2], border) and np.array_equal(o[3], border)
    assert abs(o[2][2] - 1.5) < 1e-6  # custom colours are not clamped
