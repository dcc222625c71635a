"""Seeded cases of the routine-level reference fixtures (refjit_fixtures.npz).

Shared by make_refjit_fixtures.py (which runs SwiftShader's own routines on
them, built from the reference sources by oracle/refjit/build_refjit.py) and
tests/test_oracle_reference_fixtures.py (which runs the oracle on them and
compares).  Every case is regenerated from its seed, so the fixture file holds
only the reference's outputs and a digest of the inputs they were made from.
"""
import numpy as np

from swiftshader_gb300 import abi, scenes

# (fail, pass, depth_fail, compare, compare_mask, write_mask, reference) per face, clear value
K, Z, R, IC, DC, INV, IW, DW = range(8)
STENCIL = [
    ((K, IW, K, abi.COMPARE_ALWAYS, 0xFF, 0xFF, 0), (K, DW, K, abi.COMPARE_ALWAYS, 0xFF, 0xFF, 0), 7),
    ((INV, R, IC, abi.COMPARE_LESS, 0x0F, 0xF0, 5), (DC, Z, INV, abi.COMPARE_GREATER_OR_EQUAL, 0xFF, 0x3F, 9), 6),
    ((R, K, K, abi.COMPARE_EQUAL, 0xFF, 0xFF, 4), (R, K, K, abi.COMPARE_NOT_EQUAL, 0xFF, 0xFF, 4), 4),
    ((K, IC, K, abi.COMPARE_LESS_OR_EQUAL, 0xFF, 0x00, 200), (K, DC, K, abi.COMPARE_GREATER, 0xFF, 0xFF, 3), 250),
]


def _clip_heavy(s, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    v = s.vertices
    v[:, 0:2] = rng.uniform(-3.0, 3.0, (v.shape[0], 2))
    v[:, 2] = rng.uniform(-1.0, 2.0, v.shape[0])
    v[:, 3] = rng.uniform(-0.5, 2.0, v.shape[0])
    return s


def _degenerate(s):
    v = s.vertices
    v[3:6, 0:2] = v[3, 0:2]
    v[6:9, 0] = np.array([0.1, 0.2, 0.3])
    v[6:9, 1] = np.array([0.1, 0.2, 0.3])
    v[9:12, 0:2] = v[9, 0:2] + np.array([[0, 0], [1e-4, 0], [0, 1e-4]], np.float32)
    v[12, 0] = np.inf
    v[15, 1] = np.nan
    return s


def setup_cases():
    """name -> scene whose triangles the setup routine is pinned on."""
    c = {}
    c["small"] = scenes.scene_small(n_tris=200, width=96, height=80, seed_index=21)
    c["clip_all_planes"] = _clip_heavy(scenes.scene_small(n_tris=300, width=128, height=128, seed_index=22), 99)
    s = scenes.scene_small(n_tris=200, width=72, height=56, seed_index=42)
    s.samples = 4
    c["msaa4"] = s
    s = _clip_heavy(scenes.scene_small(n_tris=150, width=64, height=64, seed_index=43), 98)
    s.samples = 4
    c["msaa4_clip"] = s
    for i, (cull, ff) in enumerate([(abi.CULL_BACK, abi.FRONT_FACE_CCW), (abi.CULL_FRONT, abi.FRONT_FACE_CW)]):
        s = scenes.scene_small(n_tris=150, width=64, height=48, seed_index=44 + i)
        s.cull_mode, s.front_face = cull, ff
        c["cull%d" % i] = s
    s = scenes.scene_small(n_tris=200, width=160, height=120, seed_index=23)
    s.viewport = (10, -5, 130, 110)
    s.scissor = (7, 9, 101, 77)
    c["scissor_viewport"] = s
    for i, bias in enumerate([(3.0, 1.5, 0.002), (-200.0, -2.0, -0.001)]):
        s = scenes.scene_small(n_tris=150, width=96, height=80, seed_index=74)
        s.depth_bias = bias
        c["bias%d" % i] = s
    s = scenes.scene_small(n_tris=150, width=96, height=80, seed_index=74)
    s.depth_bias = (3.0, 1.5, 0.0)
    s.depth_format = abi.FORMAT_D16_UNORM
    c["bias_d16"] = s
    c["degenerate"] = _degenerate(scenes.scene_small(n_tris=64, width=64, height=64, seed_index=26))
    c["textured"] = scenes.scene_textured_small(n_tris=120)
    c["heightfield"] = scenes.scene_heightfield(quads_x=24, quads_y=12, width=160, height=90, tex_size=64)
    return c


def raster_cases():
    """name -> scene drawn depth / stencil only by the reference's rasteriser."""
    c = {}
    c["small"] = scenes.scene_small(n_tris=300, width=96, height=80, seed_index=21)
    for op in range(8):
        s = scenes.scene_small(n_tris=100, width=48, height=40, seed_index=25)
        s.depth_compare = op
        s.clear_depth = 0.5
        c["compare%d" % op] = s
    c["clip_all_planes"] = _clip_heavy(scenes.scene_small(n_tris=300, width=96, height=96, seed_index=22), 99)
    s = scenes.scene_small(n_tris=250, width=64, height=48, seed_index=42)
    s.samples = 4
    c["msaa4"] = s
    s = scenes.scene_small(n_tris=250, width=64, height=48, seed_index=42)
    s.depth_format = abi.FORMAT_D16_UNORM
    c["d16"] = s
    s = scenes.scene_small(n_tris=500, width=80, height=64, seed_index=74)
    s.depth_bias = (3.0, 1.5, 0.002)
    c["bias"] = s
    s = scenes.scene_small(n_tris=500, width=64, height=56, seed_index=75)
    s.depth_bounds = (0.3, 0.7)
    s.clear_depth = 0.6
    c["bounds"] = s
    s = scenes.scene_small(n_tris=300, width=56, height=48, seed_index=76)
    s.depth_bounds = (0.2, 0.8)
    s.clear_depth = 0.7
    s.depth_format = abi.FORMAT_D16_UNORM
    s.samples = 4
    c["bounds_d16_msaa4"] = s
    for i, (front, back, clear) in enumerate(STENCIL):
        s = scenes.scene_small(n_tris=500, width=72, height=56, seed_index=77 + i)
        s.stencil = {"front": front, "back": back, "clear": clear}
        s.depth_test = i != 2
        s.samples = 4 if i == 1 else 1
        c["stencil%d" % i] = s
    c["degenerate"] = _degenerate(scenes.scene_small(n_tris=64, width=48, height=48, seed_index=26))
    return c


SAMPLER_FORMATS = [abi.FORMAT_R8G8B8A8_UNORM, abi.FORMAT_B8G8R8A8_UNORM, abi.FORMAT_R8G8B8A8_SRGB,
                   abi.FORMAT_R16G16B16A16_SFLOAT, abi.FORMAT_R32G32B32A32_SFLOAT]
SAMPLER_ADDRESS = [abi.ADDRESS_REPEAT, abi.ADDRESS_CLAMP_TO_EDGE, abi.ADDRESS_MIRRORED_REPEAT,
                   abi.ADDRESS_MIRROR_CLAMP_TO_EDGE, abi.ADDRESS_CLAMP_TO_BORDER]
QUADS_PER_CONFIG = 8


def sampler_textures():
    """(format, w, h) -> full mip chain (seeded texels)."""
    out = {}
    for fi, fmt in enumerate(SAMPLER_FORMATS):
        for (w, h) in [(32, 32), (37, 23)]:
            rng = np.random.Generator(np.random.PCG64(0x5357_1000 + 16 * fi + w))
            if fmt in (abi.FORMAT_R16G16B16A16_SFLOAT, abi.FORMAT_R32G32B32A32_SFLOAT):
                dt = np.float16 if fmt == abi.FORMAT_R16G16B16A16_SFLOAT else np.float32
                chain = scenes.float_mip_chain(rng.uniform(-0.5, 1.5, (h, w, 4)), dt)
            else:
                chain = scenes.box_mip_chain(rng.integers(0, 256, (h, w, 4), dtype=np.uint8))
            out[(fmt, w, h)] = [np.ascontiguousarray(l) for l in chain]
    return out


def sampler_configs():
    """List of (format, w, h, filter, mipmap_mode, address, border, lod_bias, min_lod, max_lod)."""
    out = []
    for fmt in SAMPLER_FORMATS:
        for (w, h) in [(32, 32), (37, 23)]:
            for filt in (abi.FILTER_NEAREST, abi.FILTER_LINEAR):
                for mip in (abi.MIPMAP_MODE_NEAREST, abi.MIPMAP_MODE_LINEAR):
                    for addr in SAMPLER_ADDRESS:
                        borders = ([abi.BORDER_COLOR_FLOAT_TRANSPARENT_BLACK, abi.BORDER_COLOR_FLOAT_OPAQUE_WHITE,
                                    abi.BORDER_COLOR_FLOAT_CUSTOM_EXT] if addr == abi.ADDRESS_CLAMP_TO_BORDER
                                   else [abi.BORDER_COLOR_FLOAT_TRANSPARENT_BLACK])
                        for b in borders:
                            out.append((fmt, w, h, filt, mip, addr, b, 0.0, 0.0, 1000.0))
            # LOD bias and clamps
            out.append((fmt, w, h, abi.FILTER_LINEAR, abi.MIPMAP_MODE_LINEAR, abi.ADDRESS_REPEAT,
                        abi.BORDER_COLOR_FLOAT_TRANSPARENT_BLACK, 1.25, 0.5, 2.75))
            out.append((fmt, w, h, abi.FILTER_LINEAR, abi.MIPMAP_MODE_LINEAR, abi.ADDRESS_REPEAT,
                        abi.BORDER_COLOR_FLOAT_TRANSPARENT_BLACK, -0.75, 0.0, 1000.0))
    return out


def sampler_quads(ci, w, h):
    """QUADS_PER_CONFIG quads of (u, v) for config index ci: footprints from
    strong magnification to minification past the last level."""
    rng = np.random.Generator(np.random.PCG64(0x5357_2000 + ci))
    us, vs = [], []
    for _ in range(QUADS_PER_CONFIG):
        scale = 2.0 ** rng.uniform(-6, 4)
        u0, v0 = rng.uniform(-1.5, 2.5, 2)
        du = rng.uniform(-1, 1, 2) * scale / w
        dv = rng.uniform(-1, 1, 2) * scale / h
        us.append([u0, u0 + du[0], u0 + du[1], u0 + du[0] + du[1]])
        vs.append([v0, v0 + dv[0], v0 + dv[1], v0 + dv[0] + dv[1]])
    return np.asarray(us, np.float32), np.asarray(vs, np.float32)


def texture_struct(chain, cfg):
    """abi.Texture over host arrays for one sampler config."""
    import ctypes as C
    fmt, w, h, filt, mip, addr, border, bias, mn, mx = cfg
    t = abi.Texture()
    t.format = fmt
    t.level_count = len(chain)
    for i, lv in enumerate(chain):
        t.levels[i] = abi.TextureLevel(lv.ctypes.data, lv.shape[1], lv.shape[0], lv.shape[1], 0)
    t.mag_filter = t.min_filter = filt
    t.mipmap_mode = mip
    t.address_u = t.address_v = addr
    t.mip_lod_bias, t.min_lod, t.max_lod = bias, mn, mx
    t.border_color = border
    t.custom_border_color = (C.c_float * 4)(0.125, 0.625, -0.25, 0.75)
    return t
