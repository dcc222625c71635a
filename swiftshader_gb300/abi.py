"""ctypes mirror of include/swgb.h.

The structs here are byte-for-byte the C-ABI structs; ``tests/test_abi.py``
checks their sizes and offsets against the header.  The same structs drive the
GB300 library (device pointers) and the CPU oracle used by the tests (host
pointers).
"""
import ctypes as C

# swgb_status
OK = 0
UNSUPPORTED_STATE = 1
INVALID_ARG = 2
OOM = 3
DEVICE_TIMEOUT = 4
DEVICE_ERROR = 5
NO_DEVICE = 6
STATUS_NAMES = {0: "OK", 1: "UNSUPPORTED_STATE", 2: "INVALID_ARG", 3: "OOM",
                4: "DEVICE_TIMEOUT", 5: "DEVICE_ERROR", 6: "NO_DEVICE"}

# VkFormat subset
FORMAT_R8G8B8A8_UNORM = 37
FORMAT_R8G8B8A8_SRGB = 43
FORMAT_B8G8R8A8_UNORM = 44
FORMAT_B8G8R8A8_SRGB = 50
FORMAT_D16_UNORM = 124
FORMAT_R16G16B16A16_SFLOAT = 97
FORMAT_R32G32_SFLOAT = 103
FORMAT_R32G32B32A32_SFLOAT = 109
FORMAT_D32_SFLOAT = 126
FORMAT_S8_UINT = 127
TOPOLOGY_TRIANGLE_LIST = 3
TOPOLOGY_TRIANGLE_STRIP = 4
TOPOLOGY_TRIANGLE_FAN = 5
INDEX_TYPE_UINT16 = 0
INDEX_TYPE_UINT32 = 1
INDEX_TYPE_UINT8 = 1000265000
INDEX_TYPE_NONE = 0xFFFFFFFF
CULL_NONE, CULL_FRONT, CULL_BACK, CULL_FRONT_AND_BACK = 0, 1, 2, 3
FRONT_FACE_CCW, FRONT_FACE_CW = 0, 1
(COMPARE_NEVER, COMPARE_LESS, COMPARE_EQUAL, COMPARE_LESS_OR_EQUAL, COMPARE_GREATER,
 COMPARE_NOT_EQUAL, COMPARE_GREATER_OR_EQUAL, COMPARE_ALWAYS) = range(8)
(BLEND_ZERO, BLEND_ONE, BLEND_SRC_COLOR, BLEND_ONE_MINUS_SRC_COLOR, BLEND_DST_COLOR,
 BLEND_ONE_MINUS_DST_COLOR, BLEND_SRC_ALPHA, BLEND_ONE_MINUS_SRC_ALPHA, BLEND_DST_ALPHA,
 BLEND_ONE_MINUS_DST_ALPHA) = range(10)
BLEND_OP_ADD, BLEND_OP_SUBTRACT, BLEND_OP_REVERSE_SUBTRACT, BLEND_OP_MIN, BLEND_OP_MAX = range(5)
FILTER_NEAREST, FILTER_LINEAR = 0, 1
MIPMAP_MODE_NEAREST, MIPMAP_MODE_LINEAR = 0, 1
ADDRESS_REPEAT, ADDRESS_MIRRORED_REPEAT, ADDRESS_CLAMP_TO_EDGE = 0, 1, 2
ADDRESS_CLAMP_TO_BORDER = 3
ADDRESS_MIRROR_CLAMP_TO_EDGE = 4
BORDER_COLOR_FLOAT_TRANSPARENT_BLACK, BORDER_COLOR_FLOAT_OPAQUE_BLACK, BORDER_COLOR_FLOAT_OPAQUE_WHITE = 0, 2, 4
BORDER_COLOR_FLOAT_CUSTOM_EXT = 1000287003
VS_MVP_PASSTHROUGH = 1
FS_VCOLOR = 1
FS_TEX_X_VCOLOR = 2
PRECISION_CMAKE = 0
PRECISION_LEGACY = 1
MAX_ATTRIBS = 4
MAX_MIP_LEVELS = 15


class VertexAttrib(C.Structure):
    _fields_ = [("format", C.c_uint32), ("binding", C.c_uint32),
                ("offset", C.c_uint32), ("reserved", C.c_uint32)]


class VertexBinding(C.Structure):
    _fields_ = [("buffer", C.c_void_p), ("stride", C.c_uint32), ("reserved", C.c_uint32)]


class TextureLevel(C.Structure):
    _fields_ = [("buffer", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32),
                ("pitch_texels", C.c_uint32), ("reserved", C.c_uint32)]


class Texture(C.Structure):
    _fields_ = [("format", C.c_uint32), ("level_count", C.c_uint32),
                ("levels", TextureLevel * MAX_MIP_LEVELS),
                ("mag_filter", C.c_uint32), ("min_filter", C.c_uint32), ("mipmap_mode", C.c_uint32),
                ("address_u", C.c_uint32), ("address_v", C.c_uint32),
                ("mip_lod_bias", C.c_float), ("min_lod", C.c_float), ("max_lod", C.c_float),
                ("border_color", C.c_uint32), ("custom_border_color", C.c_float * 4)]


class StencilOpState(C.Structure):
    _fields_ = [("fail_op", C.c_uint32), ("pass_op", C.c_uint32), ("depth_fail_op", C.c_uint32), ("compare_op", C.c_uint32),
                ("compare_mask", C.c_uint32), ("write_mask", C.c_uint32), ("reference", C.c_uint32), ("reserved", C.c_uint32)]


STENCIL_OP_KEEP, STENCIL_OP_ZERO, STENCIL_OP_REPLACE, STENCIL_OP_INCREMENT_AND_CLAMP = 0, 1, 2, 3
STENCIL_OP_DECREMENT_AND_CLAMP, STENCIL_OP_INVERT, STENCIL_OP_INCREMENT_AND_WRAP, STENCIL_OP_DECREMENT_AND_WRAP = 4, 5, 6, 7


class PipelineState(C.Structure):
    _fields_ = [
        ("topology", C.c_uint32), ("attrib_count", C.c_uint32),
        ("attribs", VertexAttrib * MAX_ATTRIBS), ("bindings", VertexBinding * MAX_ATTRIBS),
        ("vertex_shader", C.c_uint32), ("fragment_shader", C.c_uint32),
        ("mvp", C.c_float * 16),
        ("viewport_x", C.c_float), ("viewport_y", C.c_float),
        ("viewport_width", C.c_float), ("viewport_height", C.c_float),
        ("viewport_min_depth", C.c_float), ("viewport_max_depth", C.c_float),
        ("scissor_x", C.c_int32), ("scissor_y", C.c_int32),
        ("scissor_width", C.c_uint32), ("scissor_height", C.c_uint32),
        ("cull_mode", C.c_uint32), ("front_face", C.c_uint32),
        ("depth_clip_enable", C.c_uint32), ("depth_clamp_enable", C.c_uint32),
        ("depth_bias_constant", C.c_float), ("depth_bias_slope", C.c_float), ("depth_bias_clamp", C.c_float),
        ("depth_test_enable", C.c_uint32), ("depth_write_enable", C.c_uint32), ("depth_compare_op", C.c_uint32),
        ("color_format", C.c_uint32), ("blend_enable", C.c_uint32),
        ("src_color_factor", C.c_uint32), ("dst_color_factor", C.c_uint32), ("color_blend_op", C.c_uint32),
        ("src_alpha_factor", C.c_uint32), ("dst_alpha_factor", C.c_uint32), ("alpha_blend_op", C.c_uint32),
        ("color_write_mask", C.c_uint32), ("sample_count", C.c_uint32),
        ("color", C.c_void_p), ("color_pitch_bytes", C.c_uint32), ("reserved0", C.c_uint32),
        ("color_slice_bytes", C.c_uint64),
        ("depth", C.c_void_p), ("depth_pitch_bytes", C.c_uint32), ("depth_format", C.c_uint32),
        ("depth_slice_bytes", C.c_uint64),
        ("framebuffer_width", C.c_uint32), ("framebuffer_height", C.c_uint32),
        ("texture", Texture),
        ("precision_profile", C.c_uint32), ("provoking_vertex", C.c_uint32),
        ("depth_bounds_test_enable", C.c_uint32), ("min_depth_bounds", C.c_float), ("max_depth_bounds", C.c_float),
        ("stencil_test_enable", C.c_uint32), ("stencil", C.c_void_p), ("stencil_pitch_bytes", C.c_uint32),
        ("reserved3", C.c_uint32), ("stencil_slice_bytes", C.c_uint64),
        ("front", StencilOpState), ("back", StencilOpState),
    ]


class DrawArgs(C.Structure):
    _fields_ = [
        ("count", C.c_uint32), ("base_vertex", C.c_int32), ("first_vertex", C.c_uint32),
        ("index_type", C.c_uint32), ("indices", C.c_void_p), ("vertex_count", C.c_uint32),
        ("instance_id", C.c_int32), ("layer", C.c_int32),
        ("render_area_x", C.c_int32), ("render_area_y", C.c_int32),
        ("render_area_width", C.c_uint32), ("render_area_height", C.c_uint32),
        ("restart_index_count", C.c_uint32), ("raster_wait_event", C.c_void_p),
    ]


class Counters(C.Structure):
    _fields_ = [("triangles_in", C.c_uint64), ("triangles_rejected", C.c_uint64),
                ("triangles_clipped", C.c_uint64), ("triangles_visible", C.c_uint64),
                ("quads", C.c_uint64), ("fragments_tested", C.c_uint64),
                ("fragments_passed", C.c_uint64), ("texture_levels_mask", C.c_uint64),
                ("adjoint_fragments", C.c_uint64), ("adjoint_depth_mismatch", C.c_uint64),
                ("adjoint_list_overflow", C.c_uint64), ("reserved", C.c_uint64)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_ if k != "reserved"}


ADJOINT_MAX_FRAGMENTS_PER_PIXEL = 2048


class AdjointArgs(C.Structure):
    _fields_ = [("grad_color", C.c_void_p), ("grad_color_pitch_bytes", C.c_uint32), ("reserved0", C.c_uint32),
                ("grad_color_slice_bytes", C.c_uint64), ("clear_color", C.c_float * 4), ("clear_depth", C.c_float),
                ("reserved1", C.c_uint32), ("grad_texels", C.c_void_p * MAX_MIP_LEVELS),
                ("grad_vertices", C.c_void_p * MAX_ATTRIBS)]


class RasterConfig(C.Structure):
    """swgb_raster_config: the bin one raster warp owns and depth rejection."""
    _fields_ = [("bin_width", C.c_uint32), ("bin_height", C.c_uint32), ("hiz", C.c_uint32), ("reserved", C.c_uint32)]

    def as_dict(self):
        return {"bin": "%dx%d" % (self.bin_width, self.bin_height), "hiz": int(self.hiz)}


BIN_SHAPES = ((16, 16), (32, 16), (32, 32))
AUTOTUNE_CANDIDATES = 6
AUTOTUNE_DEFAULT_RUNS = 3
AUTOTUNE_MAX_RUNS = 15


class Image(C.Structure):
    """swgb_image: one level and layer of an image in device memory."""
    _fields_ = [("data", C.c_void_p), ("format", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32),
                ("samples", C.c_uint32), ("pitch_bytes", C.c_uint64), ("slice_bytes", C.c_uint64)]


class Rect(C.Structure):
    """swgb_rect (VkRect2D)."""
    _fields_ = [("x", C.c_int32), ("y", C.c_int32), ("width", C.c_uint32), ("height", C.c_uint32)]


class ResolveRegion(C.Structure):
    """swgb_resolve_region (VkImageResolve, 2D)."""
    _fields_ = [("src_x", C.c_int32), ("src_y", C.c_int32), ("dst_x", C.c_int32), ("dst_y", C.c_int32),
                ("width", C.c_uint32), ("height", C.c_uint32)]


class BlitRegion(C.Structure):
    """swgb_blit_region (VkImageBlit, 2D): {x0, y0, x1, y1} per image."""
    _fields_ = [("src", C.c_int32 * 4), ("dst", C.c_int32 * 4)]


# bytes per texel of the formats the Blitter entry points take
TEXEL_BYTES = {FORMAT_R8G8B8A8_UNORM: 4, FORMAT_R8G8B8A8_SRGB: 4, FORMAT_B8G8R8A8_UNORM: 4, FORMAT_B8G8R8A8_SRGB: 4,
               FORMAT_R16G16B16A16_SFLOAT: 8, FORMAT_R32G32B32A32_SFLOAT: 16, FORMAT_D32_SFLOAT: 4,
               FORMAT_D16_UNORM: 2, FORMAT_S8_UINT: 1}
