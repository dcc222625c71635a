"""Seeded synthetic scenes for the five draw workloads the path is measured on.

Every generator is deterministic: ``seed = 0x53570000 + workload index`` feeds
numpy's PCG64 generator.  A scene is host data only (numpy arrays plus pipeline
state values); ``Renderer`` uploads it, and the tests hand the same arrays to
the CPU oracle.

Vertex layout (AoS, 40 bytes): position R32G32B32A32_SFLOAT at 0, colour
R32G32B32A32_SFLOAT at 16, uv R32G32_SFLOAT at 32.
"""
from dataclasses import dataclass, field
import math

import ctypes

import numpy as np

from . import abi

SEED_BASE = 0x53570000
VERTEX_FLOATS = 10
VERTEX_STRIDE = VERTEX_FLOATS * 4


@dataclass
class Scene:
    name: str
    width: int
    height: int
    vertices: np.ndarray              # float32 [N, 10]
    indices: np.ndarray = None        # uint8/uint16/uint32 index buffer or None (non-indexed)
    tri_count: int = 0
    mvp: np.ndarray = None            # float32 [4, 4] row-major math matrix
    fragment_shader: int = abi.FS_VCOLOR
    texture_levels: list = field(default_factory=list)  # [h, w, 4] per level (uint8 / float16 / float32)
    texture_format: int = abi.FORMAT_R8G8B8A8_UNORM
    sampler: dict = field(default_factory=dict)
    blend: tuple = None               # (srcC, dstC, opC, srcA, dstA, opA) or None
    cull_mode: int = abi.CULL_NONE
    front_face: int = abi.FRONT_FACE_CCW
    depth_compare: int = abi.COMPARE_LESS
    clear_color: tuple = (0, 0, 0, 0)
    clear_depth: float = 1.0
    color_format: int = abi.FORMAT_R8G8B8A8_UNORM
    viewport: tuple = None            # (x, y, w, h) default full framebuffer
    scissor: tuple = None             # (x, y, w, h)
    samples: int = 1                  # 1 or 4 (4x MSAA: one plane per sample)
    topology: int = abi.TOPOLOGY_TRIANGLE_LIST
    first_vertex: int = 0
    base_vertex: int = 0
    provoking_vertex: int = 0         # 0 = FIRST_VERTEX, 1 = LAST_VERTEX (VK_EXT_provoking_vertex)
    depth_format: int = abi.FORMAT_D32_SFLOAT  # or FORMAT_D16_UNORM
    color_write_mask: int = 0xF       # VkColorComponentFlags
    depth_bias: tuple = (0.0, 0.0, 0.0)     # (constant, slope, clamp)
    depth_bounds: tuple = None        # (min, max) enables the depth bounds test
    depth_test: bool = True
    # stencil: {"front": (fail, pass, depth_fail, compare, compare_mask, write_mask, reference),
    #           "back": (...), "clear": value} on an S8_UINT attachment, or None
    stencil: dict = None
    restart_index_count: int = 0      # > 0: primitive restart over this many indices (tri_count ignored)

    @property
    def vertex_count(self):
        return int(self.vertices.shape[0])

    def mvp_column_major(self):
        m = np.eye(4, dtype=np.float32) if self.mvp is None else np.asarray(self.mvp, np.float32)
        return m.T.reshape(-1).copy()


def _rng(index):
    return np.random.Generator(np.random.PCG64(SEED_BASE + index))


def random_triangles(rng, n, textured=False):
    """n independent triangles, uniform in clip space: x,y in [-1,1],
    z in [0.1,0.9], w = 1; RGBA uniform in [0,1]; uv uniform in [0,1]."""
    v = np.zeros((3 * n, VERTEX_FLOATS), np.float32)
    v[:, 0:2] = rng.uniform(-1.0, 1.0, (3 * n, 2))
    v[:, 2] = rng.uniform(0.1, 0.9, 3 * n)
    v[:, 3] = 1.0
    v[:, 4:8] = rng.uniform(0.0, 1.0, (3 * n, 4))
    if textured:
        v[:, 8:10] = rng.uniform(0.0, 1.0, (3 * n, 2))
    return v


def box_mip_chain(level0):
    """Full box-filtered mip chain of an RGBA8 image (rounded average of 2x2)."""
    levels = [np.ascontiguousarray(level0)]
    cur = level0.astype(np.uint32)
    while cur.shape[0] > 1 or cur.shape[1] > 1:
        h, w = cur.shape[:2]
        h2, w2 = max(1, h // 2), max(1, w // 2)
        if h > 1 and w > 1:
            s = cur[0:2 * h2:2, 0:2 * w2:2] + cur[1:2 * h2:2, 0:2 * w2:2] + cur[0:2 * h2:2, 1:2 * w2:2] + cur[1:2 * h2:2, 1:2 * w2:2]
            cur = (s + 2) // 4
        elif h > 1:
            cur = (cur[0:2 * h2:2] + cur[1:2 * h2:2] + 1) // 2
        else:
            cur = (cur[:, 0:2 * w2:2] + cur[:, 1:2 * w2:2] + 1) // 2
        levels.append(np.ascontiguousarray(cur.astype(np.uint8)))
    return levels


def perspective_vk(fovy_deg, aspect, near, far):
    """Vulkan clip space (y down, depth [0,1]) perspective matrix."""
    f = 1.0 / math.tan(math.radians(fovy_deg) / 2.0)
    return np.array([[f / aspect, 0, 0, 0],
                     [0, -f, 0, 0],
                     [0, 0, far / (near - far), near * far / (near - far)],
                     [0, 0, -1, 0]], np.float64)


def translate(x, y, z):
    m = np.eye(4)
    m[:3, 3] = (x, y, z)
    return m


def scene_small(n_tris=1000, width=256, height=256, seed_index=0):
    """Plain forward, small: independent Gouraud triangles, identity MVP,
    RGBA8 + D32F, depth LESS, no blending, no texture."""
    rng = _rng(seed_index)
    return Scene(name="tris%d_%dx%d" % (n_tris, width, height), width=width, height=height,
                 vertices=random_triangles(rng, n_tris), tri_count=n_tris,
                 fragment_shader=abi.FS_VCOLOR, clear_color=(0, 0, 0, 0), clear_depth=1.0)


def scene_heightfield(quads_x=1000, quads_y=500, width=1920, height=1080, tex_size=2048, seed_index=1):
    """Plain forward, large textured: a (quads_x x quads_y)-quad height-field
    grid (2 triangles per quad, uint32 indices), heights uniform in [0,0.2],
    perspective fov 60 deg, near 0.1, far 100, camera 2 units back.  UVs span
    [0,4]^2 with REPEAT; tex_size^2 RGBA8 uniform texels with a box-filtered mip
    chain, trilinear; colour = texel * vertex colour; depth LESS; blend
    SRC_ALPHA / ONE_MINUS_SRC_ALPHA with vertex alpha in [0.5,1]."""
    rng = _rng(seed_index)
    nx, ny = quads_x + 1, quads_y + 1
    aspect = width / height
    half_h = 2.0 * math.tan(math.radians(30.0)) * 1.08   # slightly wider than the view: edges get clipped
    half_w = half_h * aspect
    gx = np.linspace(-half_w, half_w, nx, dtype=np.float64)
    gy = np.linspace(-half_h, half_h, ny, dtype=np.float64)
    X, Y = np.meshgrid(gx, gy)
    Z = rng.uniform(0.0, 0.2, (ny, nx))
    v = np.zeros((ny * nx, VERTEX_FLOATS), np.float32)
    v[:, 0] = X.reshape(-1)
    v[:, 1] = Y.reshape(-1)
    v[:, 2] = Z.reshape(-1)
    v[:, 3] = 1.0
    v[:, 4:7] = rng.uniform(0.0, 1.0, (ny * nx, 3))
    v[:, 7] = rng.uniform(0.5, 1.0, ny * nx)
    U, V = np.meshgrid(np.linspace(0.0, 4.0, nx), np.linspace(0.0, 4.0, ny))
    v[:, 8] = U.reshape(-1)
    v[:, 9] = V.reshape(-1)
    # indices: quad (i, j) -> (a, b, c), (c, b, d) with a=(j,i) b=(j,i+1) c=(j+1,i) d=(j+1,i+1)
    j, i = np.meshgrid(np.arange(quads_y, dtype=np.uint32), np.arange(quads_x, dtype=np.uint32), indexing="ij")
    a = (j * nx + i).reshape(-1)
    b = a + 1
    c = a + nx
    d = c + 1
    idx = np.stack([a, b, c, c, b, d], axis=1).reshape(-1).astype(np.uint32)
    tex0 = rng.integers(0, 256, (tex_size, tex_size, 4), dtype=np.uint8)
    mvp = perspective_vk(60.0, aspect, 0.1, 100.0) @ translate(0.0, 0.0, -2.0)
    return Scene(name="heightfield%dk_%dx%d" % (len(idx) // 3 // 1000, width, height),
                 width=width, height=height, vertices=v, indices=idx, tri_count=len(idx) // 3,
                 mvp=mvp.astype(np.float32), fragment_shader=abi.FS_TEX_X_VCOLOR,
                 texture_levels=box_mip_chain(tex0),
                 sampler=dict(mag_filter=abi.FILTER_LINEAR, min_filter=abi.FILTER_LINEAR,
                              mipmap_mode=abi.MIPMAP_MODE_LINEAR, address_u=abi.ADDRESS_REPEAT,
                              address_v=abi.ADDRESS_REPEAT, mip_lod_bias=0.0, min_lod=0.0, max_lod=1000.0),
                 blend=(abi.BLEND_SRC_ALPHA, abi.BLEND_ONE_MINUS_SRC_ALPHA, abi.BLEND_OP_ADD,
                        abi.BLEND_SRC_ALPHA, abi.BLEND_ONE_MINUS_SRC_ALPHA, abi.BLEND_OP_ADD),
                 clear_color=(26, 51, 77, 255), clear_depth=1.0)


def scene_textured_small(n_tris=200, width=128, height=96, tex_size=64, mip=True, address=abi.ADDRESS_REPEAT,
                         blend=True, seed_index=5):
    """Small textured case for parity tests: random triangles with uv in
    [-1.5, 2.5] so wrap/clamp addressing is exercised, optional mips/blend."""
    rng = _rng(seed_index)
    v = random_triangles(rng, n_tris, textured=True)
    v[:, 8:10] = rng.uniform(-1.5, 2.5, (3 * n_tris, 2))
    v[:, 7] = rng.uniform(0.3, 1.0, 3 * n_tris)
    tex0 = rng.integers(0, 256, (tex_size, tex_size, 4), dtype=np.uint8)
    levels = box_mip_chain(tex0) if mip else [tex0]
    s = Scene(name="textured%d" % n_tris, width=width, height=height, vertices=v, tri_count=n_tris,
              fragment_shader=abi.FS_TEX_X_VCOLOR, texture_levels=levels,
              sampler=dict(mag_filter=abi.FILTER_LINEAR, min_filter=abi.FILTER_LINEAR,
                           mipmap_mode=abi.MIPMAP_MODE_LINEAR if mip else abi.MIPMAP_MODE_NEAREST,
                           address_u=address, address_v=address, mip_lod_bias=0.0, min_lod=0.0,
                           max_lod=1000.0),
              clear_color=(10, 20, 30, 40))
    if blend:
        s.blend = (abi.BLEND_SRC_ALPHA, abi.BLEND_ONE_MINUS_SRC_ALPHA, abi.BLEND_OP_ADD,
                   abi.BLEND_SRC_ALPHA, abi.BLEND_ONE_MINUS_SRC_ALPHA, abi.BLEND_OP_ADD)
    return s


def uv_sphere(rng, seg_u, seg_v, radius=1.0, noise_sigma=0.0):
    """Vertices and uint32 indices of a uv-sphere with seg_u x seg_v quads
    (2 triangles each, the pole rows degenerate), optional radial Gaussian
    displacement per point of the sphere, uv = (u, v) in [0,1]^2, RGBA
    uniform in [0,1]."""
    nu, nv = seg_u + 1, seg_v + 1
    th = np.linspace(0.0, 2.0 * math.pi, nu)
    ph = np.linspace(0.0, math.pi, nv)
    TH, PH = np.meshgrid(th, ph)
    noise = 0.0
    if noise_sigma > 0:
        # one displacement per point of the sphere: the seam column repeats
        # column 0 and each pole row is one point, so the mesh stays closed
        noise = rng.normal(0.0, noise_sigma, TH.shape)
        noise[:, -1] = noise[:, 0]
        noise[0, :] = noise[0, 0]
        noise[-1, :] = noise[-1, 0]
    r = radius * (1.0 + noise)
    x = r * np.sin(PH) * np.cos(TH)
    y = r * np.cos(PH)
    z = r * np.sin(PH) * np.sin(TH)
    v = np.zeros((nu * nv, VERTEX_FLOATS), np.float32)
    v[:, 0], v[:, 1], v[:, 2], v[:, 3] = x.reshape(-1), y.reshape(-1), z.reshape(-1), 1.0
    v[:, 4:8] = rng.uniform(0.0, 1.0, (nu * nv, 4))
    U, V = np.meshgrid(np.linspace(0.0, 1.0, nu), np.linspace(0.0, 1.0, nv))
    v[:, 8], v[:, 9] = U.reshape(-1), V.reshape(-1)
    j, i = np.meshgrid(np.arange(seg_v, dtype=np.uint32), np.arange(seg_u, dtype=np.uint32), indexing="ij")
    a = (j * nu + i).reshape(-1)
    b, c = a + 1, a + nu
    d = c + 1
    idx = np.stack([a, c, b, b, c, d], axis=1).reshape(-1).astype(np.uint32)
    return v, idx


def look_at(eye, target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0)):
    eye, target, up = (np.asarray(a, np.float64) for a in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    if abs(np.dot(f, up)) > 0.99:
        up = np.array([1.0, 0.0, 0.0])
    sd = np.cross(f, up)
    sd /= np.linalg.norm(sd)
    u = np.cross(sd, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = sd, u, -f
    m[:3, 3] = -m[:3, :3] @ eye
    return m


def scene_sphere_fp32(seg=100, width=512, height=512, tex_size=1024, seed_index=3, texels=None):
    """Adjoint workload, forward part: a seg x seg uv-sphere (~2*seg^2
    triangles) under a fixed perspective MVP, RGBA32F texture uniform in [0,1]
    sampled bilinearly with CLAMP (the fp32 SamplerCore path), FP32 vertex
    colours, colour = texel * vertex colour, RGBA32F attachment, depth LESS."""
    rng = _rng(seed_index)
    v, idx = uv_sphere(rng, seg, seg)
    tex = texels if texels is not None else rng.uniform(0.0, 1.0, (tex_size, tex_size, 4)).astype(np.float32)
    mvp = perspective_vk(45.0, width / height, 0.1, 100.0) @ look_at((0.4, 0.6, 3.0))
    return Scene(name="sphere%d_fp32_%dx%d" % (len(idx) // 3, width, height), width=width, height=height,
                 vertices=v, indices=idx, tri_count=len(idx) // 3, mvp=mvp.astype(np.float32),
                 fragment_shader=abi.FS_TEX_X_VCOLOR, texture_levels=[np.ascontiguousarray(tex)],
                 texture_format=abi.FORMAT_R32G32B32A32_SFLOAT,
                 sampler=dict(mag_filter=abi.FILTER_LINEAR, min_filter=abi.FILTER_LINEAR,
                              mipmap_mode=abi.MIPMAP_MODE_NEAREST, address_u=abi.ADDRESS_CLAMP_TO_EDGE,
                              address_v=abi.ADDRESS_CLAMP_TO_EDGE, mip_lod_bias=0.0, min_lod=0.0, max_lod=0.0),
                 color_format=abi.FORMAT_R32G32B32A32_SFLOAT, clear_color=(0.0, 0.0, 0.0, 0.0))


def float_mip_chain(level0, dtype):
    """Box-filtered chain of a float image (averaged in float64, stored as dtype)."""
    levels = [np.ascontiguousarray(level0.astype(dtype))]
    cur = level0.astype(np.float64)
    while cur.shape[0] > 1 or cur.shape[1] > 1:
        h, w = cur.shape[:2]
        if h > 1:
            cur = 0.5 * (cur[0:h // 2 * 2:2] + cur[1:h // 2 * 2:2])
        if w > 1:
            cur = 0.5 * (cur[:, 0:w // 2 * 2:2] + cur[:, 1:w // 2 * 2:2])
        levels.append(np.ascontiguousarray(cur.astype(dtype)))
    return levels


def scene_sphere_views(view, n_views=256, seg_u=250, seg_v=200, width=512, height=512, tex_size=2048,
                       seed_index=4, mesh=None, levels=None):
    """Batched-adjoint workload, one view: a ~100k-triangle sphere with radial
    N(0, 0.02^2) displacement seen from camera 'view' of n_views placed
    uniformly on a radius-3 sphere; RGBA16F mipmapped texture, trilinear;
    premultiplied-alpha OVER (ONE, ONE_MINUS_SRC_ALPHA) into RGBA16F."""
    rng = _rng(seed_index)
    if mesh is None:
        mesh = uv_sphere(rng, seg_u, seg_v, noise_sigma=0.02)
    v, idx = mesh
    if levels is None:
        tex0 = rng.uniform(0.0, 1.0, (tex_size, tex_size, 4))
        levels = float_mip_chain(tex0, np.float16)
    crng = np.random.Generator(np.random.PCG64(SEED_BASE + 0x100 + seed_index))
    dirs = crng.normal(0.0, 1.0, (n_views, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    eye = 3.0 * dirs[view]
    mvp = perspective_vk(45.0, width / height, 0.1, 100.0) @ look_at(eye)
    return Scene(name="spherenoise%d_view%d" % (len(idx) // 3, view), width=width, height=height, vertices=v,
                 indices=idx, tri_count=len(idx) // 3, mvp=mvp.astype(np.float32),
                 fragment_shader=abi.FS_TEX_X_VCOLOR, texture_levels=levels,
                 texture_format=abi.FORMAT_R16G16B16A16_SFLOAT,
                 sampler=dict(mag_filter=abi.FILTER_LINEAR, min_filter=abi.FILTER_LINEAR,
                              mipmap_mode=abi.MIPMAP_MODE_LINEAR, address_u=abi.ADDRESS_REPEAT,
                              address_v=abi.ADDRESS_CLAMP_TO_EDGE, mip_lod_bias=0.0, min_lod=0.0, max_lod=1000.0),
                 blend=(abi.BLEND_ONE, abi.BLEND_ONE_MINUS_SRC_ALPHA, abi.BLEND_OP_ADD,
                        abi.BLEND_ONE, abi.BLEND_ONE_MINUS_SRC_ALPHA, abi.BLEND_OP_ADD),
                 color_format=abi.FORMAT_R16G16B16A16_SFLOAT, clear_color=(0.0, 0.0, 0.0, 0.0))


def build_state(scene, color_ptr, depth_ptr, vertex_ptr, level_ptrs=None, color_pitch=None, depth_pitch=None, stencil_ptr=None):
    """PipelineState for a scene given buffer addresses (device pointers for
    the GB300 path, host pointers for the oracle)."""
    st = abi.PipelineState()
    st.topology = scene.topology
    st.provoking_vertex = scene.provoking_vertex
    st.attrib_count = 3
    st.attribs[0] = abi.VertexAttrib(abi.FORMAT_R32G32B32A32_SFLOAT, 0, 0, 0)
    st.attribs[1] = abi.VertexAttrib(abi.FORMAT_R32G32B32A32_SFLOAT, 0, 16, 0)
    st.attribs[2] = abi.VertexAttrib(abi.FORMAT_R32G32_SFLOAT, 0, 32, 0)
    st.bindings[0] = abi.VertexBinding(vertex_ptr, VERTEX_STRIDE, 0)
    st.vertex_shader = abi.VS_MVP_PASSTHROUGH
    st.fragment_shader = scene.fragment_shader
    for k, val in enumerate(scene.mvp_column_major()):
        st.mvp[k] = float(val)
    vx, vy, vw, vh = scene.viewport or (0, 0, scene.width, scene.height)
    st.viewport_x, st.viewport_y, st.viewport_width, st.viewport_height = float(vx), float(vy), float(vw), float(vh)
    st.viewport_min_depth, st.viewport_max_depth = 0.0, 1.0
    sx, sy, sw, sh = scene.scissor or (0, 0, scene.width, scene.height)
    st.scissor_x, st.scissor_y, st.scissor_width, st.scissor_height = sx, sy, sw, sh
    st.cull_mode = scene.cull_mode
    st.front_face = scene.front_face
    st.depth_clip_enable = 1
    st.depth_test_enable = 1 if scene.depth_test else 0
    st.depth_write_enable = 1
    st.depth_bias_constant, st.depth_bias_slope, st.depth_bias_clamp = (float(x) for x in scene.depth_bias)
    if scene.depth_bounds is not None:
        st.depth_bounds_test_enable = 1
        st.min_depth_bounds, st.max_depth_bounds = (float(x) for x in scene.depth_bounds)
    if scene.stencil is not None:
        st.stencil_test_enable = 1
        st.stencil = stencil_ptr
        st.stencil_pitch_bytes = scene.width
        st.stencil_slice_bytes = scene.width * scene.height
        for face in ("front", "back"):
            v = scene.stencil[face]
            setattr(st, face, abi.StencilOpState(*(int(x) for x in v), 0))
    st.depth_compare_op = scene.depth_compare
    st.color_format = scene.color_format
    if scene.blend is not None:
        st.blend_enable = 1
        (st.src_color_factor, st.dst_color_factor, st.color_blend_op,
         st.src_alpha_factor, st.dst_alpha_factor, st.alpha_blend_op) = scene.blend
    st.color_write_mask = scene.color_write_mask
    st.sample_count = scene.samples
    bpp = {abi.FORMAT_R8G8B8A8_UNORM: 4, abi.FORMAT_B8G8R8A8_UNORM: 4, abi.FORMAT_R8G8B8A8_SRGB: 4,
           abi.FORMAT_B8G8R8A8_SRGB: 4, abi.FORMAT_R16G16B16A16_SFLOAT: 8,
           abi.FORMAT_R32G32B32A32_SFLOAT: 16}[scene.color_format]
    st.color = color_ptr
    st.color_pitch_bytes = color_pitch or scene.width * bpp
    st.color_slice_bytes = st.color_pitch_bytes * scene.height
    st.depth = depth_ptr
    st.depth_format = scene.depth_format
    st.depth_pitch_bytes = depth_pitch or scene.width * (2 if scene.depth_format == abi.FORMAT_D16_UNORM else 4)
    st.depth_slice_bytes = st.depth_pitch_bytes * scene.height
    st.framebuffer_width, st.framebuffer_height = scene.width, scene.height
    if scene.fragment_shader == abi.FS_TEX_X_VCOLOR:
        t = st.texture
        t.format = scene.texture_format
        t.level_count = len(scene.texture_levels)
        for i, lv in enumerate(scene.texture_levels):
            t.levels[i] = abi.TextureLevel(level_ptrs[i], lv.shape[1], lv.shape[0], lv.shape[1], 0)
        for k, val in scene.sampler.items():
            if k == "custom_border_color":
                val = (ctypes.c_float * 4)(*val)
            setattr(t, k, val)
    st.precision_profile = abi.PRECISION_CMAKE
    return st


INDEX_TYPES = {np.dtype(np.uint8): abi.INDEX_TYPE_UINT8, np.dtype(np.uint16): abi.INDEX_TYPE_UINT16,
               np.dtype(np.uint32): abi.INDEX_TYPE_UINT32}


def build_args(scene, index_ptr=None):
    a = abi.DrawArgs()
    a.count = scene.tri_count
    a.base_vertex = scene.base_vertex
    a.first_vertex = scene.first_vertex
    if scene.indices is None:
        a.index_type = abi.INDEX_TYPE_NONE
        a.indices = None
    else:
        a.index_type = INDEX_TYPES[np.asarray(scene.indices).dtype]
        a.indices = index_ptr
    a.vertex_count = scene.vertex_count
    a.restart_index_count = scene.restart_index_count
    a.render_area_x, a.render_area_y = 0, 0
    a.render_area_width, a.render_area_height = scene.width, scene.height
    return a


def index_bytes(scene):
    """The scene's index buffer as raw bytes (uint8 array), any index type."""
    return np.ascontiguousarray(scene.indices).view(np.uint8)


def strip_fan_scene(topology, n_tris=300, width=96, height=80, indexed=None, seed_index=50):
    """Random clip-space triangles (as scene_small) assembled as a triangle
    strip or fan over n_tris + 2 vertices; indexed with a shuffled index
    buffer of the given dtype (uint8 / uint16 / uint32) or non-indexed."""
    rng = _rng(seed_index)
    nv = n_tris + 2
    v = random_triangles(rng, (nv + 2) // 3)[:nv]
    if topology == abi.TOPOLOGY_TRIANGLE_FAN:
        v[0, 0:3] = (0.0, 0.0, 0.5)  # fan centre inside the frame
    indices = None
    if indexed is not None:
        perm = rng.permutation(nv)
        verts = np.empty_like(v)
        verts[perm] = v
        v = verts
        indices = perm.astype(indexed)
    return Scene(name="topo%d_%d_%s" % (topology, n_tris, "none" if indexed is None else np.dtype(indexed).name),
                 width=width, height=height, vertices=v, indices=indices, tri_count=n_tris, topology=topology,
                 cull_mode=abi.CULL_BACK)


def restart_scene(topology, n_indices=600, width=96, height=80, dtype=np.uint16, restart_every=(1, 40), seed_index=51):
    """Primitive restart: an index stream of n_indices entries over random
    clip-space vertices (as scene_small), cut by all-ones restart indices at
    random gaps in [restart_every] -- including back-to-back restarts, a leading
    one and segments too short to hold a triangle; back faces culled."""
    rng = _rng(seed_index)
    nv = min(n_indices, int(np.iinfo(dtype).max))  # all-ones stays free for restart
    v = random_triangles(rng, (nv + 2) // 3)[:nv]
    if topology == abi.TOPOLOGY_TRIANGLE_FAN:
        v[:, 0:2] *= 0.6
    idx = rng.integers(0, nv, n_indices).astype(np.int64)
    restart = np.iinfo(dtype).max
    pos = 0
    while pos < n_indices:
        idx[pos] = restart
        pos += int(rng.integers(restart_every[0], restart_every[1] + 1))
    idx[-3:] = restart if n_indices > 8 else idx[-3:]
    idx[0] = restart
    return Scene(name="restart%d_%d_%s" % (topology, n_indices, np.dtype(dtype).name), width=width, height=height,
                 vertices=v, indices=idx.astype(dtype), tri_count=0, topology=topology, cull_mode=abi.CULL_BACK,
                 restart_index_count=n_indices)


def attachment_shapes(scene):
    """Colour and depth array shapes: (h, w, 4) / (h, w), or with 4x MSAA one
    plane per sample in front, (4, h, w, 4) / (4, h, w)."""
    lead = (scene.samples,) if scene.samples > 1 else ()
    return lead + (scene.height, scene.width, 4), lead + (scene.height, scene.width)


def color_dtype(scene):
    return {abi.FORMAT_R8G8B8A8_UNORM: np.uint8, abi.FORMAT_B8G8R8A8_UNORM: np.uint8, abi.FORMAT_R8G8B8A8_SRGB: np.uint8,
            abi.FORMAT_B8G8R8A8_SRGB: np.uint8, abi.FORMAT_R32G32B32A32_SFLOAT: np.float32,
            abi.FORMAT_R16G16B16A16_SFLOAT: np.float16}[scene.color_format]


def depth_dtype(scene):
    return np.uint16 if scene.depth_format == abi.FORMAT_D16_UNORM else np.float32


def depth_clear_value(scene):
    """The stored clear depth: the float, or for D16_UNORM its 16-bit unorm
    (round to nearest, as a depth clear converts it)."""
    if scene.depth_format == abi.FORMAT_D16_UNORM:
        return np.uint16(int(np.rint(np.float32(scene.clear_depth) * np.float32(65535.0))))
    return np.float32(scene.clear_depth)


def stencil_buffer(scene):
    """The scene's S8_UINT stencil attachment on the host, cleared (None without stencil)."""
    if scene.stencil is None:
        return None
    _, ds = attachment_shapes(scene)
    return np.full(ds, scene.stencil.get("clear", 0), np.uint8)


def clear_buffers(scene):
    """Host colour (uint8/float) and depth (float32 / uint16) attachments, cleared."""
    cs, ds = attachment_shapes(scene)
    color = np.empty(cs, color_dtype(scene))
    color[...] = np.asarray(scene.clear_color, color.dtype)
    depth = np.full(ds, depth_clear_value(scene), depth_dtype(scene))
    return color, depth


def shelf_pack(sides, page_size):
    """Shelf-pack squares into pages of page_size x page_size, tallest first.
    Returns (page, x, y) per input square, in input order."""
    sides = np.asarray(sides, np.int64)
    order = np.argsort(-sides, kind="stable")
    out = np.zeros((len(sides), 3), np.int64)
    page, x, y, shelf_h = 0, 0, 0, 0
    for i in order:
        s = int(sides[i])
        if s > page_size:
            raise ValueError("viewport %d larger than the atlas page %d" % (s, page_size))
        if x + s > page_size:
            x, y, shelf_h = 0, y + shelf_h, 0
        if y + s > page_size:
            page, x, y, shelf_h = page + 1, 0, 0, 0
        out[i] = (page, x, y)
        x += s
        shelf_h = max(shelf_h, s)
    return out


@dataclass
class BatchScene:
    """Independent draws into disjoint viewports of an atlas (one or more
    square pages of RGBA8 + D32F).  Draw i renders vertices
    [vstart[i], vstart[i] + 3 * tris[i]) with texture textures[i] into the
    side[i] x side[i] square at (x, y) of page `page`."""
    name: str
    tris: np.ndarray          # int64 [n]
    sides: np.ndarray         # int64 [n]
    place: np.ndarray         # int64 [n, 3]: page, x, y
    vertices: np.ndarray      # float32 [3 * sum(tris), 10]
    vstart: np.ndarray        # int64 [n]
    textures: np.ndarray      # uint8 [n, T, T, 4]
    page_size: int
    pages: int
    sampler: dict = field(default_factory=dict)
    clear_color: tuple = (0, 0, 0, 0)
    clear_depth: float = 1.0

    @property
    def n(self):
        return len(self.tris)

    def subset(self, idx):
        """The draws idx (ascending) of this batch, keeping their atlas places."""
        idx = np.asarray(idx, np.int64)
        tris = self.tris[idx]
        verts = np.concatenate([self.vertices[self.vstart[i]:self.vstart[i] + 3 * self.tris[i]] for i in idx]) \
            if len(idx) else self.vertices[:0]
        vstart = np.concatenate([[0], np.cumsum(3 * tris)[:-1]]).astype(np.int64) if len(idx) else tris
        return BatchScene(name="%s_part%d" % (self.name, len(idx)), tris=tris, sides=self.sides[idx], place=self.place[idx],
                          vertices=verts, vstart=vstart, textures=self.textures[idx], page_size=self.page_size,
                          pages=self.pages, sampler=dict(self.sampler), clear_color=self.clear_color,
                          clear_depth=self.clear_depth)

    def draw_scene(self, i):
        """Draw i as a stand-alone Scene (its own side x side framebuffer)."""
        s = int(self.sides[i])
        v0 = int(self.vstart[i])
        return Scene(name="%s_draw%d" % (self.name, i), width=s, height=s,
                     vertices=self.vertices[v0:v0 + 3 * int(self.tris[i])], tri_count=int(self.tris[i]),
                     fragment_shader=abi.FS_TEX_X_VCOLOR, texture_levels=[self.textures[i]],
                     sampler=dict(self.sampler), clear_color=self.clear_color, clear_depth=self.clear_depth)


def _batch_sizes(rng, n_draws, tri_min, tri_max, sides):
    tris = np.rint(np.exp(rng.uniform(math.log(tri_min), math.log(tri_max), n_draws))).astype(np.int64)
    tris = np.clip(tris, tri_min, tri_max)
    side = rng.choice(np.asarray(sides, np.int64), n_draws)
    return tris, side


def batch_draw_sizes(n_draws=4096, tri_min=16, tri_max=65536, sides=(128, 256, 384, 512), seed_index=2):
    """Triangle counts and viewport sides of scene_batch's draws (same seed,
    no vertex data)."""
    return _batch_sizes(_rng(seed_index), n_draws, tri_min, tri_max, sides)


def scene_batch(n_draws=4096, tri_min=16, tri_max=65536, sides=(128, 256, 384, 512), page_size=16384,
                tex_size=256, seed_index=2):
    """Batched forward: n_draws independent draws, triangle counts
    log-uniform in [tri_min, tri_max] (rounded), square viewports with side
    uniform in `sides`, shelf-packed into page_size^2 RGBA8 + D32F atlas
    pages; triangles uniform in clip space as in scene_small; each draw
    samples its own tex_size^2 RGBA8 texture bilinearly (one level)."""
    rng = _rng(seed_index)
    tris, side = _batch_sizes(rng, n_draws, tri_min, tri_max, sides)
    place = shelf_pack(side, page_size)
    vertices = random_triangles(rng, int(tris.sum()), textured=True)
    vstart = np.concatenate([[0], np.cumsum(3 * tris)[:-1]]).astype(np.int64)
    textures = rng.integers(0, 256, (n_draws, tex_size, tex_size, 4), dtype=np.uint8)
    sampler = dict(mag_filter=abi.FILTER_LINEAR, min_filter=abi.FILTER_LINEAR, mipmap_mode=abi.MIPMAP_MODE_NEAREST,
                   address_u=abi.ADDRESS_REPEAT, address_v=abi.ADDRESS_REPEAT, mip_lod_bias=0.0, min_lod=0.0, max_lod=0.0)
    return BatchScene(name="batch%d_tris%d-%d_page%d" % (n_draws, tri_min, tri_max, page_size), tris=tris, sides=side,
                      place=place, vertices=vertices, vstart=vstart, textures=textures, page_size=page_size,
                      pages=int(place[:, 0].max()) + 1, sampler=sampler)
