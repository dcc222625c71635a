"""Differentiable draws: torch.autograd.Function over the C-ABI.

``render(renderer, scene, vertices, levels)`` draws ``scene`` with the given
vertex buffer (float32 [N, 10]: position, colour, uv) and texture levels
(float32 [h, w, 4] each) through swgb_draw and returns the colour attachment
as float32 ([H, W, 4], or [4, H, W, 4] with 4x MSAA).  Its backward pass calls
swgb_draw_adjoint (include/swgb.h), which holds visibility fixed and returns
dL/dvertices and dL/dlevels.

``render_views(renderer, scenes, vertices, levels)`` does the same for several
views of one mesh and texture (each scene its own camera and attachment): the
forward is one swgb_draw_batch call, the backward one swgb_draw_adjoint_batch
call, and gradients of all views accumulate into one vertex and one texture
gradient.

Both switch the renderer to torch's current stream, so the draws are ordered
with the surrounding torch work.

There is no CPU path: every call goes through libswgb.so on the device.
"""
import numpy as np
import torch

from . import abi, scenes


def _texture_dtype(scene):
    return torch.float16 if scene.texture_format == abi.FORMAT_R16G16B16A16_SFLOAT else torch.float32


class _View:
    """Device attachments and C-ABI state of one scene drawn with given
    vertex and texture tensors."""

    def __init__(self, scene, vertices, tex_levels, index_cache):
        dev = vertices.device
        cdtype = {abi.FORMAT_R32G32B32A32_SFLOAT: torch.float32, abi.FORMAT_R16G16B16A16_SFLOAT: torch.float16}.get(
            scene.color_format)
        if cdtype is None:
            raise ValueError("differentiable draws need a float colour attachment")
        cshape, dshape = scenes.attachment_shapes(scene)
        self.scene = scene
        self.color = torch.empty(cshape, dtype=cdtype, device=dev)
        self.color[...] = torch.tensor(scene.clear_color, dtype=cdtype, device=dev)
        self.depth = torch.full(dshape, scene.clear_depth, dtype=torch.float32, device=dev)
        self.state = scenes.build_state(scene, self.color.data_ptr(), self.depth.data_ptr(), vertices.data_ptr(),
                                        [l.data_ptr() for l in tex_levels])
        self.indices = None
        if scene.indices is not None:
            key = id(scene.indices)
            if key not in index_cache:  # views of one mesh share its index buffer
                index_cache[key] = torch.from_numpy(scenes.index_bytes(scene)).to(dev)
            self.indices = index_cache[key]
        self.args = scenes.build_args(scene, None if self.indices is None else self.indices.data_ptr())

    def adjoint_args(self, grad_color, grad_vertices, grad_levels):
        a = abi.AdjointArgs()
        a.grad_color = grad_color.data_ptr()
        W, H = self.scene.width, self.scene.height
        a.grad_color_pitch_bytes = W * 16
        a.grad_color_slice_bytes = W * H * 16
        for k in range(4):
            a.clear_color[k] = float(self.scene.clear_color[k])
        a.clear_depth = float(self.scene.clear_depth)
        for i, g in enumerate(grad_levels):
            a.grad_texels[i] = g.data_ptr()
        a.grad_vertices[0] = grad_vertices.data_ptr()
        return a


def _check_inputs(vertices, levels):
    if (not vertices.is_cuda or vertices.dtype != torch.float32 or vertices.dim() != 2
            or vertices.shape[1] != scenes.VERTEX_FLOATS):
        raise ValueError("vertices: float32 CUDA tensor [N, %d]" % scenes.VERTEX_FLOATS)
    for l in levels:
        if not l.is_cuda or l.dtype != torch.float32 or l.dim() != 3 or l.shape[2] != 4:
            raise ValueError("texture levels: float32 CUDA tensors [h, w, 4]")


class DrawSet:
    """Draws of one mesh and texture into one attachment pair per scene (one
    scene per view), set up once for repeated forward and adjoint calls:
    ``forward`` clears the attachments and enqueues the draws (one
    swgb_draw_batch call for several views); ``adjoint`` zeroes the gradient
    buffers and enqueues swgb_draw_adjoint(_batch) for dL/dcolour
    ``grad_color`` (float32, [V, (4,) H, W, 4])."""

    def __init__(self, scene_list, vertices, tex_levels):
        self.vertices = vertices
        self.tex = tex_levels
        cache = {}
        self.views = [_View(s, vertices, tex_levels, cache) for s in scene_list]
        self.grad_vertices = torch.zeros_like(vertices)
        self.grad_levels = [torch.zeros(l.shape, dtype=torch.float32, device=l.device) for l in tex_levels]

    def clear(self):
        for v in self.views:
            v.color[...] = torch.tensor(v.scene.clear_color, dtype=v.color.dtype, device=v.color.device)
            v.depth.fill_(v.scene.clear_depth)

    def forward(self, renderer):
        self.clear()
        if len(self.views) == 1:
            renderer.draw(self.views[0].state, self.views[0].args)
        else:
            renderer.draw_batch([v.state for v in self.views], [v.args for v in self.views])

    def colors(self):
        return torch.stack([v.color.float() for v in self.views])

    def adjoint(self, renderer, grad_color):
        g = grad_color.detach().float().contiguous()
        self._grad = g  # kept alive until the enqueued adjoint has read it
        self.grad_vertices.zero_()
        for l in self.grad_levels:
            l.zero_()
        adj = [v.adjoint_args(g[i], self.grad_vertices, self.grad_levels) for i, v in enumerate(self.views)]
        if len(self.views) == 1:
            renderer.draw_adjoint(self.views[0].state, self.views[0].args, adj[0])
        else:
            renderer.draw_adjoint_batch([v.state for v in self.views], [v.args for v in self.views], adj)


class _DrawViews(torch.autograd.Function):
    @staticmethod
    def forward(ctx, renderer, scene_list, vertices, *levels):
        _check_inputs(vertices, levels)
        renderer.set_stream(torch.cuda.current_stream(vertices.device))  # order with torch's work
        verts = vertices.detach().contiguous()
        tex = [l.detach().to(_texture_dtype(scene_list[0])).contiguous() for l in levels]
        ds = DrawSet(scene_list, verts, tex)
        ds.forward(renderer)
        ctx.renderer, ctx.drawset = renderer, ds
        return ds.colors()

    @staticmethod
    def backward(ctx, grad_out):
        ds, r = ctx.drawset, ctx.renderer
        r.set_stream(torch.cuda.current_stream(ds.vertices.device))
        ds.adjoint(r, grad_out)
        return (None, None, ds.grad_vertices) + tuple(ds.grad_levels)


def render(renderer, scene, vertices, levels=()):
    """Differentiable draw of one scene: colour as float32 [H, W, 4] ([4, H, W, 4] with 4x MSAA)."""
    return _DrawViews.apply(renderer, [scene], vertices, *levels)[0]


def render_views(renderer, scene_list, vertices, levels=()):
    """Differentiable draws of several views sharing vertices and texture:
    float32 [V, H, W, 4] ([V, 4, H, W, 4] with 4x MSAA)."""
    return _DrawViews.apply(renderer, list(scene_list), vertices, *levels)
