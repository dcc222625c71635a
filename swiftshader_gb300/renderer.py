"""Host-side mirror of sw::Renderer for the triangle-list FILL path.

``Renderer.draw(state, args)`` is the reference's
``sw::Renderer::draw(pipeline, dynamicState, count, baseVertex, events,
instanceID, layer, indexBuffer, renderArea, pushConstants)``
(src/Device/Renderer.hpp:211-213) with the pipeline state flattened into
``abi.PipelineState`` and the per-draw arguments into ``abi.DrawArgs``;
``Renderer.synchronize()`` is ``sw::Renderer::synchronize()``
(src/Device/Renderer.cpp:664-671).  Like the reference, ``draw`` returns before
the work completes; errors the device detects surface at ``synchronize``.

Every call goes through libswgb.so.  There is no CPU path: without the built
library or a CUDA device, construction raises.
"""
import ctypes as C

import numpy as np

from . import abi, scenes
from ._lib import check, load


class Renderer:
    def __init__(self, device=0, stream=None):
        self._L = load()
        ctx = C.c_void_p()
        handle = None
        if stream is not None:
            raw = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
            # handle 0 is the legacy default stream; NULL would ask the library
            # for a private stream, so pass cudaStreamLegacy (1) instead.
            handle = C.c_void_p(raw if raw else 1)
        check(self._L.swgb_ctx_create(int(device), handle, C.byref(ctx)), "swgb_ctx_create")
        self._ctx = ctx

    def draw(self, state, args):
        check(self._L.swgb_draw(self._ctx, C.byref(state), C.byref(args)), "swgb_draw")

    def draw_batch(self, states, args):
        """Enqueue draws as batches; `states`/`args` are sequences or prebuilt
        ctypes arrays of PipelineState / DrawArgs."""
        n = len(states)
        S = states if isinstance(states, C.Array) else (abi.PipelineState * n)(*states)
        A = args if isinstance(args, C.Array) else (abi.DrawArgs * n)(*args)
        check(self._L.swgb_draw_batch(self._ctx, S, A, n), "swgb_draw_batch")

    def draw_adjoint(self, state, args, adj):
        """Adjoint of one draw (swgb_draw_adjoint); adj is an abi.AdjointArgs."""
        check(self._L.swgb_draw_adjoint(self._ctx, C.byref(state), C.byref(args), C.byref(adj)), "swgb_draw_adjoint")

    def draw_adjoint_batch(self, states, args, adjs):
        n = len(states)
        S = states if isinstance(states, C.Array) else (abi.PipelineState * n)(*states)
        A = args if isinstance(args, C.Array) else (abi.DrawArgs * n)(*args)
        G = adjs if isinstance(adjs, C.Array) else (abi.AdjointArgs * n)(*adjs)
        check(self._L.swgb_draw_adjoint_batch(self._ctx, S, A, G, n), "swgb_draw_adjoint_batch")

    def synchronize(self):
        check(self._L.swgb_sync(self._ctx), "swgb_sync")

    def set_raster_config(self, bin_width=16, bin_height=16, hiz=True):
        cfg = abi.RasterConfig(bin_width, bin_height, 1 if hiz else 0, 0)
        check(self._L.swgb_ctx_set_raster_config(self._ctx, C.byref(cfg)), "swgb_ctx_set_raster_config")

    def raster_config(self):
        cfg = abi.RasterConfig()
        check(self._L.swgb_ctx_get_raster_config(self._ctx, C.byref(cfg)), "swgb_ctx_get_raster_config")
        return cfg.as_dict()

    def autotune(self, states, args, batched=True, runs=abi.AUTOTUNE_DEFAULT_RUNS, table=None):
        """Picks the raster configuration for these draws and keeps it on this
        renderer; returns (best, [(config, {"median", "min", "max"})]).

        With a tuning.TuningTable that already holds the draws' workload class
        the recorded configuration is set without running anything (the
        returned list is then the recorded one, and the attachments are not
        touched).  Otherwise swgb_autotune runs the draws under every
        candidate (one warm-up and `runs` timed runs each, the lowest median
        wins, the attachments left as one run leaves them) and the result is
        recorded in the table when one is given."""
        n = len(states)
        S = states if isinstance(states, C.Array) else (abi.PipelineState * n)(*states)
        A = args if isinstance(args, C.Array) else (abi.DrawArgs * n)(*args)
        key = None
        if table is not None:
            from .tuning import workload_class
            key = workload_class(S, A, batched)
            hit = table.get(key)
            if hit is not None:
                w, h = (int(x) for x in hit["bin"].split("x"))
                self.set_raster_config(w, h, bool(hit["hiz"]))
                cands = []
                for name, t in hit["candidates_ms"].items():
                    shape, hz = name.split(" hiz")
                    cands.append(({"bin": shape, "hiz": int(hz)}, t))
                return {"bin": hit["bin"], "hiz": int(hit["hiz"])}, cands
        best = abi.RasterConfig()
        cands = (abi.RasterConfig * abi.AUTOTUNE_CANDIDATES)()
        ms = (C.c_double * abi.AUTOTUNE_CANDIDATES)()
        lo = (C.c_double * abi.AUTOTUNE_CANDIDATES)()
        hi = (C.c_double * abi.AUTOTUNE_CANDIDATES)()
        check(self._L.swgb_autotune(self._ctx, S, A, n, 1 if batched else 0, int(runs), C.byref(best), cands, ms, lo, hi),
              "swgb_autotune")
        res = [(c.as_dict(), {"median": float(t), "min": float(a), "max": float(b)})
               for c, t, a, b in zip(cands, ms, lo, hi)]
        if table is not None:
            table.record(key, best.as_dict(), res)
        return best.as_dict(), res

    def counters(self):
        c = abi.Counters()
        check(self._L.swgb_get_counters(self._ctx, C.byref(c)), "swgb_get_counters")
        return c.as_dict()

    def reset_counters(self):
        check(self._L.swgb_reset_counters(self._ctx), "swgb_reset_counters")

    def launch_count(self):
        return int(self._L.swgb_launch_count(self._ctx))

    def set_kernel_timing(self, enable, kinds=None):
        """Event pairs around every kernel launch (enable), or only around the
        launches of the kernel kinds named in kinds (KERNEL_NAMES)."""
        v = 1 if enable else 0
        if enable and kinds is not None:
            v = 0x10000 | sum(1 << self.KERNEL_NAMES.index(k) for k in kinds)  # SWGB_KERNEL_TIMING_KINDS
        check(self._L.swgb_set_kernel_timing(self._ctx, v), "swgb_set_kernel_timing")

    # --- sw::Blitter steps either side of a draw (swgb_clear / swgb_resolve /
    # swgb_blit); images are abi.Image views, e.g. from image_view().

    def clear_image(self, image, value):
        """Blitter::clear of a whole image: value is an RGBA float sequence for
        colour images, a float depth for D32_SFLOAT / D16_UNORM, an int for
        S8_UINT stencil planes."""
        self.clear_area(image, value, None)

    def clear_area(self, image, value, area):
        """Blitter::clear of area = (x, y, width, height) (None: whole image)."""
        if image.format == abi.FORMAT_S8_UINT:
            v, fmt = (C.c_uint32 * 4)(int(value), 0, 0, 0), abi.FORMAT_S8_UINT
        elif image.format in (abi.FORMAT_D32_SFLOAT, abi.FORMAT_D16_UNORM):
            v, fmt = (C.c_float * 4)(float(value), 0.0, 0.0, 0.0), abi.FORMAT_D32_SFLOAT
        else:
            v, fmt = (C.c_float * 4)(*[float(x) for x in value]), abi.FORMAT_R32G32B32A32_SFLOAT
        r = C.byref(abi.Rect(*area)) if area is not None else None
        check(self._L.swgb_clear(self._ctx, v, fmt, C.byref(image), r), "swgb_clear")

    def resolve(self, src, dst, region=None):
        """Blitter::resolve of a 4-sample image into a single-sample one;
        region = (src_x, src_y, dst_x, dst_y, width, height) or None (whole)."""
        r = C.byref(abi.ResolveRegion(*region)) if region is not None else None
        check(self._L.swgb_resolve(self._ctx, C.byref(src), C.byref(dst), r), "swgb_resolve")

    def blit(self, src, dst, src_box, dst_box, filter=abi.FILTER_LINEAR):
        """Blitter::blit of src_box = (x0, y0, x1, y1) onto dst_box."""
        reg = abi.BlitRegion((C.c_int32 * 4)(*src_box), (C.c_int32 * 4)(*dst_box))
        check(self._L.swgb_blit(self._ctx, C.byref(src), C.byref(dst), C.byref(reg), int(filter)), "swgb_blit")

    def generate_mipmaps(self, levels):
        """Fills levels[1:] from levels[0] with one LINEAR blit per level, the
        vkCmdBlitImage sequence applications record for mip generation."""
        for a, b in zip(levels[:-1], levels[1:]):
            self.blit(a, b, (0, 0, a.width, a.height), (0, 0, b.width, b.height), abi.FILTER_LINEAR)

    KERNEL_NAMES = ("vertex", "setup", "raster", "batch", "adjoint", "bin_order", "blit")

    def kernel_times(self):
        """{kernel: (total ms, launches)} since the last call (synchronises)."""
        ms = (C.c_double * 8)()
        n = (C.c_uint32 * 8)()
        check(self._L.swgb_get_kernel_times(self._ctx, ms, n), "swgb_get_kernel_times")
        return {name: (ms[i], int(n[i])) for i, name in enumerate(self.KERNEL_NAMES) if n[i]}

    def set_stream(self, stream):
        raw = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
        check(self._L.swgb_ctx_set_stream(self._ctx, C.c_void_p(raw if raw else 1)), "swgb_ctx_set_stream")

    def close(self):
        if getattr(self, "_ctx", None):
            self._L.swgb_ctx_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceScene:
    """A scene's buffers resident in device memory (torch tensors), plus the
    C-ABI state that points at them.

    All of them live in one device allocation (``arena``): the draw's inputs
    first (vertices and indices, ``geometry_region``; texture levels,
    ``texture_region``), then the attachments (colour, depth, stencil;
    ``outputs()``), each 256-byte aligned.  A caller that re-uploads the inputs
    and reads the attachments back every frame makes few, large copies, and can
    upload the textures while the draw's first stages run
    (``swgb_draw_args.raster_wait_event``)."""

    ALIGN = 256

    def __init__(self, scene, device="cuda"):
        import torch
        self.scene = scene
        self.device = torch.device(device)
        cdtype = {abi.FORMAT_R8G8B8A8_UNORM: torch.uint8, abi.FORMAT_B8G8R8A8_UNORM: torch.uint8,
                  abi.FORMAT_R8G8B8A8_SRGB: torch.uint8, abi.FORMAT_B8G8R8A8_SRGB: torch.uint8,
                  abi.FORMAT_R32G32B32A32_SFLOAT: torch.float32, abi.FORMAT_R16G16B16A16_SFLOAT: torch.float16}[scene.color_format]
        cshape, dshape = scenes.attachment_shapes(scene)
        # D16_UNORM attachments live in int16 tensors (the same bits; torch has no uint16 arithmetic)
        self.d16 = scene.depth_format == abi.FORMAT_D16_UNORM
        ddtype = torch.int16 if self.d16 else torch.float32
        up = lambda n: (n + self.ALIGN - 1) // self.ALIGN * self.ALIGN
        inputs = [np.ascontiguousarray(scene.vertices)]
        if scene.indices is not None:
            inputs.append(scenes.index_bytes(scene))
        inputs += [np.ascontiguousarray(l) for l in scene.texture_levels]
        off, where = 0, []
        first_level = len(inputs) - len(scene.texture_levels)
        self.texture_offset = None
        for i, a in enumerate(inputs):
            if i == first_level:
                self.texture_offset = off  # geometry before it, texture levels from it
            where.append(off)
            off = up(off + a.nbytes)
        self.input_bytes = off
        if self.texture_offset is None:
            self.texture_offset = off
        esize = lambda dt: torch.empty((), dtype=dt).element_size()
        outputs = [(cshape, cdtype), (dshape, ddtype)] + ([(dshape, torch.uint8)] if scene.stencil is not None else [])
        for shape, dt in outputs:
            where.append(off)
            off = up(off + int(np.prod(shape)) * esize(dt))
        self.arena = torch.empty(off, dtype=torch.uint8, device=self.device)
        host = np.zeros(self.input_bytes, np.uint8)
        for a, o in zip(inputs, where):
            host[o:o + a.nbytes] = a.reshape(-1).view(np.uint8)
        self.arena[:self.input_bytes].copy_(torch.from_numpy(host))

        def view(o, shape, dt):
            n = int(np.prod(shape)) * esize(dt)
            return self.arena[o:o + n].view(dt).view(shape)

        tdt = {np.dtype(np.float32): torch.float32, np.dtype(np.float16): torch.float16, np.dtype(np.uint8): torch.uint8}
        k = 0
        self.vertices = view(where[k], inputs[k].shape, tdt[inputs[k].dtype])
        k += 1
        self.indices = None
        if scene.indices is not None:
            self.indices = view(where[k], inputs[k].shape, torch.uint8)
            k += 1
        self.levels = []
        for _ in scene.texture_levels:
            a = inputs[k]
            self.levels.append(view(where[k], a.shape, tdt[a.dtype]))
            k += 1
        self.color = view(where[k], cshape, cdtype)
        self.depth = view(where[k + 1], dshape, ddtype)
        self.stencil = view(where[k + 2], dshape, torch.uint8) if scene.stencil is not None else None
        self.output_region = (where[k], off)
        self._clear_rgba = None
        self.clear()

    @property
    def input_region(self):
        """The arena's input bytes (vertices, indices, texture levels)."""
        return self.arena[:self.input_bytes]

    @property
    def geometry_region(self):
        """The input bytes of vertices and indices."""
        return self.arena[:self.texture_offset]

    @property
    def texture_region(self):
        """The input bytes of the texture levels."""
        return self.arena[self.texture_offset:self.input_bytes]

    def outputs(self):
        """The arena's attachment bytes (colour, depth, stencil)."""
        return self.arena[self.output_region[0]:self.output_region[1]]

    # colour formats whose clear value the Blitter clear takes exactly as
    # normalised floats (UNORM8: byte / 255 rounds back to the byte)
    _BLITTER_CLEAR = {abi.FORMAT_R8G8B8A8_UNORM: 255.0, abi.FORMAT_B8G8R8A8_UNORM: 255.0,
                      abi.FORMAT_R32G32B32A32_SFLOAT: 1.0}

    def clear(self, renderer=None):
        """Clears the attachments to the scene's clear values: with a renderer
        through the library's Blitter clear (swgb_clear, one kernel per
        attachment), else by torch fills."""
        sc = self.scene
        scale = self._BLITTER_CLEAR.get(sc.color_format)
        if renderer is not None and scale is not None and not self.d16 and self.stencil is None:
            # clear_color holds the attachment's bytes in memory order; the
            # Blitter clear takes R, G, B, A (B8G8R8A8 stores B first)
            cc = list(sc.clear_color)
            if sc.color_format == abi.FORMAT_B8G8R8A8_UNORM:
                cc = [cc[2], cc[1], cc[0], cc[3]]
            renderer.clear_image(image_view(self.color, sc.color_format, sc.samples), [v / scale for v in cc])
            renderer.clear_image(image_view(self.depth, abi.FORMAT_D32_SFLOAT, sc.samples), sc.clear_depth)
            return
        self.color[...] = device_value(self, "_clear_rgba", self.scene.clear_color, self.color)
        if self.d16:
            self.depth.fill_(int(np.array(scenes.depth_clear_value(self.scene)).view(np.int16)))
        else:
            self.depth.fill_(self.scene.clear_depth)
        if self.stencil is not None:
            self.stencil.fill_(int(self.scene.stencil.get("clear", 0)))

    def depth_numpy(self):
        """The depth attachment on the host: float32, or uint16 for D16_UNORM."""
        d = self.depth.cpu().numpy()
        return d.view(np.uint16) if self.d16 else d

    def state(self):
        return scenes.build_state(self.scene, self.color.data_ptr(), self.depth.data_ptr(), self.vertices.data_ptr(),
                                  [l.data_ptr() for l in self.levels],
                                  stencil_ptr=None if self.stencil is None else self.stencil.data_ptr())

    def args(self):
        return scenes.build_args(self.scene, None if self.indices is None else self.indices.data_ptr())


class DeviceBatch:
    """A BatchScene resident in device memory: one vertex array, one texture
    array, atlas pages of colour (RGBA8) and depth (D32F), and the C-ABI
    state/args arrays of every draw."""

    def __init__(self, batch, device="cuda"):
        import torch
        self.batch = batch
        self.device = torch.device(device)
        P = batch.page_size
        self.vertices = torch.from_numpy(np.ascontiguousarray(batch.vertices)).to(self.device)
        self.textures = torch.from_numpy(np.ascontiguousarray(batch.textures)).to(self.device)
        self.color = torch.empty((batch.pages, P, P, 4), dtype=torch.uint8, device=self.device)
        self.depth = torch.empty((batch.pages, P, P), dtype=torch.float32, device=self.device)
        self.clear()
        n = batch.n
        self.states = (abi.PipelineState * n)()
        self.args = (abi.DrawArgs * n)()
        cbase, dbase = self.color.data_ptr(), self.depth.data_ptr()
        vbase, tbase = self.vertices.data_ptr(), self.textures.data_ptr()
        tex_bytes = batch.textures[0].nbytes
        for i in range(n):
            sc = batch.draw_scene(i)
            page, x, y = (int(v) for v in batch.place[i])
            off = (page * P + y) * P + x
            self.states[i] = scenes.build_state(sc, cbase + off * 4, dbase + off * 4,
                                                vbase + int(batch.vstart[i]) * scenes.VERTEX_STRIDE,
                                                [tbase + i * tex_bytes], color_pitch=P * 4, depth_pitch=P * 4)
            self.args[i] = scenes.build_args(sc)

    def clear(self):
        self.color[...] = device_value(self, "_clear_rgba", self.batch.clear_color, self.color)
        self.depth.fill_(self.batch.clear_depth)

    def draw_batch(self, renderer):
        renderer.draw_batch(self.states, self.args)

    def draw_each(self, renderer, indices=None):
        for i in (range(self.batch.n) if indices is None else indices):
            renderer.draw(self.states[i], self.args[i])

    def view(self, i):
        """Colour and depth of draw i's viewport (device tensor views)."""
        page, x, y = (int(v) for v in self.batch.place[i])
        s = int(self.batch.sides[i])
        return self.color[page, y:y + s, x:x + s], self.depth[page, y:y + s, x:x + s]


def image_view(tensor, format, samples=1):
    """abi.Image over a contiguous CUDA tensor shaped [H, W, C] (or [H, W] for
    depth and stencil), or [samples, H, W, ...] for multisampled images."""
    t = tensor
    if samples > 1:
        assert t.shape[0] == samples
        h, w = t.shape[1], t.shape[2]
    else:
        h, w = t.shape[0], t.shape[1]
    assert t.is_contiguous()
    bpp = abi.TEXEL_BYTES[format]
    pitch = w * bpp
    return abi.Image(t.data_ptr(), format, w, h, samples, pitch, pitch * h)


def device_value(owner, attr, values, like):
    """values as a device tensor like 'like', kept on owner.attr and made again
    only when values change: a clear then copies on the device alone, with no
    host-to-device copy in the stream."""
    key = (tuple(values), like.dtype, like.device)
    cached = getattr(owner, attr, None)
    if cached is None or cached[0] != key:
        cached = (key, torch_tensor(values, like))
        setattr(owner, attr, cached)
    return cached[1]


def torch_tensor(values, like):
    import torch
    return torch.tensor(values, dtype=like.dtype, device=like.device)
