"""TEST INFRASTRUCTURE ONLY (the checker, never the product).

FP64 host reference of the draw adjoint that libswgb implements in
swgb_draw_adjoint (include/swgb.h states the differentiated model).  The
reference renderer has no backward pass; this module restates the model in
float64 numpy so the device gradients can be checked against it and against
central finite differences of the same model.

Visibility is held fixed and taken from the CPU oracle
(oracle.render_visibility): per sample and pixel, the primitives whose
fragment passed the depth test, in primitive order.  Given parameters
(object-space positions, vertex colours, texture coordinates, texture
levels), the model colour of a sample is

  * no blending: the shaded colour of its last passing primitive;
  * premultiplied OVER: C <- S + (1 - S.a) C over its passing primitives,
    from the clear colour;

where the shaded colour of primitive t at pixel (px, py) is the perspective-
correct interpolation at the pixel centre (homogeneous barycentrics of the
clip-space vertices), times the fp32 SamplerCore filter (bilinear, optional
trilinear between two levels) at the interpolated coordinates, with the level
of detail computed once from the quad's lanes 0, 1 and 2 and held constant.
"""
import numpy as np

ONE_BELOW = float(np.frombuffer(np.uint32(0x3F7FFFFF).tobytes(), np.float32)[0])
CLAMP, MIRROR, REPEAT = 2, 1, 0  # VkSamplerAddressMode values used by the scenes


def log2sqrt_f32(x):
    """SamplerCore's log2(sqrt(x)) bit trick (src/Pipeline/SamplerCore.cpp:1333-1341), in float32."""
    x = np.asarray(x, np.float32)
    x = x * x
    bits = x.view(np.int32).astype(np.float32)
    return (bits - np.float32(1065353216.0)) * np.float32(2.0 ** -25)


def triangle_vertices(scene):
    """Vertex-buffer index of each corner of each triangle [T, 3]: list,
    strip or fan positions (setBatchIndices, first vertex provoking,
    src/Device/Renderer.cpp:97-134), through the index buffer when indexed,
    plus first_vertex (non-indexed) and base_vertex."""
    from swiftshader_gb300 import abi
    t = np.arange(scene.tri_count, dtype=np.int64)
    if scene.topology == abi.TOPOLOGY_TRIANGLE_STRIP:
        pos = np.stack([t, t + 1 + (t & 1), t + 2 - (t & 1)], axis=1)
    elif scene.topology == abi.TOPOLOGY_TRIANGLE_FAN:
        pos = np.stack([t + 1, t + 2, np.zeros_like(t)], axis=1)
    else:
        pos = 3 * t[:, None] + np.arange(3)
    if scene.indices is None:
        return pos + scene.first_vertex + scene.base_vertex
    return np.asarray(scene.indices, np.int64)[pos] + scene.base_vertex


class Model:
    """The differentiable draw of one scene with fixed visibility."""

    def __init__(self, scene, vis, vis_len):
        from swiftshader_gb300 import abi
        assert (vis_len <= vis.shape[-1]).all(), "visibility list overflow"
        self.scene = scene
        self.abi = abi
        self.S, self.H, self.W = vis_len.shape
        self.mvp = np.asarray(scene.mvp if scene.mvp is not None else np.eye(4), np.float64)
        self.tri_vertices = triangle_vertices(scene)
        vx, vy, vw, vh = scene.viewport or (0, 0, scene.width, scene.height)
        self.rx_of = lambda px: (np.asarray(px, np.float64) + 0.5 - vx - 0.5 * vw) / (0.5 * vw)
        self.ry_of = lambda py: (np.asarray(py, np.float64) + 0.5 - vy - 0.5 * vh) / (0.5 * vh)
        self.blend = scene.blend is not None
        self.textured = scene.fragment_shader == abi.FS_TEX_X_VCOLOR
        smp = scene.sampler
        nlev = len(scene.texture_levels)
        self.min_lod = float(np.clip(smp.get("min_lod", 0.0), 0, 13)) if nlev > 1 else 0.0
        self.max_lod = float(np.clip(smp.get("max_lod", 0.0), 0, 13)) if nlev > 1 else 0.0
        self.lod_bias = float(smp.get("mip_lod_bias", 0.0))
        self.linear = smp.get("mag_filter", 0) == abi.FILTER_LINEAR
        self.mip_linear = smp.get("mipmap_mode", 0) == abi.MIPMAP_MODE_LINEAR
        self.addr = (smp.get("address_u", REPEAT), smp.get("address_v", REPEAT))
        # passing entries: sample, y, x, position in list, primitive
        s, y, x = np.nonzero(vis_len)
        lens = vis_len[s, y, x].astype(np.int64)
        rep = np.repeat(np.arange(len(s)), lens)
        k = np.arange(len(rep)) - np.repeat(np.cumsum(lens) - lens, lens)
        self.e_s, self.e_y, self.e_x, self.e_k = s[rep], y[rep], x[rep], k
        self.e_t = vis[self.e_s, self.e_y, self.e_x, self.e_k].astype(np.int64)
        self.e_len = lens[rep]

    # ---- parameters ---------------------------------------------------------

    def params(self):
        sc = self.scene
        v = np.asarray(sc.vertices, np.float64)
        return {"positions": v[:, 0:4].copy(), "colors": v[:, 4:8].copy(), "uvs": v[:, 8:10].copy(),
                "levels": [np.asarray(l, np.float64) for l in sc.texture_levels]}

    # ---- texture filter -----------------------------------------------------

    def _address(self, coord, mode, dim):
        if mode == CLAMP:
            c = np.clip(coord, 0.0, ONE_BELOW)
            slope = ((coord > 0.0) & (coord < 1.0)).astype(np.float64)
        elif mode == MIRROR:
            h = coord * 0.5
            d = h - np.rint(h)
            c = np.minimum(2.0 * np.abs(d), ONE_BELOW)
            slope = np.sign(d)
        else:
            c = np.minimum(coord - np.floor(coord), ONE_BELOW)
            slope = np.ones_like(coord)
        c = c * dim
        if not self.linear:
            x0 = np.floor(c).astype(np.int64)
            return x0, x0, np.zeros_like(c), slope * dim
        c = c - 0.5
        fl = np.floor(c)
        f = c - fl
        x0 = fl.astype(np.int64)
        x1 = x0 + 1
        if mode == REPEAT:
            x0 = np.where(x0 < 0, dim - 1, x0)
            x1 = np.where(x1 >= dim, 0, x1)
        else:
            x0 = np.maximum(x0, 0)
            x1 = np.minimum(x1, dim - 1)
        return x0, x1, f, slope * dim

    def _lod(self, uq, vq):
        if self.min_lod == self.max_lod:
            return np.full(uq.shape[0], self.min_lod, np.float32)
        W, H = self.scene.texture_levels[0].shape[1], self.scene.texture_levels[0].shape[0]
        uq, vq = uq.astype(np.float32), vq.astype(np.float32)
        a = (uq[:, 1] - uq[:, 0]) * np.float32(W)
        b = (uq[:, 2] - uq[:, 0]) * np.float32(W)
        c = (vq[:, 1] - vq[:, 0]) * np.float32(H)
        e = (vq[:, 2] - vq[:, 0]) * np.float32(H)
        lod = log2sqrt_f32(np.maximum(a * a + c * c, b * b + e * e)) + np.float32(self.lod_bias)
        return np.minimum(np.maximum(lod, np.float32(self.min_lod)), np.float32(self.max_lod))

    def _filter(self, levels, u, v, lod, gt=None, grads=None):
        """Filtered texels [F,4] and their derivatives by u and v; with gt,
        adds gt * filter weight into grads[level]."""
        F = u.shape[0]
        tex, du, dv = np.zeros((F, 4)), np.zeros((F, 4)), np.zeros((F, 4))
        lod64 = lod.astype(np.float64)
        fr = lod64 - np.floor(lod64)
        nlev = len(levels)
        if self.mip_linear:
            ilod = np.trunc(lod64).astype(np.int64)
        else:
            ilod = np.rint(lod64).astype(np.int64)
        for second in range(2 if self.mip_linear else 1):
            wl = (fr if second else 1.0 - fr) if self.mip_linear else np.ones(F)
            li = np.clip(ilod + second, 0, nlev - 1)
            for L in np.unique(li):
                m = li == L
                lv = levels[L]
                h, w = lv.shape[:2]
                x0, x1, fu, su = self._address(u[m], self.addr[0], w)
                y0, y1, fv, sv = self._address(v[m], self.addr[1], h)
                wm = wl[m][:, None]
                if not self.linear:
                    tex[m] += wm * lv[y0, x0]
                    if gt is not None:
                        np.add.at(grads[L], (y0, x0), wm * gt[m])
                    continue
                c00, c10, c01, c11 = lv[y0, x0], lv[y0, x1], lv[y1, x0], lv[y1, x1]
                fu_, fv_ = fu[:, None], fv[:, None]
                a0 = c00 + fu_ * (c10 - c00)
                a1 = c01 + fu_ * (c11 - c01)
                tex[m] += wm * (a0 + fv_ * (a1 - a0))
                du[m] += wm * su[:, None] * ((1 - fv_) * (c10 - c00) + fv_ * (c11 - c01))
                dv[m] += wm * sv[:, None] * (a1 - a0)
                if gt is not None:
                    g = gt[m] * wm
                    np.add.at(grads[L], (y0, x0), (1 - fu_) * (1 - fv_) * g)
                    np.add.at(grads[L], (y0, x1), fu_ * (1 - fv_) * g)
                    np.add.at(grads[L], (y1, x0), (1 - fu_) * fv_ * g)
                    np.add.at(grads[L], (y1, x1), fu_ * fv_ * g)
        return tex, du, dv

    # ---- shading ------------------------------------------------------------

    def _geometry(self, p, t, px, py):
        idx = self.tri_vertices[t]                      # [F,3]
        clip = p["positions"][idx] @ self.mvp.T          # [F,3,4]
        q = clip[..., [0, 1, 3]]
        r = np.stack([self.rx_of(px), self.ry_of(py), np.ones(len(t))], axis=1)
        K = np.stack([np.cross(q[:, 1], q[:, 2]), np.cross(q[:, 2], q[:, 0]), np.cross(q[:, 0], q[:, 1])], axis=1)
        return idx, q, r, K

    def _entry_lod(self):
        """Level of detail of every entry at the scene's own parameters; the
        model holds it constant (also under finite-difference perturbations)."""
        if getattr(self, "lod_e", None) is None:
            p = self.params()
            t, px, py = self.e_t, self.e_x, self.e_y
            idx, q, r, K = self._geometry(p, t, px, py)
            uv_v = p["uvs"][idx]
            qx, qy = px & ~1, py & ~1
            uq, vq = np.zeros((len(t), 3)), np.zeros((len(t), 3))
            for j, (ox, oy) in enumerate(((0, 0), (1, 0), (0, 1))):
                rj = np.stack([self.rx_of(qx + ox), self.ry_of(qy + oy), np.ones(len(t))], axis=1)
                wj = np.einsum("fk,fik->fi", rj, K)
                bj = wj / wj.sum(1)[:, None]
                uvj = np.einsum("fi,fik->fk", bj, uv_v)
                uq[:, j], vq[:, j] = uvj[:, 0], uvj[:, 1]
            self.lod_e = self._lod(uq, vq)
        return self.lod_e

    def shade(self, p, sel, gS=None, grads=None):
        """Shaded colour [F,4] of the entries 'sel' (index array into the
        entry table); with gS, adds the shading adjoint into grads."""
        t, px, py = self.e_t[sel], self.e_x[sel], self.e_y[sel]
        idx, q, r, K = self._geometry(p, t, px, py)
        uu = np.einsum("fk,fik->fi", r, K)
        U = uu.sum(1)
        b = uu / U[:, None]
        col_v, uv_v = p["colors"][idx], p["uvs"][idx]
        col = np.einsum("fi,fik->fk", b, col_v)
        uv = np.einsum("fi,fik->fk", b, uv_v)
        if self.textured:
            lod = self._entry_lod()[sel]
            gt = None if gS is None else gS * col
            tex, du, dv = self._filter(p["levels"], uv[:, 0], uv[:, 1], lod, gt, None if grads is None else grads["levels"])
            S = tex * col
        else:
            S = col
        if gS is None:
            return S
        if self.textured:
            gcol = gS * tex
            gu = (gt * du).sum(1)
            gv = (gt * dv).sum(1)
        else:
            gcol = gS
            gu = gv = np.zeros(len(t))
        guv = np.stack([gu, gv], axis=1)
        for i in range(3):
            np.add.at(grads["colors"], idx[:, i], b[:, i:i + 1] * gcol)
            np.add.at(grads["uvs"], idx[:, i], b[:, i:i + 1] * guv)
        gb = np.einsum("fk,fik->fi", gcol, col_v) + np.einsum("fk,fik->fi", guv, uv_v)
        gU = (gb - (b * gb).sum(1, keepdims=True)) / U[:, None]
        rq = [np.cross(r, q[:, i]) for i in range(3)]
        gq = [gU[:, 1:2] * rq[2] - gU[:, 2:3] * rq[1],
              gU[:, 2:3] * rq[0] - gU[:, 0:1] * rq[2],
              gU[:, 0:1] * rq[1] - gU[:, 1:2] * rq[0]]
        for i in range(3):
            gclip = np.stack([gq[i][:, 0], gq[i][:, 1], np.zeros(len(t)), gq[i][:, 2]], axis=1)
            np.add.at(grads["positions"], idx[:, i], gclip @ self.mvp)
        return S

    # ---- the draw -----------------------------------------------------------

    def _entries(self, p):
        return self.shade(p, np.arange(len(self.e_t)))

    def colors(self, p=None):
        """Model colour of every sample [S,H,W,4] (float64)."""
        p = p or self.params()
        out = np.empty((self.S, self.H, self.W, 4))
        out[...] = np.asarray(self.scene.clear_color, np.float64)
        Se = self._entries(p)
        if not self.blend:
            last = self.e_k == self.e_len - 1
            out[self.e_s[last], self.e_y[last], self.e_x[last]] = Se[last]
            return out
        for k in range(int(self.e_k.max()) + 1 if len(self.e_k) else 0):
            m = self.e_k == k
            s, y, x = self.e_s[m], self.e_y[m], self.e_x[m]
            out[s, y, x] = Se[m] + (1.0 - Se[m, 3:4]) * out[s, y, x]
        return out

    def gradients(self, grad_color, p=None):
        """dL/d(parameters) for dL/d(colour) = grad_color [S,H,W,4]."""
        p = p or self.params()
        grads = {"positions": np.zeros_like(p["positions"]), "colors": np.zeros_like(p["colors"]),
                 "uvs": np.zeros_like(p["uvs"]), "levels": [np.zeros_like(l) for l in p["levels"]]}
        G = np.asarray(grad_color, np.float64).reshape(self.S, self.H, self.W, 4)
        if not self.blend:
            last = np.nonzero(self.e_k == self.e_len - 1)[0]
            gS = G[self.e_s[last], self.e_y[last], self.e_x[last]]
            self.shade(p, last, gS, grads)
            return grads
        Se = self._entries(p)
        kmax = int(self.e_k.max()) + 1 if len(self.e_k) else 0
        # colour before each entry (forward), then the reverse sweep
        before = np.empty_like(Se)
        cur = np.empty((self.S, self.H, self.W, 4))
        cur[...] = np.asarray(self.scene.clear_color, np.float64)
        for k in range(kmax):
            m = self.e_k == k
            s, y, x = self.e_s[m], self.e_y[m], self.e_x[m]
            before[m] = cur[s, y, x]
            cur[s, y, x] = Se[m] + (1.0 - Se[m, 3:4]) * cur[s, y, x]
        g = G.copy()
        dS = np.zeros_like(Se)
        for k in range(kmax - 1, -1, -1):
            m = self.e_k == k
            s, y, x = self.e_s[m], self.e_y[m], self.e_x[m]
            gk = g[s, y, x]
            d = dS[m]
            d += gk
            d[:, 3] -= (gk * before[m]).sum(1)
            dS[m] = d
            g[s, y, x] = (1.0 - Se[m, 3:4]) * gk
        self.shade(p, np.arange(len(self.e_t)), dS, grads)
        return grads


def l2_loss(colors, target):
    d = colors - target
    return float((d * d).sum()), 2.0 * d
