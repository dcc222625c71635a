"""The adjoint on the device (swgb_draw_adjoint / swgb_draw_adjoint_batch
through the torch.autograd.Function of swiftshader_gb300.adjoint) against
the FP64 host reference (oracle/adjoint_ref.py, visibility from the CPU
oracle) and against central finite differences (h = 1e-3) of the device
renderer itself.

Tolerances: gradients within 1e-4 relative error (Frobenius norm per
parameter group) of the FP64 reference; finite differences of the real
renderer within 2e-3 relative for texels and vertex colours (the renderer
interpolates plane equations of sub-pixel-snapped vertices, the model ideal
barycentrics)."""
import numpy as np
import pytest

from swiftshader_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def device_inputs(scene):
    import torch
    verts = torch.from_numpy(np.ascontiguousarray(scene.vertices, np.float32)).cuda().requires_grad_(True)
    levels = [torch.from_numpy(np.ascontiguousarray(l).astype(np.float32)).cuda().requires_grad_(True)
              for l in scene.texture_levels]
    return verts, levels


def reference(scene, G, cap=96):
    """FP64 gradients for dL/dcolour = G ([S, H, W, 4] or [H, W, 4])."""
    import oracle
    import adjoint_ref
    _, _, _, vis, vis_len = oracle.render_visibility(scene, 4, cap=cap)
    m = adjoint_ref.Model(scene, vis, vis_len)
    return m.gradients(np.asarray(G, np.float64).reshape(m.S, m.H, m.W, 4)), m


def compare(grads_ref, gv, gl, tol=1e-4):
    gv = gv.detach().cpu().numpy().astype(np.float64)
    errs = {"positions": rel_err(gv[:, 0:4], grads_ref["positions"]),
            "colors": rel_err(gv[:, 4:8], grads_ref["colors"]),
            "uvs": rel_err(gv[:, 8:10], grads_ref["uvs"])}
    for i, g in enumerate(gl):
        if np.abs(grads_ref["levels"][i]).sum() > 0:
            errs["level%d" % i] = rel_err(g.detach().cpu().numpy(), grads_ref["levels"][i])
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, errs
    return errs


def test_adjoint_sphere_fp32_against_fp64(gpu_lib):
    """The adjoint workload at reduced size: uv-sphere, RGBA32F texture
    bilinear CLAMP, colour = texel x vertex colour, RGBA32F attachment; L2
    loss against a render with perturbed texels."""
    import torch
    from swiftshader_gb300 import Renderer, adjoint
    sc = scenes.scene_sphere_fp32(seg=40, width=128, height=128, tex_size=128)
    r = Renderer(0)
    verts, levels = device_inputs(sc)
    rng = np.random.Generator(np.random.PCG64(33))
    noisy = [l.detach() + torch.from_numpy(rng.normal(0.0, 0.05, l.shape).astype(np.float32)).cuda() for l in levels]
    with torch.no_grad():
        target = adjoint.render(r, sc, verts.detach(), noisy)
    r.reset_counters()
    color = adjoint.render(r, sc, verts, levels)
    loss = ((color - target) ** 2).sum()
    loss.backward()
    cnt = r.counters()
    assert cnt["adjoint_depth_mismatch"] == 0 and cnt["adjoint_list_overflow"] == 0
    assert cnt["adjoint_fragments"] > 1000
    # the forward through the autograd function is the bit-exact draw
    import oracle
    c_ref, _, _ = oracle.render(sc, 4)
    assert np.array_equal(color.detach().cpu().numpy().view(np.uint32), c_ref.view(np.uint32))
    G = (2.0 * (color - target)).detach().cpu().numpy()
    gref, _ = reference(sc, G)
    compare(gref, verts.grad, [l.grad for l in levels])


def test_adjoint_finite_differences_of_device_renderer(gpu_lib):
    """Central differences (h = 1e-3) of the device renderer's loss along
    random directions in texels and vertex colours."""
    import torch
    from swiftshader_gb300 import Renderer, adjoint
    sc = scenes.scene_sphere_fp32(seg=30, width=96, height=96, tex_size=64, seed_index=5)
    r = Renderer(0)
    verts, levels = device_inputs(sc)
    rng = np.random.Generator(np.random.PCG64(34))
    target = torch.from_numpy(rng.uniform(0.0, 0.5, (96, 96, 4)).astype(np.float32)).cuda()
    color = adjoint.render(r, sc, verts, levels)
    ((color - target) ** 2).sum().backward()

    def loss(v, ls):
        with torch.no_grad():
            c = adjoint.render(r, sc, v, ls)
            return float(((c.double() - target.double()) ** 2).sum())

    h = 1e-3
    d = torch.from_numpy(rng.normal(0.0, 1.0, levels[0].shape).astype(np.float32)).cuda()
    fd = (loss(verts.detach(), [levels[0].detach() + h * d]) - loss(verts.detach(), [levels[0].detach() - h * d])) / (2 * h)
    an = float((levels[0].grad.double() * d.double()).sum())
    assert abs(fd - an) <= 2e-3 * abs(an), (fd, an)
    d = torch.zeros_like(verts)
    d[:, 4:8] = torch.from_numpy(rng.normal(0.0, 1.0, (verts.shape[0], 4)).astype(np.float32)).cuda()
    lv = [l.detach() for l in levels]
    fd = (loss(verts.detach() + h * d, lv) - loss(verts.detach() - h * d, lv)) / (2 * h)
    an = float((verts.grad.double() * d.double()).sum())
    assert abs(fd - an) <= 2e-3 * abs(an), (fd, an)


def _views_setup(n_views=3, size=96):
    rng = np.random.Generator(np.random.PCG64(4))
    mesh = scenes.uv_sphere(rng, 60, 40, noise_sigma=0.02)
    levels = scenes.float_mip_chain(rng.uniform(0.0, 1.0, (128, 128, 4)), np.float16)
    views = [scenes.scene_sphere_views(v, width=size, height=size, mesh=mesh, levels=levels) for v in (0, 7, 200)[:n_views]]
    for s in views:
        s.samples = 4
    return views


def test_batched_views_msaa_over_against_fp64(gpu_lib):
    """The batched-adjoint workload at reduced size: views of a noisy
    sphere, 4x MSAA, RGBA16F mipmapped trilinear texture, premultiplied OVER
    into RGBA16F; forward as one batch, adjoint as one batch; gradients summed
    over views against the FP64 reference."""
    import torch
    from swiftshader_gb300 import Renderer, adjoint
    views = _views_setup()
    r = Renderer(0)
    verts, levels = device_inputs(views[0])
    rng = np.random.Generator(np.random.PCG64(35))
    noisy = [l.detach() + torch.from_numpy(rng.normal(0.0, 0.05, l.shape).astype(np.float32)).cuda() for l in levels]
    with torch.no_grad():
        target = adjoint.render_views(r, views, verts.detach(), noisy)
    r.reset_counters()
    color = adjoint.render_views(r, views, verts, levels)
    ((color - target) ** 2).sum().backward()
    cnt = r.counters()
    assert cnt["adjoint_depth_mismatch"] == 0 and cnt["adjoint_list_overflow"] == 0
    G = (2.0 * (color - target)).detach().cpu().numpy()
    total = None
    for i, sc in enumerate(views):
        g, _ = reference(sc, G[i])
        if total is None:
            total = g
        else:
            for k in ("positions", "colors", "uvs"):
                total[k] += g[k]
            total["levels"] = [a + b for a, b in zip(total["levels"], g["levels"])]
    compare(total, verts.grad, [l.grad for l in levels])


def test_single_and_batched_adjoint_agree(gpu_lib):
    """One view through swgb_draw_adjoint and through a one-segment batch of
    the same view twice gives gradients in ratio 2."""
    import torch
    from swiftshader_gb300 import Renderer, adjoint
    v = _views_setup(1, 64)[0]
    r = Renderer(0)
    verts, levels = device_inputs(v)
    c1 = adjoint.render(r, v, verts, levels)
    c1.sum().backward()
    g1 = verts.grad.clone()
    t1 = [l.grad.clone() for l in levels]
    verts.grad = None
    for l in levels:
        l.grad = None
    c2 = adjoint.render_views(r, [v, v], verts, levels)
    c2.sum().backward()
    assert torch.equal(c2[0], c1) and torch.equal(c2[1], c1)
    assert rel_err(verts.grad.cpu().numpy(), 2 * g1.cpu().numpy()) < 1e-5
    for a, b in zip(levels, t1):
        assert rel_err(a.grad.cpu().numpy(), 2 * b.cpu().numpy()) < 1e-5


def layered_scene(n, size=16, seed=36):
    """n full-screen triangles, each nearer than the last, premultiplied OVER
    into RGBA32F: every pixel holds n blended fragments."""
    rng = np.random.Generator(np.random.PCG64(seed))
    v = np.zeros((3 * n, scenes.VERTEX_FLOATS), np.float32)
    for k in range(n):
        v[3 * k:3 * k + 3, 0:2] = [(-1, -1), (3, -1), (-1, 3)]
        v[3 * k:3 * k + 3, 0:2] += rng.normal(0.0, 0.05, (3, 2))
        v[3 * k:3 * k + 3, 2] = 0.9 - 0.8 * k / n
        v[3 * k:3 * k + 3, 3] = 1.0
        v[3 * k:3 * k + 3, 4:8] = rng.uniform(0.0, 0.3, (3, 4))
    return scenes.Scene(name="layers%d" % n, width=size, height=size, vertices=v, tri_count=n,
                        color_format=abi.FORMAT_R32G32B32A32_SFLOAT,
                        blend=(abi.BLEND_ONE, abi.BLEND_ONE_MINUS_SRC_ALPHA, abi.BLEND_OP_ADD,
                               abi.BLEND_ONE, abi.BLEND_ONE_MINUS_SRC_ALPHA, abi.BLEND_OP_ADD))


def test_deep_blended_layers_against_fp64(gpu_lib):
    """40 blended fragments on every pixel (the views workload reaches such
    depths where its rough surface folds): adjoint of the whole OVER chain."""
    import torch
    from swiftshader_gb300 import Renderer, adjoint
    sc = layered_scene(40)
    r = Renderer(0)
    verts = torch.from_numpy(sc.vertices).cuda().requires_grad_(True)
    r.reset_counters()
    color = adjoint.render(r, sc, verts)
    target = torch.full_like(color, 0.25)
    ((color - target) ** 2).sum().backward()
    cnt = r.counters()
    assert cnt["adjoint_list_overflow"] == 0 and cnt["adjoint_depth_mismatch"] == 0
    G = (2.0 * (color - target)).detach().cpu().numpy()
    gref, m = reference(sc, G, cap=64)
    assert cnt["adjoint_fragments"] == len(m.e_t) and m.e_len.max() >= 36
    compare(gref, verts.grad, [])


def test_blended_fragment_overflow_is_counted(gpu_lib):
    """More than 2048 blended fragments on a pixel: the excess is counted in
    adjoint_list_overflow and the rest is still processed."""
    import torch
    from swiftshader_gb300 import Renderer, adjoint
    n = abi.ADJOINT_MAX_FRAGMENTS_PER_PIXEL + 52
    sc = layered_scene(n, size=8)
    r = Renderer(0)
    verts = torch.from_numpy(sc.vertices).cuda().requires_grad_(True)
    r.reset_counters()
    adjoint.render(r, sc, verts).sum().backward()
    cnt = r.counters()
    import oracle
    _, _, ocnt = oracle.render(sc, 4)
    per_pixel = ocnt["fragments_passed"]  # every covered pixel of the 8x8 frame
    cap = abi.ADJOINT_MAX_FRAGMENTS_PER_PIXEL
    assert cnt["adjoint_fragments"] + cnt["adjoint_list_overflow"] == per_pixel
    assert cnt["adjoint_list_overflow"] > 0 and cnt["adjoint_fragments"] <= 64 * cap


def test_unsupported_states_are_rejected(gpu_lib):
    import torch
    from swiftshader_gb300 import DeviceScene, Renderer
    from swiftshader_gb300._lib import SwgbError
    r = Renderer(0)
    sc = scenes.scene_small(n_tris=10, width=32, height=32)  # RGBA8 attachment
    ds = DeviceScene(sc)
    g = torch.zeros((32, 32, 4), dtype=torch.float32, device="cuda")
    a = abi.AdjointArgs()
    a.grad_color = g.data_ptr()
    a.grad_color_pitch_bytes = 32 * 16
    with pytest.raises(SwgbError) as e:
        r.draw_adjoint(ds.state(), ds.args(), a)
    assert e.value.status == abi.UNSUPPORTED_STATE


def test_adjoint_of_indexed_strip(gpu_lib):
    """Triangle-strip assembly (uint16 indices) in the adjoint: vertex
    colour and position gradients against the FP64 reference."""
    import torch
    from swiftshader_gb300 import Renderer, adjoint
    sc = scenes.strip_fan_scene(abi.TOPOLOGY_TRIANGLE_STRIP, n_tris=120, indexed=np.uint16)
    sc.color_format = abi.FORMAT_R32G32B32A32_SFLOAT
    sc.cull_mode = abi.CULL_NONE
    r = Renderer(0)
    verts, _ = device_inputs(sc)
    color = adjoint.render(r, sc, verts)
    target = torch.full_like(color, 0.3)
    ((color - target) ** 2).sum().backward()
    G = (2.0 * (color - target)).detach().cpu().numpy()
    gref, _ = reference(sc, G)
    compare(gref, verts.grad, [])


def test_adjoint_sphere_full_size(gpu_lib):
    """The sphere adjoint workload at full size: the 20k-triangle uv-sphere
    (100 x 100 segments) at 512^2 RGBA32F with its 1024^2 RGBA32F texture.
    The forward through the autograd function is bit-exact against the
    oracle; every gradient group is within 1e-4 of the FP64 reference."""
    import torch
    from swiftshader_gb300 import Renderer, adjoint
    sc = scenes.scene_sphere_fp32()
    assert sc.tri_count >= 19000 and (sc.width, sc.height) == (512, 512)
    assert sc.texture_levels[0].shape[:2] == (1024, 1024)
    r = Renderer(0)
    verts, levels = device_inputs(sc)
    rng = np.random.Generator(np.random.PCG64(37))
    noisy = [l.detach() + torch.from_numpy(rng.normal(0.0, 0.05, l.shape).astype(np.float32)).cuda() for l in levels]
    with torch.no_grad():
        target = adjoint.render(r, sc, verts.detach(), noisy)
    r.reset_counters()
    color = adjoint.render(r, sc, verts, levels)
    ((color - target) ** 2).sum().backward()
    cnt = r.counters()
    assert cnt["adjoint_depth_mismatch"] == 0 and cnt["adjoint_list_overflow"] == 0
    import oracle
    c_ref, _, _ = oracle.render(sc, 8)
    assert np.array_equal(color.detach().cpu().numpy().view(np.uint32), c_ref.view(np.uint32))
    G = (2.0 * (color - target)).detach().cpu().numpy()
    gref, _ = reference(sc, G)
    compare(gref, verts.grad, [l.grad for l in levels])


def test_views_workload_full_size_view(gpu_lib):
    """One view of the 256-view workload at full size: the 100k-triangle
    noisy sphere (250 x 200 segments), 512^2 4x MSAA RGBA16F, the 2048^2
    RGBA16F 12-level chain trilinear, premultiplied OVER.  The forward is
    bit-exact against the oracle (every sample plane); the gradients through
    the batched adjoint are within 1e-4 of the FP64 reference (the rough
    surface stacks up to 60 blended fragments on one sample)."""
    import torch
    from swiftshader_gb300 import Renderer, adjoint
    sc = scenes.scene_sphere_views(0)
    sc.samples = 4
    assert sc.tri_count == 100000 and (sc.width, sc.height) == (512, 512)
    assert sc.texture_levels[0].shape[:2] == (2048, 2048)
    r = Renderer(0)
    verts, levels = device_inputs(sc)
    target = torch.full((4, 512, 512, 4), 0.25, dtype=torch.float32, device="cuda")
    r.reset_counters()
    color = adjoint.render_views(r, [sc], verts, levels)
    ((color[0] - target) ** 2).sum().backward()
    cnt = r.counters()
    assert cnt["adjoint_depth_mismatch"] == 0 and cnt["adjoint_list_overflow"] == 0
    import oracle
    c_ref, _, _ = oracle.render(sc, 8)
    got = color[0].detach().to(torch.float16).cpu().numpy()
    assert np.array_equal(got.view(np.uint16), np.asarray(c_ref, np.float16).view(np.uint16))
    G = (2.0 * (color[0] - target)).detach().cpu().numpy()
    gref, _ = reference(sc, G, cap=64)
    compare(gref, verts.grad, [l.grad for l in levels])
