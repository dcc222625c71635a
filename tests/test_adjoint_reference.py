"""The FP64 adjoint reference on the CPU: its model colour against the
oracle's rendered colour (same visibility), and its analytic gradients
against central finite differences (h = 1e-3) of its own model."""
import numpy as np
import pytest

from swiftshader_gb300 import scenes


def small_sphere(blend=False, samples=1, mip=False):
    if not blend:
        return scenes.scene_sphere_fp32(seg=14, width=40, height=40, tex_size=32)
    rng = np.random.Generator(np.random.PCG64(4))
    mesh = scenes.uv_sphere(rng, 16, 12, noise_sigma=0.02)
    levels = scenes.float_mip_chain(rng.uniform(0.0, 1.0, (32, 32, 4)), np.float16)
    s = scenes.scene_sphere_views(5, width=40, height=40, mesh=mesh, levels=levels)
    s.samples = samples
    return s


def model_for(scene):
    import oracle
    import adjoint_ref
    color, depth, cnt, vis, vis_len = oracle.render_visibility(scene, 4)
    return adjoint_ref.Model(scene, vis, vis_len), color


@pytest.mark.parametrize("blend,samples", [(False, 1), (True, 1), (True, 4)])
def test_model_colour_matches_oracle(oracle_mod, blend, samples):
    """With the oracle's visibility, the model's colour is the rendered colour
    up to interpolation and attachment rounding: the model differentiates ideal
    perspective-correct interpolation at the pixel centre, the renderer
    interpolates plane equations of sub-pixel-snapped vertices (which differ
    most where a 4x MSAA edge pixel extrapolates far outside its triangle)."""
    sc = small_sphere(blend, samples)
    m, color = model_for(sc)
    mc = m.colors()
    rendered = color.astype(np.float64).reshape(mc.shape)
    d = np.abs(mc - rendered).max(-1)[(m.e_s, m.e_y, m.e_x)]
    assert d.size > 0
    assert np.percentile(d, 99) < 3e-3
    assert (d > 1e-2).mean() < 0.01


@pytest.mark.parametrize("blend,samples", [(False, 1), (True, 4)])
def test_reference_gradients_match_central_differences(oracle_mod, blend, samples):
    import adjoint_ref
    sc = small_sphere(blend, samples)
    m, _ = model_for(sc)
    p = m.params()
    rng = np.random.Generator(np.random.PCG64(99))
    target = m.colors(p) + rng.normal(0.0, 0.05, m.colors(p).shape)
    _, G = adjoint_ref.l2_loss(m.colors(p), target)
    g = m.gradients(G, p)
    h = 1e-3

    def loss(pp):
        return adjoint_ref.l2_loss(m.colors(pp), target)[0]

    def directional(key, d, level=None, step=h):
        pp = {k: (v if k != "levels" else list(v)) for k, v in p.items()}
        pm = {k: (v if k != "levels" else list(v)) for k, v in p.items()}
        if level is None:
            pp[key] = p[key] + step * d
            pm[key] = p[key] - step * d
        else:
            pp["levels"][level] = p["levels"][level] + step * d
            pm["levels"][level] = p["levels"][level] - step * d
        return (loss(pp) - loss(pm)) / (2 * step)

    # texels and vertex colours: the shaded colour is linear in them, so
    # without blending the loss is quadratic and the h = 1e-3 quotient exact
    # to rounding; OVER multiplies shaded colours (O(h^2) terms remain)
    tol = 1e-4 if blend else 1e-7
    for lv in range(len(p["levels"])):
        d = rng.normal(0.0, 1.0, p["levels"][lv].shape)
        fd = directional("levels", d, level=lv)
        an = float((g["levels"][lv] * d).sum())
        assert abs(fd - an) <= tol * max(abs(an), 1e-2), (lv, fd, an)
    d = rng.normal(0.0, 1.0, p["colors"].shape)
    fd, an = directional("colors", d), float((g["colors"] * d).sum())
    assert abs(fd - an) <= tol * max(abs(an), 1e-2)
    # non-linear: texture coordinates and positions.  At h = 1e-3 the quotient
    # straddles texel-centre kinks of the bilinear filter (and, with 4x MSAA,
    # steep extrapolation at edge samples), so the derivative is checked as
    # the FP64 quotient converges, at h = 1e-8.
    for key in ("uvs", "positions"):
        d = rng.normal(0.0, 1.0, p[key].shape)
        if key == "positions":
            d[:, 3] = 0.0
        an = float((g[key] * d).sum())
        fd = directional(key, d, step=1e-8)
        assert abs(fd - an) <= 1e-5 * max(abs(an), 1e-3 * np.abs(g[key]).sum()), (key, fd, an)
