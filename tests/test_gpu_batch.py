"""Batched draws (swgb_draw_batch) against the same draws issued one by one
(swgb_draw), bit for bit: colour, depth and every counter.  The per-draw
path is itself checked against the oracle in test_gpu_parity.py; a few atlas
draws are also checked against the oracle directly here."""
import numpy as np
import pytest

from swiftshader_gb300 import abi, scenes

from gpu_helpers import assert_bit_exact, render_oracle

pytestmark = pytest.mark.gpu


def small_batch(n_draws=96, seed_index=21, page_size=512):
    return scenes.scene_batch(n_draws=n_draws, tri_min=4, tri_max=600, sides=(32, 64, 96, 128), page_size=page_size,
                              tex_size=32, seed_index=seed_index)


def run_atlas(db, r, batched):
    import torch
    db.clear()
    torch.cuda.synchronize()
    r.reset_counters()
    if batched:
        db.draw_batch(r)
    else:
        db.draw_each(r)
    r.synchronize()
    return db.color.cpu().numpy(), db.depth.cpu().numpy(), r.counters()


@pytest.mark.parametrize("n_draws,page_size", [(96, 512), (300, 256)])
def test_atlas_batch_equals_per_draw(gpu_lib, n_draws, page_size):
    """Independent draws into disjoint atlas viewports (one or several
    pages), each with its own texture: one batch equals the per-draw loop."""
    from swiftshader_gb300 import DeviceBatch, Renderer
    b = small_batch(n_draws, page_size=page_size)
    db = DeviceBatch(b)
    r = Renderer(0)
    c1, d1, k1 = run_atlas(db, r, batched=False)
    c2, d2, k2 = run_atlas(db, r, batched=True)
    assert_bit_exact(d2, d1, "depth")
    assert_bit_exact(c2, c1, "color")
    assert k1 == k2
    assert k1["triangles_in"] == int(b.tris.sum())
    # replaying the captured graph gives the same bits again
    c3, d3, k3 = run_atlas(db, r, batched=True)
    assert_bit_exact(c3, c1, "color (graph replay)")
    assert_bit_exact(d3, d1, "depth (graph replay)")
    assert k3 == k1


def test_atlas_batch_against_oracle(gpu_lib):
    """Atlas viewports of the batched run against the oracle rendering each
    draw into its own framebuffer."""
    from swiftshader_gb300 import DeviceBatch, Renderer
    b = small_batch(64, seed_index=22)
    db = DeviceBatch(b)
    r = Renderer(0)
    run_atlas(db, r, batched=True)
    order = np.argsort(b.tris)
    for i in (int(order[0]), int(order[len(order) // 2]), int(order[-1])):
        c, d = db.view(i)
        c_ref, d_ref, _ = render_oracle(b.draw_scene(i))
        assert_bit_exact(d.cpu().numpy(), d_ref, "depth of draw %d" % i)
        assert_bit_exact(c.cpu().numpy(), c_ref, "color of draw %d" % i)


def shared_target_draws(n=6, width=80, height=64, seed=60):
    """n textured draws, half of them blended, some scissored, all into one
    attachment pair: every draw depends on the ones before it."""
    out = []
    for k in range(n):
        s = scenes.scene_textured_small(n_tris=60 + 10 * k, width=width, height=height, tex_size=32, mip=True,
                                        blend=(k % 2 == 1), seed_index=seed + k)
        if k % 3 == 2:
            s.scissor = (8 * k % width, 4 * k % height, width // 2, height // 2)
        out.append(s)
    return out


class Target:
    """One colour + depth attachment pair shared by several scenes."""

    def __init__(self, scene):
        from swiftshader_gb300 import DeviceScene
        self.ds = DeviceScene(scene)

    def state_for(self, ds):
        return scenes.build_state(ds.scene, self.ds.color.data_ptr(), self.ds.depth.data_ptr(), ds.vertices.data_ptr(),
                                  [l.data_ptr() for l in ds.levels])


def run_list(r, targets, states, args, batched):
    import torch
    for t in targets:
        t.ds.clear()
    torch.cuda.synchronize()
    r.reset_counters()
    if batched:
        r.draw_batch(states, args)
    else:
        for s, a in zip(states, args):
            r.draw(s, a)
    r.synchronize()
    out = []
    for t in targets:
        out += [t.ds.color.cpu().numpy(), t.ds.depth.cpu().numpy()]
    return out, r.counters()


def assert_runs_equal(r, targets, states, args):
    seq, k1 = run_list(r, targets, states, args, batched=False)
    bat, k2 = run_list(r, targets, states, args, batched=True)
    for i, (a, b) in enumerate(zip(bat, seq)):
        assert_bit_exact(a, b, "attachment %d" % i)
    assert k1 == k2
    return k1


def test_dependent_draws_keep_submission_order(gpu_lib):
    """Draws into the same attachments (blend, depth) are split into
    segments at each dependency, so the result is the sequential one."""
    from swiftshader_gb300 import DeviceScene, Renderer
    draws = shared_target_draws()
    dss = [DeviceScene(s) for s in draws]
    tgt = Target(draws[0])
    states = [tgt.state_for(ds) for ds in dss]
    args = [ds.args() for ds in dss]
    assert_runs_equal(Renderer(0), [tgt], states, args)


def test_mixed_formats_and_samples(gpu_lib):
    """RGBA8, RGBA16F, RGBA32F and 4x MSAA draws interleaved in one call, some
    onto the same attachments as earlier ones, plus empty draws."""
    from swiftshader_gb300 import DeviceScene, Renderer
    variants = []
    for fmt, samples in [(abi.FORMAT_R8G8B8A8_UNORM, 1), (abi.FORMAT_R16G16B16A16_SFLOAT, 1),
                         (abi.FORMAT_R8G8B8A8_UNORM, 4), (abi.FORMAT_R32G32B32A32_SFLOAT, 1),
                         (abi.FORMAT_R16G16B16A16_SFLOAT, 4)]:
        s = scenes.scene_textured_small(n_tris=120, width=72, height=56, tex_size=32, mip=True, blend=True,
                                        seed_index=70 + len(variants))
        s.color_format = fmt
        s.samples = samples
        s.clear_color = (10, 20, 30, 40) if fmt == abi.FORMAT_R8G8B8A8_UNORM else (0.1, 0.2, 0.3, 0.4)
        variants.append(s)
    dss = [DeviceScene(s) for s in variants]
    targets = [Target(s) for s in variants]
    states, args = [], []
    order = [0, 1, 2, 0, 3, 4, 2, 1, 0]   # revisits attachments 0, 1, 2
    for k in order:
        states.append(targets[k].state_for(dss[k]))
        args.append(dss[k].args())
    empty = dss[0].args()
    empty.count = 0
    states.insert(4, targets[0].state_for(dss[0]))
    args.insert(4, empty)
    k = assert_runs_equal(Renderer(0), targets, states, args)
    assert k["fragments_passed"] > 0


def test_batch_many_small_disjoint_draws_one_target(gpu_lib):
    """Many draws with disjoint scissors on one shared attachment: one segment."""
    from swiftshader_gb300 import DeviceScene, Renderer
    W, H = 256, 128
    draws = []
    for k in range(32):
        s = scenes.scene_small(n_tris=40, width=W, height=H, seed_index=80 + k)
        s.scissor = ((k % 8) * 32, (k // 8) * 32, 32, 32)
        draws.append(s)
    dss = [DeviceScene(s) for s in draws]
    tgt = Target(draws[0])
    states = [tgt.state_for(ds) for ds in dss]
    args = [ds.args() for ds in dss]
    r = Renderer(0)
    r.set_kernel_timing(True)
    r.kernel_times()
    k = assert_runs_equal(r, [tgt], states, args)
    assert k["triangles_in"] == 32 * 40
    # with kernel timing on, the batch runs as three direct launches
    times = r.kernel_times()
    assert times["vertex"][1] == 33 and times["raster"][1] >= 33


def test_batch_span_scratch_fallback(gpu_lib, monkeypatch):
    """Span-row scratch exhausted inside a batch: triangles beyond it walk
    their edges in the raster kernel, same bits as the per-draw path."""
    from swiftshader_gb300 import DeviceBatch, Renderer
    monkeypatch.setenv("SWGB_SPAN_ROWS", "900")
    b = small_batch(40, seed_index=23)
    db = DeviceBatch(b)
    r = Renderer(0)
    c1, d1, k1 = run_atlas(db, r, batched=False)
    c2, d2, k2 = run_atlas(db, r, batched=True)
    assert_bit_exact(d2, d1, "depth")
    assert_bit_exact(c2, c1, "color")
    assert k1 == k2


def test_batch_scratch_growth_recaptures(gpu_lib):
    """A larger batch after a smaller one grows the scratch (the graph is
    captured again); the smaller batch afterwards still matches."""
    from swiftshader_gb300 import DeviceBatch, Renderer
    r = Renderer(0)
    small = DeviceBatch(small_batch(24, seed_index=24))
    big = DeviceBatch(small_batch(200, seed_index=25, page_size=1024))
    ref_small = run_atlas(small, r, batched=False)
    ref_big = run_atlas(big, r, batched=False)
    for db, ref in ((small, ref_small), (big, ref_big), (small, ref_small)):
        c, d, k = run_atlas(db, r, batched=True)
        assert_bit_exact(c, ref[0], "color")
        assert_bit_exact(d, ref[1], "depth")
        assert k == ref[2]


def test_full_atlas_sample_against_oracle(gpu_lib):
    """The full 4096-draw atlas workload (triangle counts log-uniform in
    [16, 65536], 16384^2 pages) as one swgb_draw_batch, then a seeded sample
    of its draws -- the largest ones included -- against the oracle drawing
    each into its own framebuffer, bit for bit; and the batch's triangle
    counter against the draws' total."""
    import torch
    from swiftshader_gb300 import DeviceBatch, Renderer
    b = scenes.scene_batch()
    db = DeviceBatch(b)
    r = Renderer(0)
    db.clear()
    torch.cuda.synchronize()
    r.reset_counters()
    db.draw_batch(r)
    r.synchronize()
    cnt = r.counters()
    assert cnt["triangles_in"] == int(b.tris.sum())
    rng = np.random.Generator(np.random.PCG64(12))
    sample = list(rng.choice(b.n, 16, replace=False)) + list(np.argsort(b.tris)[-2:])
    for i in sample:
        c_ref, d_ref, _ = render_oracle(b.draw_scene(int(i)), 8)
        c, d = db.view(int(i))
        assert_bit_exact(d.cpu().numpy(), d_ref, "depth of draw %d" % i)
        assert_bit_exact(c.cpu().numpy(), c_ref, "colour of draw %d" % i)
    del db
    torch.cuda.empty_cache()
