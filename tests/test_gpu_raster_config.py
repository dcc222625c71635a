"""Raster configurations (bin shape x depth rejection) and the autotuner.

Every configuration must give the oracle's attachments and counters bit for
bit: the bin shape only changes how the framebuffer is split among warps, and
the hierarchical depth rejection only skips fragments it can prove fail (it
still counts them as tested)."""
import numpy as np
import pytest

from swiftshader_gb300 import abi, scenes

from gpu_helpers import assert_bit_exact, render_gpu, render_oracle
from test_gpu_batch import run_atlas, small_batch
from test_gpu_parity import assert_counters

pytestmark = pytest.mark.gpu

CONFIGS = [(w, h, hiz) for (w, h) in abi.BIN_SHAPES for hiz in (True, False)]


def check_config(scene, cfg):
    from swiftshader_gb300 import Renderer
    r = Renderer(0)
    r.set_raster_config(*cfg)
    assert r.raster_config() == {"bin": "%dx%d" % cfg[:2], "hiz": int(cfg[2])}
    c_gpu, d_gpu, cnt_gpu = render_gpu(scene, renderer=r)
    c_ref, d_ref, cnt_ref = render_oracle(scene)
    assert_bit_exact(d_gpu, d_ref, "depth %r" % (cfg,))
    assert_bit_exact(c_gpu, c_ref, "color %r" % (cfg,))
    assert_counters(cnt_gpu, cnt_ref)
    return cnt_ref


def layered_scene(compare_op, clear_depth, seed=61):
    """Stacks of large constant-depth triangles a few ulps apart, and equal:
    the depth bound meets fragment depths within its rounding margin."""
    s = scenes.scene_small(n_tris=240, width=100, height=70, seed_index=seed)
    rng = np.random.Generator(np.random.PCG64(seed))
    v = s.vertices
    base = np.float32(0.5)
    for t in range(240):
        z = np.nextafter(base, np.float32(2.0) if t % 3 else np.float32(-2.0)) if t % 5 else base
        v[3 * t:3 * t + 3, 2] = z
        if t % 2:
            v[3 * t:3 * t + 3, 0:2] = np.array([[-1.2, -1.2], [1.3, -1.1], [-0.9, 1.4]], np.float32)
    v[:, 2] += rng.integers(0, 2, v.shape[0]).astype(np.float32) * np.float32(1e-7) * (np.arange(v.shape[0]) % 7 == 0)
    s.depth_compare = compare_op
    s.clear_depth = clear_depth
    return s


@pytest.mark.parametrize("cfg", CONFIGS, ids=lambda c: "%dx%d-hiz%d" % (c[0], c[1], c[2]))
def test_configs_untextured(gpu_lib, cfg):
    """Ragged and dense Gouraud scenes, viewport and scissor offsets."""
    check_config(scenes.scene_small(), cfg)
    check_config(scenes.scene_small(n_tris=2000, width=96, height=96, seed_index=14), cfg)
    s = scenes.scene_small(n_tris=300, width=160, height=120, seed_index=23)
    s.viewport = (10, -5, 130, 110)
    s.scissor = (7, 9, 101, 77)
    check_config(s, cfg)


@pytest.mark.parametrize("cfg", CONFIGS, ids=lambda c: "%dx%d-hiz%d" % (c[0], c[1], c[2]))
def test_configs_textured_and_heightfield(gpu_lib, cfg):
    check_config(scenes.scene_textured_small(), cfg)
    check_config(scenes.scene_heightfield(quads_x=160, quads_y=80, width=320, height=180, tex_size=256), cfg)


@pytest.mark.parametrize("cfg", [(16, 16, True), (32, 16, True), (32, 32, True)], ids=lambda c: "%dx%d" % c[:2])
def test_depth_bound_edge_cases(gpu_lib, cfg):
    """Every compare op; layers equal to and one ulp from each other and from
    the clear depth; NaN in the depth attachment."""
    for op in range(8):
        s = scenes.scene_small(n_tris=120, width=64, height=48, seed_index=25)
        s.depth_compare = op
        s.clear_depth = 0.5
        check_config(s, cfg)
    for op in (abi.COMPARE_LESS, abi.COMPARE_LESS_OR_EQUAL, abi.COMPARE_GREATER, abi.COMPARE_GREATER_OR_EQUAL):
        check_config(layered_scene(op, 0.5), cfg)
        check_config(layered_scene(op, float(np.nextafter(np.float32(0.5), np.float32(1.0)))), cfg)
        check_config(layered_scene(op, float("nan")), cfg)


@pytest.mark.parametrize("cfg", [(32, 16, True), (32, 32, False)], ids=lambda c: "%dx%d-hiz%d" % c)
def test_configs_msaa_and_float(gpu_lib, cfg):
    """Four-sample draws keep 16x16 bins but take the context's depth-rejection
    setting; float attachments run the shape's other kernels."""
    s = scenes.scene_small(n_tris=300, width=72, height=56, seed_index=42)
    s.samples = 4
    check_config(s, cfg)
    s = scenes.scene_textured_small(n_tris=180, width=80, height=64, tex_size=32, blend=False, seed_index=31)
    s.color_format = abi.FORMAT_R32G32B32A32_SFLOAT
    s.clear_color = (0.1, 0.2, 0.3, 0.4)
    check_config(s, cfg)


@pytest.mark.parametrize("cfg", [(32, 32, True), (16, 16, False), (32, 16, True)], ids=lambda c: "%dx%d-hiz%d" % c)
def test_configs_batch_equals_per_draw(gpu_lib, cfg):
    """Atlas viewports in one swgb_draw_batch under a non-default configuration
    equal the default-configured per-draw result."""
    from swiftshader_gb300 import DeviceBatch, Renderer
    db = DeviceBatch(small_batch(160, seed_index=51))
    c1, d1, k1 = run_atlas(db, Renderer(0), batched=False)
    r = Renderer(0)
    r.set_raster_config(*cfg)
    c2, d2, k2 = run_atlas(db, r, batched=True)
    assert_bit_exact(d2, d1, "depth")
    assert_bit_exact(c2, c1, "color")
    assert k1 == k2


@pytest.mark.parametrize("batched", [True, False])
def test_autotune_leaves_one_run(gpu_lib, batched):
    """swgb_autotune times every candidate, keeps the fastest, and leaves the
    attachments and counters as one run of the draws would."""
    import torch
    from swiftshader_gb300 import DeviceBatch, Renderer
    db = DeviceBatch(small_batch(120, seed_index=52))
    c1, d1, k1 = run_atlas(db, Renderer(0), batched=True)
    r = Renderer(0)
    db.clear()
    torch.cuda.synchronize()
    r.reset_counters()
    from swiftshader_gb300.tuning import TuningTable, workload_class
    tt = TuningTable()
    best, table = r.autotune(db.states, db.args, batched=batched, runs=3, table=tt)
    r.synchronize()
    assert len(table) == abi.AUTOTUNE_CANDIDATES
    assert all(0.0 < t["min"] <= t["median"] <= t["max"] for _, t in table)
    assert best == min(table, key=lambda e: e[1]["median"])[0]
    assert r.raster_config() == best
    assert_bit_exact(db.depth.cpu().numpy(), d1, "depth")
    assert_bit_exact(db.color.cpu().numpy(), c1, "color")
    assert r.counters() == k1
    # a table hit sets the recorded configuration without running the draws
    assert workload_class(db.states, db.args, batched) in tt
    r2 = Renderer(0)
    r2.set_raster_config(16, 16, True) if best != {"bin": "16x16", "hiz": 1} else r2.set_raster_config(32, 32, False)
    before = db.depth.clone()
    best2, _ = r2.autotune(db.states, db.args, batched=batched, table=tt)
    torch.cuda.synchronize()
    assert best2 == best and r2.raster_config() == best
    assert torch.equal(db.depth, before)


def clustered_scene(n, width, height, seed):
    s = scenes.scene_small(n_tris=n, width=width, height=height, seed_index=seed)
    rng = np.random.Generator(np.random.PCG64(seed))
    v = s.vertices
    centers = rng.uniform(-1.0, 1.0, (n, 2)) ** 3  # denser towards the middle
    v[:, 0:2] = (np.repeat(centers, 3, axis=0) + rng.uniform(-0.03, 0.03, (3 * n, 2))).astype(np.float32)
    return s


@pytest.mark.parametrize("cfg", [(16, 16, True), (16, 16, False), (32, 16, True)], ids=lambda c: "%dx%d-hiz%d" % c)
def test_longest_first_bin_order(gpu_lib, cfg):
    """Frames with more bins than resident raster warps take the heaviest-first
    bin order (per-bin triangle counts and spread triangle area from the setup
    stage): small triangles clustered unevenly over a 1920x1088 frame, empty
    bins included."""
    check_config(clustered_scene(20000, 1920, 1088, 71), cfg)


@pytest.mark.parametrize("fmt", [abi.FORMAT_R8G8B8A8_UNORM, abi.FORMAT_R32G32B32A32_SFLOAT], ids=["rgba8", "rgba32f"])
def test_split_bins_with_offsets(gpu_lib, fmt):
    """Bins heavy enough to be queued as their top and bottom halves
    (triangles clustered in the middle of the frame), under a viewport and a
    scissor that are not aligned to the bins, with 8-bit and float colour
    attachments (each half stages and writes back only its rows)."""
    s = clustered_scene(20000, 1920, 1088, 75)
    s.viewport = (13, -7, 1900, 1080)
    s.scissor = (5, 11, 1890, 1060)
    if fmt != abi.FORMAT_R8G8B8A8_UNORM:
        s.color_format = fmt
        s.clear_color = (0.0, 0.0, 0.0, 0.0)
    check_config(s, (16, 16, False))


def test_bin_order_by_count_only(gpu_lib):
    """A bin grid too large for both difference arrays in the order kernel's
    shared memory (171 x 171 cells of 16x16 bins) orders by triangle count
    alone."""
    check_config(clustered_scene(20000, 2720, 2720, 73), (16, 16, False))


@pytest.mark.parametrize("cfg", [(16, 16, True), (32, 32, True)], ids=lambda c: "%dx%d" % c[:2])
def test_depth_bound_d16(gpu_lib, cfg):
    """The depth bound on a D16_UNORM attachment (quantized like the fragments)."""
    for op in (abi.COMPARE_LESS, abi.COMPARE_LESS_OR_EQUAL, abi.COMPARE_GREATER, abi.COMPARE_GREATER_OR_EQUAL):
        s = layered_scene(op, 0.5)
        s.depth_format = abi.FORMAT_D16_UNORM
        check_config(s, cfg)
    s = scenes.scene_small(n_tris=2000, width=96, height=96, seed_index=14)
    s.depth_format = abi.FORMAT_D16_UNORM
    check_config(s, cfg)
