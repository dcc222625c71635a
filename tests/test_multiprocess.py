"""The N > 1 host path on CPU ranks (gloo, world size 2): the bench's
max-over-ranks timing reduction, the reference arm's rank-0-only rule, and
the sharded workloads on real data -- atlas draws split longest-processing-
time-first and rendered per rank (by the oracle, the CPU stand-in for each
rank's GPU) assemble into the single-process atlas, and per-view FP64
gradients summed by the all-reduce equal the single-process sum."""
import os
import subprocess
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    got = bench.max_over_ranks([1.0 + rank, 10.0 - rank])
    q.put((rank, got))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29517
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0] == [2.0, 10.0] and res[1] == [2.0, 10.0]


def test_reference_arm_non_zero_rank_exits_quietly():
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def _shard_main(rank, world, port, q):
    """Each rank computes the LPT partition of the atlas draws and takes its share."""
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    from swiftshader_gb300 import scenes, shard
    b = scenes.scene_batch(n_draws=200, tri_min=4, tri_max=400, sides=(32, 64, 96, 128), page_size=512, tex_size=8)
    parts = shard.lpt_partition(shard.draw_costs(b.tris, b.sides), world)
    q.put((rank, [p.tolist() for p in parts], parts[rank].tolist()))
    dist.barrier()
    dist.destroy_process_group()


def test_draw_partition_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_shard_main, args=(r, 2, 29518, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(2):
        rank, parts, mine = q.get(timeout=120)
        res[rank] = (parts, mine)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][0] == res[1][0]  # every rank computes the same partition
    a, b = res[0][1], res[1][1]
    assert sorted(a + b) == list(range(200)) and not set(a) & set(b)
    assert a == sorted(a) and b == sorted(b)  # submission order kept


def test_lpt_balance():
    import numpy as np
    from swiftshader_gb300 import scenes, shard
    c = shard.draw_costs(*scenes.batch_draw_sizes())
    for world in (2, 4, 8):
        parts = shard.lpt_partition(c, world)
        loads = np.array([c[p].sum() for p in parts])
        assert loads.max() <= loads.mean() + c.max()  # LPT bound
        assert loads.max() / loads.mean() < 1.01


def _atlas_batch():
    from swiftshader_gb300 import scenes
    return scenes.scene_batch(n_draws=24, tri_min=4, tri_max=120, sides=(32, 48, 64), page_size=128, tex_size=8)


def _render_atlas(b, draws):
    """Renders the given draws of an atlas batch into fresh atlas pages
    (each draw's viewport receives its own stand-alone render)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    P = b.page_size
    color = np.zeros((b.pages, P, P, 4), np.uint8)
    color[...] = np.asarray(b.clear_color, np.uint8)
    depth = np.full((b.pages, P, P), b.clear_depth, np.float32)
    for i in draws:
        c, d, _ = oracle.render(b.draw_scene(int(i)), 1)
        page, x, y = (int(v) for v in b.place[i])
        s = int(b.sides[i])
        color[page, y:y + s, x:x + s] = c
        depth[page, y:y + s, x:x + s] = d
    return color, depth


def _atlas_main(rank, world, port, q):
    import numpy as np
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    from swiftshader_gb300 import shard
    b = _atlas_batch()
    parts = shard.lpt_partition(shard.draw_costs(b.tris, b.sides), world)
    color, depth = _render_atlas(b, parts[rank])
    cs = [torch.zeros_like(torch.from_numpy(color)) for _ in range(world)]
    ds = [torch.zeros_like(torch.from_numpy(depth)) for _ in range(world)]
    dist.all_gather(cs, torch.from_numpy(color))
    dist.all_gather(ds, torch.from_numpy(depth))
    if rank == 0:
        # assemble: every draw's viewport from the rank that owns it
        P = b.page_size
        out_c = np.zeros((b.pages, P, P, 4), np.uint8)
        out_c[...] = np.asarray(b.clear_color, np.uint8)
        out_d = np.full((b.pages, P, P), b.clear_depth, np.float32)
        for r, idx in enumerate(parts):
            c, d = cs[r].numpy(), ds[r].numpy()
            for i in idx:
                page, x, y = (int(v) for v in b.place[i])
                s = int(b.sides[i])
                out_c[page, y:y + s, x:x + s] = c[page, y:y + s, x:x + s]
                out_d[page, y:y + s, x:x + s] = d[page, y:y + s, x:x + s]
        # a rank's pages outside its own viewports hold the clear values
        untouched = []
        for r, idx in enumerate(parts):
            m = np.ones((b.pages, P, P), bool)
            for i in idx:
                page, x, y = (int(v) for v in b.place[i])
                s = int(b.sides[i])
                m[page, y:y + s, x:x + s] = False
            untouched.append(bool((ds[r].numpy()[m] == b.clear_depth).all()))
        q.put((out_c, out_d, untouched, [p.tolist() for p in parts]))
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_atlas_assembles_to_single_render():
    import numpy as np
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_atlas_main, args=(r, 2, 29519, q)) for r in range(2)]
    for p in procs:
        p.start()
    out_c, out_d, untouched, parts = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert all(len(p) > 0 for p in parts)
    b = _atlas_batch()
    ref_c, ref_d = _render_atlas(b, range(b.n))
    assert np.array_equal(out_c, ref_c)
    assert np.array_equal(out_d.view(np.uint32), ref_d.view(np.uint32))
    assert all(untouched)
    assert (ref_d != b.clear_depth).any()


def _views():
    import numpy as np
    from swiftshader_gb300 import scenes
    rng = np.random.Generator(np.random.PCG64(4))
    mesh = scenes.uv_sphere(rng, 10, 8, noise_sigma=0.02)
    levels = scenes.float_mip_chain(rng.uniform(0.0, 1.0, (16, 16, 4)), np.float16)
    return [scenes.scene_sphere_views(v, n_views=5, width=24, height=24, mesh=mesh, levels=levels) for v in range(5)]


def _view_gradients(views, idx):
    """Sum over the views idx of the FP64 reference gradients of an L2 loss
    against a grey target (vertex colours, uvs, positions, texel levels)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import adjoint_ref
    import oracle
    total = None
    for v in idx:
        sc = views[int(v)]
        _, _, _, vis, vis_len = oracle.render_visibility(sc, 1)
        m = adjoint_ref.Model(sc, vis, vis_len)
        p = m.params()
        _, G = adjoint_ref.l2_loss(m.colors(p), np.full(m.colors(p).shape, 0.25))
        g = m.gradients(G, p)
        flat = np.concatenate([g["colors"].ravel(), g["uvs"].ravel(), g["positions"].ravel()] +
                              [lv.ravel() for lv in g["levels"]])
        total = flat if total is None else total + flat
    return total


def _views_main(rank, world, port, q):
    import numpy as np
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    from swiftshader_gb300 import shard
    views = _views()
    mine = shard.lpt_partition(np.ones(len(views)), world)[rank]
    g = torch.from_numpy(_view_gradients(views, mine))
    shard.allreduce_gradients([g])
    q.put((rank, mine.tolist(), g.numpy()))
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_view_gradients_sum_to_single_process():
    import numpy as np
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_views_main, args=(r, 2, 29520, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(2):
        rank, mine, g = q.get(timeout=300)
        res[rank] = (mine, g)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert sorted(res[0][0] + res[1][0]) == list(range(5))
    assert np.array_equal(res[0][1], res[1][1])  # every rank holds the same sum
    ref = _view_gradients(_views(), range(5))
    assert np.abs(ref).max() > 0
    # the all-reduce adds the two ranks' partial sums: equal to the
    # single-process sum up to the order of the FP64 additions
    assert np.allclose(res[0][1], ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
