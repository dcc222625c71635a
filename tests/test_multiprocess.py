"""The N > 1 host path on CPU ranks (gloo, world size 2): the bench's
max-over-ranks timing reduction, and the reference arm's rank-0-only rule."""
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
    """Each rank takes its LPT share of the atlas draws and of the views, and
    sums its views' (stand-in) gradients with the other rank's."""
    import numpy as np
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    from swiftshader_gb300 import scenes, shard
    b = scenes.scene_batch(n_draws=200, tri_min=4, tri_max=400, sides=(32, 64, 96, 128), page_size=512, tex_size=8)
    parts = shard.lpt_partition(shard.draw_costs(b.tris, b.sides), world)
    mine = parts[rank]
    # views: gradient of view v stands in as v * ones; the all-reduce sums all views
    views = shard.lpt_partition(np.ones(7), world)[rank]
    g = torch.zeros(16, dtype=torch.float64)
    for v in views:
        g += float(v)
    shard.allreduce_gradients([g])
    q.put((rank, [p.tolist() for p in parts], mine.tolist(), g.tolist()))
    dist.barrier()
    dist.destroy_process_group()


def test_draw_and_view_partition_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_shard_main, args=(r, 2, 29518, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(2):
        rank, parts, mine, g = q.get(timeout=120)
        res[rank] = (parts, mine, g)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][0] == res[1][0]  # every rank computes the same partition
    a, b = res[0][1], res[1][1]
    assert sorted(a + b) == list(range(200)) and not set(a) & set(b)
    assert a == sorted(a) and b == sorted(b)  # submission order kept
    assert res[0][2] == res[1][2] == [float(sum(range(7)))] * 16


def test_lpt_balance():
    import numpy as np
    from swiftshader_gb300 import scenes, shard
    c = shard.draw_costs(*scenes.batch_draw_sizes())
    for world in (2, 4, 8):
        parts = shard.lpt_partition(c, world)
        loads = np.array([c[p].sum() for p in parts])
        assert loads.max() <= loads.mean() + c.max()  # LPT bound
        assert loads.max() / loads.mean() < 1.01
