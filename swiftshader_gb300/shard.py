"""Multi-GPU partition of independent draws and views (one process per GPU).

A single frame is not split: it runs as a replica per GPU.  Work made of
independent draws is split instead:

* atlas draws: each draw goes to one rank by longest-processing-time-first
  on its estimated cost (triangles x viewport area); a rank draws its share
  with one swgb_draw_batch call into its own copy of the atlas pages, and the
  shares touch disjoint viewports, so the data path needs no collective;
* views of one scene (the adjoint workload): views are partitioned the same
  way; each rank runs the forward and the adjoint of its views, then one
  all_reduce(sum) of the vertex and texel gradients gives every rank the
  gradient of all views.

Every function here is host logic; the collective is torch.distributed's
(NCCL between GPUs, gloo on CPU in the tests).
"""
import numpy as np


def lpt_partition(costs, world):
    """Longest-processing-time-first: items in decreasing cost (ties by
    index) go to the rank with the least load so far (ties to the lowest
    rank).  Returns one ascending index array per rank, so each rank keeps
    the submission order of its items.  Deterministic on every rank."""
    costs = np.asarray(costs, np.float64)
    if world < 1:
        raise ValueError("world must be >= 1")
    order = np.lexsort((np.arange(len(costs)), -costs))
    load = np.zeros(world)
    owner = np.empty(len(costs), np.int64)
    for i in order:
        r = int(np.argmin(load))
        owner[i] = r
        load[r] += costs[i]
    return [np.nonzero(owner == r)[0] for r in range(world)]


def draw_costs(tris, sides):
    """Estimated cost of each draw: triangles x viewport area."""
    return np.asarray(tris, np.float64) * np.asarray(sides, np.float64) ** 2


def allreduce_gradients(tensors, group=None):
    """Sums gradient tensors over all ranks in place (no-op on one rank)."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size(group) == 1:
        return tensors
    for t in tensors:
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return tensors
