"""Instance-level data parallelism across ranks (one process per GPU).

Instances of a batch are independent, so a multi-GPU run shards them across ranks with no
data-path collective: each rank solves its shard and the results are gathered on the host.
Shards are balanced by an instance cost estimate (greedy longest-processing-time assignment).
"""
import numpy as np


def instance_cost(qp):
    """Work estimate of one instance: dense root factorisation + sparse residual passes."""
    nr = qp.n + qp.zero
    return nr ** 3 / 6.0 + 30.0 * (2 * qp.P.nnz + 2 * qp.A.nnz + 9 * qp.m)


def shard_indices(costs, world_size):
    """Greedy LPT assignment: returns a list of index arrays, one per rank, each sorted."""
    costs = np.asarray(costs, dtype=float)
    load = np.zeros(world_size)
    owner = np.empty(len(costs), dtype=np.int64)
    for i in np.argsort(-costs, kind="stable"):
        r = int(np.argmin(load))
        owner[i] = r
        load[r] += costs[i]
    return [np.sort(np.where(owner == r)[0]) for r in range(world_size)]


def gather_solutions(local_idx, local_x, local_status, count, group=None):
    """All-gather per-instance results (host side, torch.distributed, any backend).

    local_x: list of 1-D float64 arrays (one per local instance); returns (x list, status array)
    indexed by global instance id on every rank."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    payload = {"idx": np.asarray(local_idx).tolist(), "x": [np.asarray(v).tolist() for v in local_x],
               "status": np.asarray(local_status).tolist()}
    gathered = [None] * world
    dist.all_gather_object(gathered, payload, group=group)
    xs = [None] * count
    status = np.zeros(count, dtype=np.int64)
    for part in gathered:
        for i, xv, st in zip(part["idx"], part["x"], part["status"]):
            xs[i] = np.asarray(xv)
            status[i] = st
    del torch
    return xs, status
