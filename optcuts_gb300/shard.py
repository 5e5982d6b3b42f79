"""The topology step's candidates sharded over processes, one GPU each.

The reference evaluates every split / merge candidate of a topology step on
its host threads (TriMesh::querySplit / queryMerge, src/TriMesh.cpp:548-951)
and applies the one with the largest E_w decrease.  The candidates are
independent, so each process (rank r of n) enumerates the same candidate
lists on its own copy of the state and solves only candidates c with
c % n == r (oc_topology_queries_sharded); one all-gather of the per-candidate
results then gives every rank the full lists (energyChanges, paths,
newVertPos -- what the critical-lambda scheme re-ranks) and the same argmax.
No device collective is involved: the exchange is one host all-gather per
step over torch.distributed (gloo or NCCL's object path).
"""
from __future__ import annotations

import numpy as np

KEYS = ("EwDec", "energyChanges", "path", "newVertPos", "posRows")


def merge(per_rank):
    """per_rank[r] = the list of per-op dicts rank r produced (the same ops in
    the same order).  Returns one merged dict per op: candidate c taken from
    rank c % n, plus 'best' (the first index of the largest EwDec, -1 when
    there is no candidate) and 'EwDec_max'."""
    n = len(per_rank)
    merged = []
    for op in range(len(per_rank[0])):
        lists = [per_rank[r][op] for r in range(n)]
        nc = len(lists[0]["EwDec"])
        if any(len(l["EwDec"]) != nc for l in lists):
            raise ValueError("shards enumerated different candidate lists")
        out = {k: np.array(lists[0][k], copy=True) for k in KEYS}
        out["pool"] = lists[0]["pool"]
        for c in range(nc):
            src = lists[c % n]
            for k in KEYS:
                out[k][c] = src[k][c]
        best = int(np.argmax(out["EwDec"])) if nc else -1
        out["best"] = best
        out["EwDec_max"] = float(out["EwDec"][best]) if best >= 0 else 0.0
        merged.append(out)
    return merged


def topology_step(mesh, lambda_t, rank=None, world=None, group=None, filterExp=0.6, fp32=False, ops=(0, 2, 1)):
    """One topology step's queries split over the ranks of a
    torch.distributed group; every rank returns the same merged lists."""
    import torch.distributed as dist
    if world is None:
        world = dist.get_world_size(group) if dist.is_initialized() else 1
    if rank is None:
        rank = dist.get_rank(group) if dist.is_initialized() else 0
    mine = mesh.topologyStepShard(lambda_t, rank, world, filterExp=filterExp, fp32=fp32, ops=ops)
    if world == 1:
        return merge([mine])
    gathered = [None] * world
    dist.all_gather_object(gathered, mine, group=group)
    return merge(gathered)
