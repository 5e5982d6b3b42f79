"""The sharded topology step's exchange on CPU: two gloo ranks, each holding
the candidate lists with only its own candidates solved (candidate c on rank
c % 2), all-gather and merge (optcuts_gb300.shard) -- both ranks end with the
same full lists and the same argmax as the unsharded lists."""
import os
import socket

import numpy as np
import pytest

from optcuts_gb300 import shard

torch = pytest.importorskip("torch")


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def full_lists(seed=0):
    """Two ops' full candidate lists, as an unsharded query reports them."""
    rng = np.random.default_rng(seed)
    ops = []
    for nc in (7, 12):
        ew = rng.normal(size=nc)
        ew[3] = -np.finfo(np.float64).max        # an infeasible candidate
        ops.append({"EwDec": ew, "energyChanges": rng.normal(size=(nc, 2)),
                    "path": rng.integers(0, 100, size=(nc, 3)).astype(np.int32),
                    "newVertPos": rng.normal(size=(nc, 8)), "posRows": rng.integers(1, 5, size=nc).astype(np.int32),
                    "pool": nc})
    return ops


def shard_of(full, rank, world):
    """What rank `rank` reports: its candidates solved, the rest unsolved."""
    out = []
    for d in full:
        e = {k: (np.array(v, copy=True) if k != "pool" else v) for k, v in d.items()}
        for c in range(len(e["EwDec"])):
            if c % world != rank:
                e["EwDec"][c] = -np.finfo(np.float64).max
                e["energyChanges"][c] = np.finfo(np.float64).max
        out.append(e)
    return out


def worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        full = full_lists()
        gathered = [None] * world
        dist.all_gather_object(gathered, shard_of(full, rank, world))
        merged = shard.merge(gathered)
        q.put((rank, [(m["best"], m["EwDec"].tolist(), m["energyChanges"].tolist(), m["path"].tolist())
                      for m in merged]))
    finally:
        dist.destroy_process_group()


def test_two_rank_exchange_matches_unsharded():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0] == res[1]
    full = full_lists()
    for (best, ew, ec, path), d in zip(res[0], full):
        assert best == int(np.argmax(d["EwDec"]))
        np.testing.assert_array_equal(ew, d["EwDec"])
        np.testing.assert_array_equal(ec, d["energyChanges"])
        np.testing.assert_array_equal(path, d["path"])


def test_merge_rejects_different_lists():
    full = full_lists()
    a = shard_of(full, 0, 2)
    b = shard_of(full_lists(seed=1), 1, 2)
    b[1] = {k: (v[:-1] if k != "pool" else v) for k, v in b[1].items()}
    with pytest.raises(ValueError):
        shard.merge([a, b])
