"""Sharding of batched systems across ranks: two gloo ranks on the CPU each
take their share of the 256 seeded immersed-boundary systems; the shares
are disjoint, cover every system, and the heaviest rank stays within the
largest system of the mean load."""
import os
import socket

import numpy as np
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from phase_gb300 import shard, workloads


def _sizes():
    return [5 * s["nx"] * s["ny"] for s in workloads.gcib_specs(256, seed=5)]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = shard.my_share(_sizes(), rank, world)
    t = torch.zeros(256, dtype=torch.int64)
    t[mine] = rank + 1
    out = [torch.zeros_like(t) for _ in range(world)]
    dist.all_gather(out, t)
    if rank == 0:
        q.put(torch.stack(out).numpy())
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_split_the_batch():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    tab = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    owners = (tab > 0).sum(axis=0)
    assert np.all(owners == 1)                  # disjoint and complete
    sizes = np.array(_sizes())
    loads = [sizes[tab[r] > 0].sum() for r in range(2)]
    assert max(loads) <= sizes.sum() / 2 + sizes.max()


def test_partition_is_deterministic_and_greedy():
    sizes = [7, 3, 9, 1, 4, 4, 8]
    p = shard.partition_by_nnz(sizes, 3)
    assert p == shard.partition_by_nnz(sizes, 3)
    assert sorted(sum(p, [])) == list(range(len(sizes)))
    assert shard.partition_by_nnz(sizes, 1) == [list(range(len(sizes)))]
