"""Host logic of the multi-rank batched path (CPU, gloo, world size 2).

Each rank partitions the same seeded batch independently; the ranks then
exchange their index lists and loads: together they must cover every system
exactly once, agree on the loads, and keep the largest load within one
system's cost of the average (the longest-processing-time bound).
"""
import os
import socket

import numpy as np
import pytest


def _batch(cnt=3000, seed=12345):
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(32), np.log(1024), cnt)).astype(np.int64)
    rs = rng.integers(1, 9, cnt)
    kinds = np.arange(cnt) % 2
    return ns, rs, kinds


def _worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    from slate_gb300.partition import partition_systems, system_costs
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    ns, rs, kinds = _batch()
    costs = system_costs(ns, rs, kinds)
    parts, loads = partition_systems(costs, world)
    mine = torch.from_numpy(parts[rank])
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, torch.tensor([mine.numel()]))
    gathered = [torch.zeros(int(s.item()), dtype=torch.int64) for s in sizes]
    dist.all_gather(gathered, mine)
    my_load = torch.tensor([float(costs[parts[rank]].sum())], dtype=torch.float64)
    all_loads = [torch.zeros(1, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(all_loads, my_load)
    if rank == 0:
        allidx = np.concatenate([g.numpy() for g in gathered])
        out.put((allidx.tolist(), [float(x.item()) for x in all_loads], loads.tolist(), float(costs.max()),
                 float(costs.sum())))
    dist.barrier()
    dist.destroy_process_group()


def test_partition_two_ranks_gloo():
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    allidx, gathered_loads, loads, cmax, total = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    n = len(_batch()[0])
    assert sorted(allidx) == list(range(n))               # every system exactly once
    np.testing.assert_allclose(gathered_loads, loads)     # ranks agree on the split
    assert max(loads) - total / 2 <= cmax                 # LPT bound


def test_partition_single_rank_and_errors():
    from slate_gb300.partition import partition_systems
    parts, loads = partition_systems([3.0, 1.0, 2.0], 1)
    assert parts[0].tolist() == [0, 1, 2] and loads[0] == 6.0
    with pytest.raises(ValueError):
        partition_systems([1.0], 0)
