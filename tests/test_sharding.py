"""Multi-rank host logic on CPU with gloo (world size 2): trace-range
sharding of bench.py (weak scaling, no data-path collective) and the scalar
reductions it performs (sum of pairs, max of elapsed time)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import torch
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    batches = bench.shard_steps(2000, 8, 5, 3, rank, world)
    pairs = torch.tensor([float(sum(n for _, n in batches[3:]))], dtype=torch.float64)
    t = torch.tensor([1.0 + rank], dtype=torch.float64)
    dist.all_reduce(pairs, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    gathered = [None] * world
    dist.all_gather_object(gathered, batches)
    if rank == 0:
        q.put((pairs.item(), t.item(), gathered))
    dist.destroy_process_group()


def test_two_rank_sharding_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    pairs, tmax, gathered = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert pairs == 2 * 5 * 8          # both ranks' timed traces are counted
    assert tmax == 2.0                 # the slowest rank sets the time
    starts0 = {s for s, _ in gathered[0]}
    starts1 = {s for s, _ in gathered[1]}
    assert not (starts0 & starts1)     # disjoint stretches of the track
    for b in gathered:
        assert all(0 <= s and s + n <= 2000 for s, n in b)


def test_shard_steps_single_rank():
    import bench
    b = bench.shard_steps(2000, 8, 10, 3, 0, 1)
    assert len(b) == 13 and b[0] == (500, 8) and b[1] == (508, 8)
    assert all(500 <= s and s + n <= 1500 for s, n in b)
