"""Sharding of independent solves across ranks: host logic, world_size 2 over gloo.

Each rank derives its share from the same solve list; the shares must be disjoint,
cover every solve, and be balanced.  Runs as two CPU processes (gloo backend).
"""
import os

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from qsf_gb300 import shard


def _costs(seed=0, n=256):
    rng = np.random.default_rng(seed)
    edges = rng.choice([256, 384, 512, 768, 1024], n)
    lam = rng.uniform(400.0, 1600.0, n)
    steps = (3 * 2 * np.pi / (45.563352529 / lam) / 0.05).astype(int) + 2
    return [shard.cost(int(e) * int(e), int(s)) for e, s in zip(edges, steps)]


def test_partition_covers_and_balances():
    c = _costs()
    for ws in (1, 2, 4, 8):
        parts = shard.partition(c, ws)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(c)))
        assert shard.imbalance(c, parts) < 1.02


def _worker(rank, ws, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    c = _costs()
    mine = shard.my_share(c, ws, rank)
    t = torch.zeros(len(c), dtype=torch.int64)
    t[mine] = 1
    dist.all_reduce(t)
    load = torch.tensor([sum(c[i] for i in mine)], dtype=torch.float64)
    loads = [torch.zeros(1, dtype=torch.float64) for _ in range(ws)]
    dist.all_gather(loads, load)
    if rank == 0:
        q.put((t.tolist(), [float(x.item()) for x in loads]))
    dist.destroy_process_group()


def _bench_worker(rank, ws, port, q):
    """The batched bench's own assignment (bench.batch_specs / bench.batch_share) and
    the served bench's stream assignment (shard.StreamAssigner), each rank on its own."""
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    specs = bench.batch_specs(256, 0)
    mine = bench.batch_share(specs, 23, ws, rank)
    t = torch.zeros(len(specs), dtype=torch.int64)
    t[mine] = 1
    dist.all_reduce(t)
    rng = np.random.default_rng(5)
    stream_costs = [float(rng.choice([1024, 4096, 65536, 262144])) * 256 for _ in range(500)]
    a = shard.StreamAssigner(ws)
    mine_s = [i for i, c in enumerate(stream_costs) if a.assign(c) == rank]
    u = torch.zeros(len(stream_costs), dtype=torch.int64)
    u[mine_s] = 1
    dist.all_reduce(u)
    load = torch.tensor([sum(stream_costs[i] for i in mine_s)], dtype=torch.float64)
    loads = [torch.zeros(1, dtype=torch.float64) for _ in range(ws)]
    dist.all_gather(loads, load)
    if rank == 0:
        q.put((t.tolist(), u.tolist(), [float(x.item()) for x in loads]))
    dist.destroy_process_group()


def test_two_ranks_gloo_split_the_bench_workloads():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 30500 + os.getpid() % 1000
    procs = [ctx.Process(target=_bench_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    counts, scounts, loads = q.get(timeout=180)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert all(v == 1 for v in counts)   # every batched solve on exactly one rank
    assert all(v == 1 for v in scounts)  # every served request on exactly one rank
    assert max(loads) / (sum(loads) / 2) < 1.05


def test_two_ranks_gloo_take_disjoint_shares():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    counts, loads = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert all(v == 1 for v in counts)
    assert max(loads) / (sum(loads) / 2) < 1.02
