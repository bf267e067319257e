"""Partition of a batch of scenes over ranks and the host gather of their
results, with two gloo ranks on the CPU (no GPU)."""
import os
import socket

import pytest

import shard

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def test_partition_covers_and_balances():
    loads = [64 * 64, 512 * 512, 100 * 100, 300 * 300, 80 * 80, 512 * 512, 200 * 200]
    for world in (1, 2, 3, 8):
        parts = shard.partition(loads, world)
        flat = sorted(k for p in parts for k in p)
        assert flat == list(range(len(loads)))
        tot = [sum(loads[k] for k in p) for p in parts]
        assert max(tot) - min(tot) <= max(loads)   # LPT bound
    assert shard.partition(loads, 2) == shard.partition(list(loads), 2)   # deterministic
    with pytest.raises(ValueError):
        shard.partition(loads, 0)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, loads, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    parts = shard.partition(loads, world)
    # each rank "computes" its scenes' results: here a loss derived from the index
    mine = {k: (k, float(k) * 0.5, rank) for k in parts[rank]}
    allv = shard.gather(mine, parts, rank, world)
    q.put((rank, allv, parts))
    dist.destroy_process_group()


def test_gather_two_gloo_ranks():
    loads = [4096, 262144, 10000, 90000, 6400, 250000, 40000, 1]
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, loads, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    parts = res[0][2]
    for rank, allv, _ in res:
        assert [v[0] for v in allv] == list(range(len(loads)))
        assert [v[1] for v in allv] == [0.5 * k for k in range(len(loads))]
        owner = {k: r for r, p in enumerate(parts) for k in p}
        assert [v[2] for v in allv] == [owner[k] for k in range(len(loads))]
