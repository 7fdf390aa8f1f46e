"""The N>1 path on the CPU with gloo (world_size 2): instance sharding covers
every instance once, and the throughput reduction uses the slowest rank."""
import os
import socket

import numpy as np
import pytest

from swe import parallel as P


def test_shard_instances_partition():
    rng = np.random.default_rng(0)
    sizes = np.exp(rng.uniform(np.log(2e3), np.log(2e5), 512)).astype(int)
    for world in (1, 2, 3, 8):
        shards = [P.shard_instances(sizes, world, r) for r in range(world)]
        allidx = sorted(i for s in shards for i in s)
        assert allidx == list(range(len(sizes)))
        loads = [sizes[s].sum() for s in shards]
        assert max(loads) - min(loads) <= sizes.max()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sizes = [5000, 3000, 7000, 1000, 2000]
        mine = P.shard_instances(sizes, world, rank)
        units = sum(sizes[i] for i in mine) * 3.0
        seconds = 1.0 + rank                       # rank 1 is the slowest
        thr = P.aggregate_throughput(units, seconds, dist)
        mx = P.allreduce_max(float(rank), dist)
        q.put((rank, mine, thr, mx))
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    assert sorted(res[0][1] + res[1][1]) == list(range(5))
    total_units = 3.0 * sum([5000, 3000, 7000, 1000, 2000])
    for _, _, thr, mx in res:
        assert thr == pytest.approx(total_units / 2.0)
        assert mx == 1.0
