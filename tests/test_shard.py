"""Bunch sharding host logic: cost-balanced contiguous ranges, and the
gather of per-rank results to rank 0 with two gloo ranks on the CPU (a
stand-in batch fills each bunch's profile with its own index, so the
gathered order and completeness are checked exactly)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from inovesa_gb300 import shard


class Desc:
    def __init__(self, n, it=4, chain=0):
        self.n, self.it, self.chain = n, it, chain


def test_partition_covers_and_balances():
    rng = np.random.default_rng(3)
    for world in (1, 2, 3, 4, 8):
        for nb in (1, 5, 96, 256):
            costs = rng.choice([128, 256, 512, 1024], size=nb) ** 2.0
            r = shard.partition(costs, world)
            assert len(r) == world
            assert r[0][0] == 0 and r[-1][1] == nb
            for (a, b), (c, d) in zip(r, r[1:]):
                assert b == c and a <= b
            if nb >= 4 * world:
                loads = [costs[a:b].sum() for a, b in r]
                # no rank gets more than its share plus one largest bunch
                assert max(loads) <= costs.sum() / world + costs.max() + 1e-9


def test_partition_uniform_scan():
    r = shard.partition(np.ones(256), 4)
    assert r == [(0, 64), (64, 128), (128, 192), (192, 256)]


class FakeBatch:
    def __init__(self, descs, offset):
        self.descs, self.offset = descs, offset

    def step(self, n):
        pass

    def profile(self, i):
        return np.full(self.descs[i].n, self.offset + i, np.float32)

    def filling(self):
        return [float(self.offset + i) for i in range(len(self.descs))]


def _rank(rank, world, port, descs, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ranges = shard.partition([shard.bunch_cost(d) for d in descs], world)
        lo = ranges[rank][0]
        s = shard.ShardedScan(descs, [], rank, world,
                              lambda local, imps: FakeBatch(local, lo),
                              dist=dist)
        s.step(5)
        prof = s.profiles()
        fill = s.fillings()
        if rank == 0:
            q.put((ranges, prof.tolist(), fill.tolist()))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("sizes", [[128, 256, 512, 64, 1024, 128, 256],
                                   [256] * 3])
def test_sharded_gather_two_ranks(sizes):
    descs = [Desc(n) for n in sizes]
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, descs, q))
             for r in range(world)]
    for p in procs:
        p.start()
    ranges, prof, fill = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    want = np.concatenate([np.full(n, i, np.float32)
                           for i, n in enumerate(sizes)])
    assert np.array_equal(np.asarray(prof, np.float32), want)
    assert fill == [float(i) for i in range(len(sizes))]
    assert ranges[0][0] == 0 and ranges[-1][1] == len(sizes)
