"""Replica helpers across two gloo processes on the CPU."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from ustb_gb300 import replicas


def test_shard_and_frame_range_cover_disjointly():
    for n, world in ((10, 3), (7, 2), (3, 4)):
        got = sorted(i for r in range(world) for i in replicas.shard(n, r, world))
        assert got == list(range(n))
        spans = [replicas.frame_range(n, r, world) for r in range(world)]
        assert spans[0][0] == 0 and spans[-1][1] == n
        assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
    with pytest.raises(ValueError):
        replicas.shard(5, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = replicas.shard(9, rank, world)
        t = replicas.max_over_ranks(1.0 + rank)  # each rank's "step time"
        total = torch.tensor([len(mine)], dtype=torch.int64)
        dist.all_reduce(total)
        out[rank] = (t, int(total.item()), mine)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_disjoint_requests_and_the_slowest_time():
    world, port = 2, _free_port()
    with mp.get_context("spawn").Manager() as m:  # no fork of this multi-threaded process
        out = m.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 2.0          # max over ranks
    assert res[0][1] == res[1][1] == 9            # every request counted once
    assert set(res[0][2]).isdisjoint(res[1][2])
