"""Multi-GPU host logic on the CPU: two gloo ranks (world size 2).

Each rank renders its own sessions (replicas, no data-path collective); the
reported time is the maximum over ranks."""
import os
import socket

import pytest

from meteoros_gb300 import replicas


def test_shard_partitions_sessions():
    for n in (0, 1, 7, 256, 257):
        for world in (1, 2, 3, 8):
            blocks = [replicas.shard(n, r, world) for r in range(world)]
            items = [i for b in blocks for i in b]
            assert items == list(range(n))
            sizes = [len(b) for b in blocks]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        replicas.shard(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 1.5 + rank  # rank 1 is the slow one
        got = replicas.max_over_ranks(ms)
        mine = list(replicas.shard(256, rank, world))
        q.put((rank, got, replicas.rank_seed(2017, rank), mine[0], len(mine)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest_rank():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [r[1] for r in res] == [2.5, 2.5]
    assert res[0][2] != res[1][2]  # each replica renders its own seeded session
    assert (res[0][3], res[0][4], res[1][3], res[1][4]) == (0, 128, 128, 128)


def test_single_process_needs_no_collective():
    assert replicas.max_over_ranks(3.25) == 3.25
