"""Replica logic of bench.py under torch.distributed, on CPU with the gloo backend
and two ranks: the job time is the slowest rank's, and the replicas' trial
ranges (hence their noise streams) are disjoint."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")
        first = bench.replica_first_trial(rank)
        firsts = [None] * world
        dist.all_gather_object(firsts, first)
        out.put((rank, t, firsts))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, firsts in res:
        assert t == 15.0   # every rank reports the slowest rank's time
        assert firsts == [0, 1_000_000]
