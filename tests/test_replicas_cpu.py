"""The multi-GPU path is replicas: every rank solves its own queries on its
own GPU and the job time is the max over ranks. The host logic of that path
runs here as two gloo ranks on CPU (bench.py's helpers)."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ids = list(bench.rank_query_ids(rank, 5))
        # rank r "measures" (10 + r) ms of device time and (1 + 2r) s of wall time
        got = bench.max_over_ranks([10.0 + rank, 1.0 + 2 * rank], dist)
        dist.barrier()
        q.put((rank, ids, got))
    finally:
        dist.destroy_process_group()


def test_two_replicas_share_nothing_and_report_the_slowest():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict()
    for _ in procs:
        r, ids, got = q.get(timeout=120)
        out[r] = (ids, got)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert set(out[0][0]).isdisjoint(out[1][0])  # no query solved twice
    assert out[0][1] == out[1][1] == [11.0, 3.0]   # max over ranks, seen by both


def test_single_rank_is_identity():
    import bench

    assert bench.max_over_ranks([1.5, 2.0]) == [1.5, 2.0]
    assert list(bench.rank_query_ids(0, 3)) == [0, 1, 2]
