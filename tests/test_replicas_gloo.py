"""The N > 1 path of bench.py (independent replicas, one per GPU: no data
exchange, a barrier and a max over ranks of the timed region) on CPU with two
gloo ranks: the aggregation every rank sees, the whole-job throughput and the
disjoint per-rank session streams."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, queue):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank 0 has the longer device time, rank 1 the longer wall time
        local = [10.0, 20.0] if rank == 0 else [30.0, 5.0]
        dist.barrier()
        got = bench.max_over_ranks(local, world)
        queue.put((rank, got, [bench.rank_session(rank, k) for k in range(3)]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, queue)) for r in range(world)]
    for p in procs:
        p.start()
    results = [queue.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    by_rank = {r: (got, sessions) for r, got, sessions in results}
    assert by_rank[0][0] == by_rank[1][0] == [30.0, 20.0]   # every rank reports the job's max
    assert not set(by_rank[0][1]) & set(by_rank[1][1])        # replicas never share a session
    # 32 stages x 100 steps on each of 2 ranks in 0.5 s (the slowest rank)
    assert bench.replica_throughput(3200, 2, 0.5) == pytest.approx(12800.0)


def test_single_rank_is_unchanged():
    assert bench.max_over_ranks([1.5, 2.5], 1) == [1.5, 2.5]
    assert bench.replica_throughput(3200, 1, 0.5) == pytest.approx(6400.0)
    assert bench.rank_session(0, 7) == 7 and bench.rank_session(1, 0) == 1 << 32
