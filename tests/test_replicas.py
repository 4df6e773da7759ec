"""Replica-parallel rank logic as two gloo ranks on CPU (the bench's N > 1 path without GPUs)."""
import os
import socket

import pytest
import torch
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    from quantax_gb300 import replicas
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert replicas.world() == world and replicas.rank() == rank
        replicas.barrier()
        elapsed = 1.5 + rank  # the slower rank sets the reported time
        m = replicas.max_over_ranks(elapsed)
        rate = replicas.aggregate_rate(10, m)
        seeds = [None] * world
        dist.all_gather_object(seeds, replicas.replica_seed(1234, rank))
        out.put((rank, m, rate, seeds))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_time_and_seed():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, m, rate, seeds in res:
        assert m == pytest.approx(2.5)            # max over ranks
        assert rate == pytest.approx(2 * 10 / 2.5)  # world * units / slowest time
        assert seeds == [1234, 1235]              # every replica samples its own chains


def test_single_process_defaults():
    from quantax_gb300 import replicas
    assert replicas.world() == 1 and replicas.rank() == 0
    assert replicas.max_over_ranks(3.0) == 3.0
    assert replicas.aggregate_rate(8, 2.0) == 4.0
