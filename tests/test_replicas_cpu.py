"""Multi-rank host logic on CPU (gloo, world size 2): timeslice partition and
max-over-ranks timing used by bench.py for N > 1 GPUs."""

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist

    from easydistillation_gb300.replicas import max_over_ranks, timeslices_for_rank

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ts = timeslices_for_rank(64, rank, world)
        m = max_over_ranks(10.0 + rank)
        dist.barrier()
        q.put((rank, ts, m))
    finally:
        dist.destroy_process_group()


def test_two_rank_partition_and_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    all_ts = sorted(out[0][1] + out[1][1])
    assert all_ts == list(range(64))
    assert set(out[0][1]).isdisjoint(out[1][1])
    assert out[0][2] == out[1][2] == 11.0


def test_partition_rejects_bad_rank():
    from easydistillation_gb300.replicas import timeslices_for_rank

    with pytest.raises(ValueError):
        timeslices_for_rank(8, 2, 2)
