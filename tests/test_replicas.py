"""Replica partitioning across ranks, run as two gloo processes on CPU.

Each rank takes its own share of the requests (no data-path collective);
the shares cover the set exactly once, and the timing reduction returns the
slowest rank's time on every rank."""

import os
import socket

import pytest
import torch.multiprocessing as mp

from ionization_gb300 import replicas, workloads


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = replicas.rank_world()
        reqs = workloads.poisson_scan_parameters(37, seed=11)
        mine = replicas.shard([p["id"] for p in reqs], r, w)
        replicas.barrier()
        slowest = replicas.max_over_ranks(1.5 + r)
        out.put((r, local, mine, slowest, replicas.sweep_seed(20261203, r)))
    finally:
        dist.destroy_process_group()


def test_two_rank_shards_cover_requests_once_and_time_is_max():
    world = 2
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    got = [out.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    got.sort()
    ids = [i for g in got for i in g[2]]
    assert sorted(ids) == list(range(37))
    assert len(set(got[0][2]) & set(got[1][2])) == 0
    assert [g[3] for g in got] == [2.5, 2.5]
    assert [g[1] for g in got] == [0, 1]
    assert [g[4] for g in got] == [20261203, 20261204]


def test_shard_rejects_bad_rank():
    with pytest.raises(ValueError):
        replicas.shard([1, 2, 3], 2, 2)
