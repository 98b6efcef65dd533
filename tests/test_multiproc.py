"""The N>1 benchmark path is replicas only (batched transforms shard by
sequence with no exchange); its one collective is the max-over-ranks timing
reduction.  This runs it as two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, results):
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms_total = 100.0 + 50.0 * rank  # rank 1 is the slow one
    ms, value = bench.aggregate_over_ranks(ms_total, 1e9, 10, world, dist, "cpu")
    results[rank] = (ms, value)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replica_timing():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    port = _free_port()
    with ctx.Manager() as m:
        results = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, results)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        # every rank sees the slowest rank's time; value counts both replicas
        for r in range(2):
            ms, value = results[r]
            assert ms == pytest.approx(15.0)
            assert value == pytest.approx(2 * 1e9 / 0.015 / 1e9)
