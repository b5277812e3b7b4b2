"""Multi-GPU form of the benchmark: independent replicas (the pass has no
exchange step at one mesh per GPU).  The job-level aggregation -- the
slowest rank's time over world x units -- is checked with two gloo ranks on
CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, ms, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms_max, value = bench.job_throughput(ms[rank], 1000, 4, world)
    out[rank] = (ms_max, value)
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        ms = [40.0, 50.0]
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, ms, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
            assert p.exitcode == 0
        for r in range(2):
            ms_max, value = out[r]
            assert ms_max == 50.0
            assert abs(value - 2 * 1000 * 4 / 0.050) < 1e-6


def test_single_replica_is_local_time():
    pytest.importorskip("torch")
    import bench
    ms_max, value = bench.job_throughput(20.0, 500, 2, 1)
    assert ms_max == 20.0 and abs(value - 500 * 2 / 0.020) < 1e-9
