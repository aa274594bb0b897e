"""The N > 1 form of the benchmark runs independent replicas (the fit is not
sharded across GPUs): the job time is the slowest rank's and the job
rate counts every rank's SNPs.  Checked with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = [37.5, 41.25][rank]                 # per-rank step times
    dist.barrier()
    m = bench.max_over_ranks(ms, dist, "cpu")
    q.put((rank, m, bench.job_rate(1000, world, m)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    import torch.multiprocessing as mp
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
    for rank, m, rate in out:
        assert m == 41.25
        assert rate == pytest.approx(2 * 1000 / 0.04125)


def test_single_process_passthrough():
    import bench
    assert bench.max_over_ranks(3.0) == 3.0
    assert bench.job_rate(2_000_000, 1, 100.0) == pytest.approx(2e7)
