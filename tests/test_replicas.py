"""The multi-GPU form of the benchmark is replicas: one process per GPU, each
multiplying its own matrices, with no collective on the data path.  The whole
job's time is the slowest rank's (a max all-reduce every rank agrees on) and
its rate counts every rank's work.  Here two ranks run that host-side logic on
the CPU over gloo (no GPU)."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = 10.0 + 5.0 * rank                # rank 1 is the slower replica
        ms = bench.job_time_ms(local_ms, dist, "cpu")
        rate = bench.job_rate_gops(2.0 * 8192 ** 3, 4, world, ms)
        out.put((rank, ms, rate))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replica_job_time_is_the_slowest_rank():
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(r for r, _, _ in got) == [0, 1]
    for _, ms, rate in got:
        assert ms == 15.0                                    # both ranks agree on the max
        assert rate == pytest.approx(2.0 * 8192 ** 3 * 4 * 2 / 15e-3 / 1e9)


def test_single_process_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_time_ms(12.5) == 12.5
    assert bench.job_rate_gops(100.0, 10, 1, 1000.0) == pytest.approx(1e-6)
