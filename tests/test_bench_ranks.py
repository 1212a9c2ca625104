"""The replicas path of bench.py (--gpus N under torchrun): every rank runs the whole
workload, and the job's time is the slowest rank's (a MAX all-reduce), so the
reported rate is N x the per-rank units over that time.  Two gloo ranks on the CPU
stand in for GPUs (the host logic is the same)."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, REPO)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local = [2.0, 3.5][rank]  # the second rank is slower
        slow = bench.slowest_rank_seconds(local, world)
        out.put((rank, slow, bench.whole_job_rate(7.0e12, world, slow)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest_time():
    torch = pytest.importorskip("torch")
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, slow, rate in got:
        assert slow == 3.5, (rank, slow)
        assert rate == pytest.approx(2 * 7.0e12 / 3.5)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, REPO)
    import bench
    assert bench.slowest_rank_seconds(1.25, 1) == 1.25
    assert bench.whole_job_rate(10.0, 1, 2.0) == 5.0
