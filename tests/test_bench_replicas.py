"""bench.py with N > 1 runs N independent replicas (each GPU solves its own
sweeps; there is no data-path collective): the job time is the slowest
rank's and the throughput counts every replica's systems.  Checked with two
gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    torch.distributed.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}",
                                         rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(100.0 + 50.0 * rank, world, "cpu")
        out.put((rank, ms, bench.replica_throughput(ms, world, 2)))
    finally:
        torch.distributed.destroy_process_group()


def test_two_replicas_report_the_slowest_rank_and_the_job_total():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    import bench
    for rank, ms, value in res:
        assert ms == 150.0                                 # the slower rank's time, on every rank
        assert value == pytest.approx(2 * 2 * bench.NFREQ / 0.150)
