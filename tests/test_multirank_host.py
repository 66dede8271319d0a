"""The multi-process parts of bench.py on CPU with the gloo backend (world size 2): the slowest
rank's time is what every rank reports, the aggregate counts every replica's work, and the
reference arm prints only on rank 0."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, times, out):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_time_over_ranks(torch, dist, times[rank], torch.device("cpu"))
    out.put((rank, ms, bench.aggregate_tflops(world, 2e12, ms)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    times = [3.0, 5.0]
    procs = [ctx.Process(target=_worker, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [5.0, 5.0]
    assert all(abs(r[2] - 2 * 2e12 / 5e-3 / 1e12) < 1e-9 for r in res)


def test_reference_arm_silent_off_rank_zero(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        steps, warmup, cpu_rows = 1, 0, 1
    assert bench.run_reference(Args(), rank=1, world=2) is None
    assert capsys.readouterr().out == ""
