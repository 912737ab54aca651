"""The multi-process (replica) path of bench.py on CPU: two gloo ranks, each with
its own step time; the reported time is the slowest rank's and the whole-job
throughput counts both ranks' bytes."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = [3.0, 5.0][rank]
    t = bench.max_over_ranks(ms, dist)
    gbps = bench.whole_job_gbps(1 << 30, world, t)
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, t, gbps))


def test_two_gloo_ranks_report_slowest_time_and_whole_job_bytes():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, gbps in got:
        assert t == 5.0
        assert abs(gbps - 2 * (1 << 30) / 5e-3 / 1e9) < 1e-9


def test_single_process_is_its_own_maximum():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(4.5, None) == 4.5
    assert abs(bench.whole_job_gbps(10**9, 1, 1000.0) - 1.0) < 1e-12
