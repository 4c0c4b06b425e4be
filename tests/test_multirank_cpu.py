"""The multi-rank (N > 1) host logic of bench.py on CPU: two gloo ranks, each
timing its own replica; the job's time is the slowest rank's and the value
counts every rank's sites."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, device="cpu")
        q.put((rank, ms, bench.job_value(world, 8_000_000, 2000, ms)))
    finally:
        torch.distributed.destroy_process_group()


def test_replicas_max_over_ranks_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [15.0, 15.0]
    assert got[0][2] == got[1][2] == 2 * 8_000_000 * 2000 / 0.015


def test_single_process_is_identity():
    pytest.importorskip("torch")
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, device="cpu") == 3.5
    assert bench.job_value(1, 100, 10, 1000.0) == 1000.0
