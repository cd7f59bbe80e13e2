"""Replica aggregation of bench.py over world-size-2 gloo ranks on CPU: the
job's time is the slowest rank's, its work the sum over ranks."""
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
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t, u = bench.reduce_across_ranks(1.0 + rank, 10.0 * (rank + 1), dist, "cpu")
    out.put((rank, t, u))
    dist.destroy_process_group()


def test_reduce_across_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, u in res:
        assert t == 2.0 and u == 30.0


def test_single_rank_is_identity():
    import importlib
    sys.path.insert(0, ROOT)
    bench = importlib.import_module("bench")
    assert bench.reduce_across_ranks(3.5, 7.0) == (3.5, 7.0)
