"""Sharded DROP protocol on CPU: two gloo ranks, each with its interleaved share
of the rows (i % 2 == rank, local block size B / 2, the global block count),
summing every block's update and counts through pct_gb300.shard.TorchAllReduce
on host buffers.  The oracle does each rank's block updates; the result must
equal the unsharded oracle DROP."""
import os
import socket
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
N, B, ITERS, LAM = 301, 100, 3, 0.1  # 4 global blocks; the last holds one row (rank 1 has none)


def _problem():
    from pct_gb300 import phantoms
    cfg = phantoms.make_config(dict(recon_cyl_radius=3.2, columns=64, rows=64, ssd_v_size=2.0))
    g = phantoms.geometry(cfg)
    rng = np.random.default_rng(11)
    lens = rng.integers(5, 40, size=N)
    offs = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    rows = rng.integers(0, g.num_voxels, size=offs[-1]).astype(np.uint32)
    chord = rng.uniform(0.08, 0.12, size=N)
    wepl = rng.uniform(0.5, 5.0, size=N).astype(np.float32)
    x0 = rng.uniform(0.5, 1.5, size=g.num_voxels)
    return cfg, offs, rows, chord, wepl, x0


def _local(offs, rows, chord, wepl, rank, world):
    keep = np.arange(N) % world == rank
    lens = np.diff(offs)[keep]
    lo = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    lr = np.concatenate([rows[offs[i]:offs[i + 1]] for i in np.nonzero(keep)[0]]).astype(np.uint32)
    return lo, lr, chord[keep], wepl[keep]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import oracle
        from pct_gb300.shard import TorchAllReduce
        cfg, offs, rows, chord, wepl, x0 = _problem()
        lo, lr, lc, lw = _local(offs, rows, chord, wepl, rank, world)
        ar = TorchAllReduce()
        nblocks = (N + B - 1) // B
        x = oracle.drop_shard(cfg, lo, lr, lc, lw, x0, ITERS, B // world, nblocks, LAM, ar)
        out.put((rank, x, repr(ar.error)))
    except Exception as e:
        out.put((rank, None, repr(e)))
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sharded_drop_equals_unsharded_on_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=180) for _ in procs), key=lambda t: t[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    sys.path.insert(0, ROOT)
    from oracle import oracle
    cfg, offs, rows, chord, wepl, x0 = _problem()
    ref = oracle.drop(cfg, offs, rows, chord, wepl, x0, ITERS, B, LAM)
    (_, x0r, e0), (_, x1r, e1) = res
    assert e0 == "None" and e1 == "None", (e0, e1)
    assert np.array_equal(x0r, x1r)  # every rank applies the same summed update
    assert np.allclose(x0r, ref, rtol=1e-12, atol=1e-12)
    assert np.abs(x0r - x0).max() > 1e-3  # the iterations did move the image


def test_host_view_round_trip():
    from pct_gb300 import _capi
    from pct_gb300.shard import host_view
    a = np.arange(7, dtype=np.float64)
    v = host_view(a.ctypes.data, 7, _capi.PCT_DT_F64)
    v += 1.0
    assert np.array_equal(a, np.arange(7) + 1.0)
    u = np.array([1, 2, 3], dtype=np.uint32)
    assert host_view(u.ctypes.data, 3, _capi.PCT_DT_U32).tolist() == [1, 2, 3]
