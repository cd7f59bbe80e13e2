"""Sharded DROP on one GPU (needs a GPU): two contexts, each with its share of
every block (pct_select_shard), run pct_drop in two host threads; their
all-reduce callback meets on the host (a barrier, then the sum of both
buffers), so no kernel waits on another context.  The image must match the
single-context DROP up to the order of the float sums, and both ranks must
hold the same image."""
import threading

import numpy as np
import pytest

from pct_gb300 import _capi, phantoms, recon
from pct_gb300.shard import numpy_dtype

pytestmark = pytest.mark.gpu

ITERS = 3


class ThreadAllReduce:
    """pct_allreduce_fn for ranks that are threads of this process."""

    def __init__(self, world):
        self.world = world
        self.barrier = threading.Barrier(world, timeout=120)
        self.slots = [None] * world
        self.calls = [0] * world

    def fn(self, rank):
        lib = _capi.load()

        def call(user, data, count, dtype, on_device):
            try:
                assert on_device == 1
                tmp = np.empty(int(count), dtype=numpy_dtype(dtype))
                nbytes = tmp.nbytes
                _capi.check(lib.pct_memcpy(tmp.ctypes.data, data, nbytes))
                self.slots[rank] = tmp
                self.barrier.wait()
                total = self.slots[0].copy()
                for s in self.slots[1:]:
                    total += s
                self.barrier.wait()
                _capi.check(lib.pct_memcpy(data, total.ctypes.data, nbytes))
                self.calls[rank] += 1
                return 0
            except Exception:
                self.barrier.abort()
                return 1

        return call


def _workload(**over):
    w = phantoms.cfg2(num_histories=300_000, seed=21)
    c = dict(w.config)
    c.update(block_size=20_000, **over)
    return phantoms.make_config(c), phantoms.generate(w)


def _prepared(cfg, data, angles):
    r = recon.run_full(cfg, data, angles)
    r.collect_mlp_endpoints()
    return r


@pytest.mark.parametrize("form", [0, 1, 2])
def test_two_shards_match_one_context(form):
    cfg, (data, angles) = _workload(drop_form=form)
    ref = _prepared(cfg, data, angles)
    n = ref.counts()["reconstruction_histories"]
    ref.mlp_rows()
    ref.drop(ITERS)
    x_ref = ref.array("X")
    ref.close()

    world = 2
    ar = ThreadAllReduce(world)
    ranks = []
    for k in range(world):
        r = _prepared(cfg, data, angles)
        r.select_shard(k, world)
        r.set_allreduce(ar.fn(k))
        r.mlp_rows()
        ranks.append(r)
    assert sum(r.counts()["reconstruction_histories"] for r in ranks) == n
    out, errs = [None] * world, [None] * world

    def run(k):
        try:
            ranks[k].drop(ITERS)
            out[k] = ranks[k].array("X")
        except Exception as e:
            errs[k] = e

    threads = [threading.Thread(target=run, args=(k,)) for k in range(world)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=600)
    for r in ranks:
        r.close()
    assert errs == [None] * world, errs
    nblocks = (n + 20_000 - 1) // 20_000
    # counts once, ||b||^2 once, then per iteration every block's update and the residual
    assert ar.calls[0] == ar.calls[1] == 2 + ITERS * (nblocks + 1)
    assert np.array_equal(out[0], out[1])
    rel = np.linalg.norm(out[0] - x_ref) / np.linalg.norm(x_ref)
    assert rel < 1e-5, rel


def test_one_shard_with_identity_callback():
    cfg, (data, angles) = _workload()
    ref = _prepared(cfg, data, angles)
    ref.mlp_rows()
    st_ref = ref.drop(ITERS)
    x_ref = ref.array("X")
    ref.close()
    r = _prepared(cfg, data, angles)
    r.select_shard(0, 1)
    calls = []
    r.set_allreduce(lambda user, data, count, dtype, on_device: calls.append(dtype) or 0)
    r.mlp_rows()
    st = r.drop(ITERS)
    x = r.array("X")
    r.set_allreduce(None)
    r.close()
    assert calls and calls.count(_capi.PCT_DT_F32) > 0
    rel = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
    assert rel < 1e-5, rel
    assert abs(st.residual[ITERS - 1] - st_ref.residual[ITERS - 1]) < 1e-5 * st_ref.residual[ITERS - 1]


def test_select_shard_checks():
    cfg, (data, angles) = _workload()
    r = _prepared(cfg, data, angles)
    with pytest.raises(_capi.PctError):
        r.select_shard(2, 2)
    with pytest.raises(_capi.PctError):
        r.select_shard(0, 3)  # 20000 is not a multiple of 3
    r.close()
