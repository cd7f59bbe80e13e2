"""Batched scans and the block-size search (needs a GPU): concurrent contexts
give the same images as the same scans one after another (up to the order of
the float reductions), and the search returns a block size whose time to the
target residual is the shortest it measured."""
import math

import numpy as np
import pytest

from pct_gb300 import batch, phantoms, recon

pytestmark = pytest.mark.gpu


def _scans():
    out = []
    for seed, cols, sl, n in ((41, 128, 8, 300_000), (42, 160, 16, 400_000), (43, 128, 24, 300_000)):
        w = phantoms.ellipsoids(seed, num_histories=n, cols=cols, slices=sl)
        c = dict(w.config)
        c.update(iterations=3, block_size=50000)
        data, angles = phantoms.generate(w)
        out.append((phantoms.make_config(c), data, angles))
    return out


def test_concurrent_scans_match_sequential():
    scans = _scans()
    seq, t_seq = batch.reconstruct_many(scans, concurrent=False)
    con, t_con = batch.reconstruct_many(scans, concurrent=True)
    print("3 scans: sequential %.3f s, concurrent %.3f s" % (t_seq, t_con))
    for a, b in zip(seq, con):
        assert a.shape == b.shape
        assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(a)


def test_block_size_search():
    cfg, data, angles = _scans()[1]
    r = recon.run_full(cfg, data, angles)
    r.collect_mlp_endpoints()
    r.mlp_rows()
    best, table = batch.autotune_block_size(r, candidates=(10000, 25000, 100000), iterations=3)
    sizes = [t[0] for t in table]
    assert best in sizes and sorted(sizes) == sorted({50000, 10000, 25000, 100000})
    times = {t[0]: t[3] for t in table}
    assert math.isfinite(times[50000])  # the current size reaches its own residual
    assert times[best] == min(times.values())
    assert r.cfg.block_size == best
    st = r.drop(1)  # the context runs with the chosen size
    assert st.iterations_run == 1
    r.close()
    for t in table:
        print("block %6d: %.3f ms/iteration, residuals %s, to target %.3f ms"
              % (t[0], t[1] * 1e3, ["%.4f" % v for v in t[2]], t[3] * 1e3))
