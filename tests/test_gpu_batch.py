"""Batched scans and the block-size search (needs a GPU): concurrent contexts
give the same images as the same scans one after another (up to the order of
the float reductions); the persistent multi-scan DROP (pct_drop_many) gives
every scan the image and residuals of its own pct_drop run, each within the
DROP tolerance of the oracle's binary64 run; packed rows (pct_compact_rows)
are the same rows; and the search returns a block size whose time to the
target residual is the shortest it measured."""
import math

import numpy as np
import pytest

from oracle import oracle
from pct_gb300 import _capi, batch, phantoms, recon

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


def _prepared(scans, sizes):
    rs = []
    for (cfg, data, angles), b in zip(scans, sizes):
        cfg.block_size = b
        r = recon.run_full(cfg, data, angles)
        r.collect_mlp_endpoints()
        r.mlp_rows()
        rs.append(r)
    return rs


def test_compact_rows_keeps_the_rows():
    cfg, data, angles = _scans()[0]
    r = recon.run_full(cfg, data, angles)
    r.collect_mlp_endpoints()
    r.mlp_rows()
    before = (r.array("ROW_OFFSETS"), r.array("ROWS"), r.array("CHORD"))
    r.compact_rows()
    after = (r.array("ROW_OFFSETS"), r.array("ROWS"), r.array("CHORD"))
    for a, b in zip(before, after):
        assert a.tobytes() == b.tobytes()
    r.close()


def test_drop_many_matches_single_scans_and_the_oracle():
    """Three scans with uneven block sizes (one block, several blocks, a ragged
    last block) in one persistent launch per iteration."""
    its = 3
    scans = _scans()
    sizes = (20000, 50000, 130000)
    single = []
    rs = _prepared(scans, sizes)
    for r in rs:
        st = r.drop(its)
        single.append((r.array("X"), [st.residual[k] for k in range(its)]))
        r.reset_iterate()
    rs[1].compact_rows()
    stats = recon.drop_many(rs, its)
    for k, (r, (x1, res1), st) in enumerate(zip(rs, single, stats)):
        x = r.array("X").astype(np.float64)
        assert st.iterations_run == its
        assert np.linalg.norm(x - x1) <= 1e-5 * np.linalg.norm(x1), "scan %d" % k
        for a, b in zip([st.residual[j] for j in range(its)], res1):
            assert abs(a - b) <= 1e-5 * b, "scan %d residuals %s vs %s" % (k, a, b)
        if k in (0, 2):
            cfg = scans[k][0]
            offs, rows, chord = r.array("ROW_OFFSETS"), r.array("ROWS"), r.array("CHORD")
            ref = oracle.drop(cfg, offs, rows, chord.astype(np.float64), r.array("H_WEPL"), r.array("X0"), its,
                              sizes[k], float(np.float32(cfg.lambda_)))
            err = np.linalg.norm(x - ref) / np.linalg.norm(ref)
            assert err <= 1e-4, "scan %d: relative L2 %.3e against the oracle" % (k, err)
    print("drop_many: %.3f ms for %d iterations of 3 scans" % (stats[0].seconds * 1e3, its))
    for r in rs:
        r.close()


def test_drop_many_rejects_other_forms():
    scans = _scans()[:2]
    rs = _prepared(scans, (50000, 50000))
    with pytest.raises(_capi.PctError):
        recon.drop_many([rs[0], rs[0]], 1)
    rs[1].close()
    cfg, data, angles = scans[1]
    cfg.drop_form = 2
    r = recon.run_full(cfg, data, angles)
    r.collect_mlp_endpoints()
    r.mlp_rows()
    with pytest.raises(_capi.PctError):
        recon.drop_many([rs[0], r], 1)
    r.close()
    rs[0].close()
