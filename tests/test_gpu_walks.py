"""Certified binary32 paths against their binary64 modes at sizes the CPU oracle
cannot reach in seconds (needs a GPU).

The hull walks (k_hull_walk_fast vs k_hull_walk) and the MLP rows (binary32
samples with binary64 recomputation vs every sample in binary64) must give
the same integers bit for bit; the binary32 paths must do almost all the work.
"""
import numpy as np
import pytest

from pct_gb300 import phantoms, recon

pytestmark = pytest.mark.gpu


def copy_config(cfg, **over):
    c = phantoms.make_config({})
    for f, _ in cfg._fields_:
        setattr(c, f, getattr(cfg, f))
    for k, v in over.items():
        setattr(c, k, v)
    return c


@pytest.mark.parametrize("case", ["cfg1_600k", "cfg2_1m"])
def test_hull_walks_match_binary64(case):
    w = phantoms.cfg1(num_histories=600_000, seed=3) if case == "cfg1_600k" else phantoms.cfg2(num_histories=1_000_000,
                                                                                               seed=4)
    over = dict(w.config)
    over.update(msc_on=1, sm_on=1, sc_on=1)
    cfg = phantoms.make_config(over)
    data, angles = phantoms.generate(w)
    out = {}
    for exact in (0, 1):
        r = recon.Reconstruction(copy_config(cfg, walk_exact=exact))
        r.reserve(data.shape[1])
        r.process_chunk(data, angles)
        out[exact] = {k: r.array(k) for k in ("SC_HULL", "MSC_COUNTS", "SM_COUNTS")}
        out[exact]["counts"] = r.counts()
        r.close()
    for k in ("SC_HULL", "MSC_COUNTS", "SM_COUNTS"):
        a, b = out[0][k], out[1][k]
        assert a.shape == b.shape and np.array_equal(a, b), "%s: %d voxels differ" % (k, int(np.sum(a != b)))
    c = out[0]["counts"]
    steps = int(out[1]["SM_COUNTS"].sum() + out[1]["MSC_COUNTS"].sum())
    assert c["walk_fp64_steps"] < 0.05 * max(steps, 1), c


def test_mlp_rows_match_binary64_at_scale():
    w = phantoms.cfg2(num_histories=1_000_000, seed=5)
    cfg = phantoms.make_config(w.config)
    data, angles = phantoms.generate(w)
    rows = {}
    for exact in (0, 1):
        r = recon.run_full(copy_config(cfg, mlp_exact=exact), data, angles)
        r.collect_mlp_endpoints()
        r.mlp_rows()
        rows[exact] = (r.array("ROW_OFFSETS"), r.array("ROWS"))
        c = r.counts()
        r.close()
        if exact == 0:
            assert c["mlp_fp64_samples"] < 0.01 * int(rows[0][0][-1]), c
    assert np.array_equal(rows[0][0], rows[1][0])
    assert np.array_equal(rows[0][1], rows[1][1])


def test_endpoint_walks_match_binary64():
    w = phantoms.cfg2(num_histories=1_000_000, seed=6)
    cfg = phantoms.make_config(w.config)
    data, angles = phantoms.generate(w)
    keys = ("H_X_ENTRY", "H_Y_ENTRY", "H_Z_ENTRY", "H_X_EXIT", "H_Y_EXIT", "H_Z_EXIT", "H_FIRST_VOXEL")
    out = {}
    for exact in (0, 1):
        r = recon.run_full(copy_config(cfg, walk_exact=exact), data, angles)
        c0 = r.counts()["walk_fp64_steps"]
        r.collect_mlp_endpoints()
        out[exact] = {k: r.array(k) for k in keys}
        out[exact]["n"] = r.counts()["reconstruction_histories"]
        out[exact]["fp64_steps"] = r.counts()["walk_fp64_steps"] - c0
        r.close()
    assert out[0]["n"] == out[1]["n"]
    for k in keys:
        assert out[0][k].tobytes() == out[1][k].tobytes(), k
    assert out[0]["fp64_steps"] < 0.1 * out[0]["n"], out[0]["fp64_steps"]
