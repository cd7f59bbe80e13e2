"""Error statement of the tabulated MLP against the analytic MLP at 1M
histories of the cfg2 geometry (needs a GPU): the share of identical rows and
of differing row entries, and the relative L2 distance of the DROP images
reconstructed from the two sets of rows."""
import numpy as np
import pytest

from pct_gb300 import phantoms, recon

pytestmark = pytest.mark.gpu


def _rows_and_image(cfg, data, angles, tabulated, its):
    c = phantoms.make_config({})
    for f, _ in cfg._fields_:
        setattr(c, f, getattr(cfg, f))
    c.mlp_tabulated = tabulated
    r = recon.run_full(c, data, angles)
    r.collect_mlp_endpoints()
    r.mlp_rows()
    offs, rows = r.array("ROW_OFFSETS"), r.array("ROWS")
    r.drop(its)
    x = r.array("X")
    r.close()
    return offs, rows, x


def test_tabulated_mlp_error_statement():
    w = phantoms.cfg2(num_histories=1_000_000, seed=8)
    cfg = phantoms.make_config(w.config)
    data, angles = phantoms.generate(w)
    its = 3
    oa, ra, xa = _rows_and_image(cfg, data, angles, 0, its)
    ot, rt, xt = _rows_and_image(cfg, data, angles, 1, its)
    n = len(oa) - 1
    assert len(ot) == n + 1
    la, lt = np.diff(oa), np.diff(ot)
    same_len = la == lt
    eq = np.zeros(n, bool)
    idx = np.nonzero(same_len)[0]
    # rows of equal length: compare entry by entry in bulk
    starts_a, starts_t = oa[idx], ot[idx]
    pos_a = np.repeat(starts_a, la[idx]) + (np.arange(la[idx].sum()) - np.repeat(np.cumsum(la[idx]) - la[idx], la[idx]))
    pos_t = np.repeat(starts_t, la[idx]) + (np.arange(la[idx].sum()) - np.repeat(np.cumsum(la[idx]) - la[idx], la[idx]))
    diff = ra[pos_a] != rt[pos_t]
    bad_rows = np.zeros(len(idx), bool)
    np.logical_or.at(bad_rows, np.repeat(np.arange(len(idx)), la[idx]), diff)
    eq[idx] = ~bad_rows
    frac_rows = eq.mean()
    frac_entries = 1.0 - (diff.sum() + np.abs(la - lt)[~same_len].sum()) / la.sum()
    rel = float(np.linalg.norm(xt.astype(np.float64) - xa) / np.linalg.norm(xa.astype(np.float64)))
    print("tabulated vs analytic MLP, %d rows: identical rows %.4f, matching entries %.5f, "
          "DROP image after %d iterations: relative L2 %.2e" % (n, frac_rows, frac_entries, its, rel))
    assert frac_rows > 0.95
    assert rel < 1e-2
