"""The oracle's tabulated MLP (find_MLP_path_GPU_tabulated restated) against its
analytic MLP on the rows of a small scan (CPU): the tables quantise the entry
angle and the depths, so the rows agree except at a small fraction of samples
near voxel faces, and every row starts at the same first voxel."""
import numpy as np

from oracle import oracle
from pct_gb300 import phantoms


def test_tabulated_rows_close_to_analytic():
    w = phantoms.tiny(num_histories=40000, seed=7, v_extent=0.3)
    cfg = phantoms.make_config(w.config)
    data, angles = phantoms.generate(w)
    out = oracle.run_pipeline(cfg, data, angles, iterations=0, keep_history=True)
    hr = out["_hr"]
    n = len(hr["WEPL"])
    assert n > 1000
    o_a, r_a, c_a = oracle.mlp_rows(cfg, hr)
    o_t, r_t, c_t = oracle.mlp_rows(cfg, hr, tabulated=True)
    assert np.array_equal(c_a, c_t)  # the chord is the analytic EffectiveChordLength in both
    same = 0
    for i in range(n):
        a, t = r_a[o_a[i]:o_a[i + 1]], r_t[o_t[i]:o_t[i + 1]]
        assert a[0] == t[0]
        same += int(np.array_equal(a, t))
    frac = same / n
    print("tabulated rows equal to analytic: %.4f of %d" % (frac, n))
    assert frac > 0.9
    la, lt = np.diff(o_a), np.diff(o_t)
    assert np.abs(la - lt).max() <= 3
