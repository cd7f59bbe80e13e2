"""The oracle's DROP variants on small synthetic rows (CPU): with eta = 0 both
reduce to the standard DROP update; with eta > 0 they differ from it."""
import numpy as np

from oracle import oracle
from pct_gb300 import phantoms


def _rows(seed=3, n=300, nv_cfg=None):
    cfg = phantoms.make_config(dict(recon_cyl_radius=3.2, columns=64, rows=64, ssd_v_size=2.0))
    g = phantoms.geometry(cfg)
    rng = np.random.default_rng(seed)
    lens = rng.integers(5, 40, size=n)
    offs = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    rows = rng.integers(0, g.num_voxels, size=offs[-1]).astype(np.uint32)
    chord = rng.uniform(0.08, 0.12, size=n)
    wepl = rng.uniform(0.5, 5.0, size=n).astype(np.float32)
    x0 = rng.uniform(0.5, 1.5, size=g.num_voxels)
    return cfg, offs, rows, chord, wepl, x0


def test_variants_reduce_to_drop_without_eta():
    cfg, offs, rows, chord, wepl, x0 = _rows()
    std = oracle.drop(cfg, offs, rows, chord, wepl, x0, 3, 100, 0.1)
    for v in (1, 2):
        x = oracle.drop_variant(cfg, offs, rows, chord, wepl, x0, 3, 100, 0.1, v, 0.0, 1)
        assert np.allclose(x, std, rtol=1e-12, atol=1e-12)


def test_variants_change_the_update_with_eta():
    cfg, offs, rows, chord, wepl, x0 = _rows()
    std = oracle.drop(cfg, offs, rows, chord, wepl, x0, 3, 100, 0.1)
    for v in (1, 2):
        x = oracle.drop_variant(cfg, offs, rows, chord, wepl, x0, 3, 100, 0.1, v, 2.5, 1)
        assert np.abs(x - std).max() > 1e-6
