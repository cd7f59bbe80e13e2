"""Edge cases of the reconstruction path (needs a GPU): empty and one-history
scans, scans that miss the volume, zero-size and ragged chunks, a block size of
one row and one larger than the scan, the gather form on one block with
hundreds of rows per voxel, grids whose size is not a multiple of
the brick (no bricks; NUM_VOXELS not a multiple of 4), the linear voxel order,
early stopping on the residual, and the status codes of out-of-order stages
and invalid settings."""
import numpy as np
import pytest

from oracle import oracle
from pct_gb300 import _capi, phantoms, recon

pytestmark = pytest.mark.gpu
DROP_TOL = 1e-4


def _cfg(w, **over):
    c = dict(w.config)
    c.update(over)
    return phantoms.make_config(c)


def _through_rows(cfg, data, angles, chunks=None):
    r = recon.Reconstruction(cfg)
    n = data.shape[1]
    r.reserve(max(n, 1))
    for a, b in (chunks or [(0, n)]):
        r.process_chunk(data[:, a:b], angles[a:b])
    r.hull_detection_finish()
    r.statistical_cuts()
    r.FBP()
    r.hull_selection()
    r.define_initial_iterate()
    r.collect_mlp_endpoints()
    r.mlp_rows()
    return r


def test_empty_scan_runs_through():
    w = phantoms.tiny(num_histories=1000, seed=3)
    cfg = _cfg(w, iterations=2)
    data = np.zeros((13, 0), np.float32)
    angles = np.zeros(0, np.float32)
    r = _through_rows(cfg, data, angles)
    c = r.counts()
    assert c["total_histories"] == 0 and c["reconstruction_histories"] == 0
    x0 = r.array("X").copy()
    st = r.drop(2)
    assert st.iterations_run == 2
    assert np.array_equal(r.array("X"), x0)  # no rows: the image stays the initial iterate
    assert r.array("ROW_OFFSETS").tolist() == [0]
    r.close()


def test_one_history_and_missing_histories():
    w = phantoms.tiny(num_histories=2000, seed=4)
    cfg = _cfg(w, iterations=1)
    data, angles = phantoms.generate(w)
    # one history, and a scan whose histories all miss the reconstruction cylinder
    for d, a in ((data[:, :1], angles[:1]), (np.full((13, 50), 1e4, np.float32), angles[:50])):
        r = _through_rows(cfg, d, a)
        c = r.counts()
        assert c["total_histories"] == d.shape[1]
        assert c["reconstruction_histories"] <= d.shape[1]
        r.drop(1)
        assert np.all(np.isfinite(r.array("X")))
        r.close()


def test_zero_size_and_ragged_chunks_equal_one_batch():
    w = phantoms.tiny(num_histories=30000, seed=5, v_extent=0.3)
    cfg = _cfg(w)
    data, angles = phantoms.generate(w)
    n = data.shape[1]
    one = _through_rows(cfg, data, angles)
    rows1, offs1 = one.array("ROWS"), one.array("ROW_OFFSETS")
    one.close()
    cuts = [0, 0, 1, 1, 8, n // 2, n // 2, n]
    rag = _through_rows(cfg, data, angles, chunks=list(zip(cuts[:-1], cuts[1:])))
    assert np.array_equal(rag.array("ROWS"), rows1)
    assert np.array_equal(rag.array("ROW_OFFSETS"), offs1)
    rag.close()


@pytest.mark.parametrize("block", [1, 10_000_000])
def test_block_size_extremes_against_oracle(block):
    w = phantoms.tiny(num_histories=20000, seed=6, v_extent=0.3)
    cfg = _cfg(w, iterations=1, block_size=block)
    data, angles = phantoms.generate(w)
    ora = oracle.run_pipeline(cfg, data, angles, iterations=1)
    r = _through_rows(cfg, data, angles)
    r.drop(1)
    x = r.array("X").astype(np.float64)
    r.close()
    ref = ora["x_1"]
    assert np.linalg.norm(x - ref) <= DROP_TOL * np.linalg.norm(ref)


def test_gather_form_with_long_columns_against_oracle():
    """One block of every row on a small grid: hundreds of rows per voxel, so
    the gather form's column lists run to thousands of words per slice of 32
    voxels and hundreds of jagged-diagonal steps; the image still matches the
    oracle."""
    w = phantoms.tiny(num_histories=300000, seed=12, v_extent=0.3)
    cfg = _cfg(w, iterations=1, block_size=10_000_000, drop_form=3)
    data, angles = phantoms.generate(w)
    ora = oracle.run_pipeline(cfg, data, angles, iterations=1)
    r = _through_rows(cfg, data, angles)
    st = r.drop(1)
    counts = r.counts()
    x = r.array("X").astype(np.float64)
    r.close()
    assert st.drop_form == 3
    slices = (x.size + 31) // 32
    assert counts["drop_list_entries"] / slices > 8 * 1024  # long slices on average
    ref = ora["x_1"]
    assert np.linalg.norm(x - ref) <= DROP_TOL * np.linalg.norm(ref)


def test_odd_grid_without_bricks_against_oracle():
    w = phantoms.tiny(num_histories=30000, seed=8, v_extent=0.3)
    cfg = _cfg(w, columns=63, rows=65, ssd_v_size=2.25, iterations=2)  # 63x65x5: 20475 voxels
    g = phantoms.geometry(cfg)
    assert g.num_voxels % 4 != 0 and g.columns % 4 != 0
    data, angles = phantoms.generate(w)
    ora = oracle.run_pipeline(cfg, data, angles, iterations=2, keep_history=True)
    r = _through_rows(cfg, data, angles)
    offs, rows, _ = oracle.mlp_rows(cfg, ora["_hr"])
    assert np.array_equal(r.array("ROW_OFFSETS"), offs)
    assert np.array_equal(r.array("ROWS"), rows)
    r.drop(2)
    x = r.array("X").astype(np.float64)
    r.close()
    assert np.linalg.norm(x - ora["x_2"]) <= DROP_TOL * np.linalg.norm(ora["x_2"])


def test_linear_voxel_order_matches_bricks():
    w = phantoms.tiny(num_histories=30000, seed=9, v_extent=0.3)
    data, angles = phantoms.generate(w)
    out = {}
    for order in (0, 1):
        r = _through_rows(_cfg(w, voxel_order=order, iterations=2), data, angles)
        rows = r.array("ROWS")
        r.drop(2)
        out[order] = (rows, r.array("X").astype(np.float64))
        r.close()
    assert np.array_equal(out[0][0], out[1][0])  # the API returns linear indices either way
    a, b = out[0][1], out[1][1]
    assert np.linalg.norm(a - b) <= DROP_TOL * np.linalg.norm(a)


def test_residual_tolerance_stops_early():
    w = phantoms.tiny(num_histories=30000, seed=10, v_extent=0.3)
    data, angles = phantoms.generate(w)
    r = _through_rows(_cfg(w, iterations=12), data, angles)
    st = r.drop(12)
    first = st.residual[0]
    r.close()
    r = _through_rows(_cfg(w, iterations=12, residual_tol=first * 0.999), data, angles)
    st = r.drop(12)
    r.close()
    assert 1 <= st.iterations_run < 12


def test_status_codes():
    w = phantoms.tiny(num_histories=2000, seed=11)
    with pytest.raises(_capi.PctError) as e:
        recon.Reconstruction(_cfg(w, drop_form=7))
    assert e.value.status == _capi.PCT_ERR_ARGUMENT
    r = recon.Reconstruction(_cfg(w))
    with pytest.raises(_capi.PctError) as e:
        r.drop(1)  # no rows yet
    assert e.value.status == _capi.PCT_ERR_STATE
    with pytest.raises(_capi.PctError) as e:
        r.mlp_rows()
    assert e.value.status == _capi.PCT_ERR_STATE
    r.close()
