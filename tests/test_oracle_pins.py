"""The oracle against reference functions outside the driver sequence (CPU).

Fixtures with "pin.*" entries (tests/golden/make_golden.py, scenario `pins`)
hold the outputs of:
  write_MLP_endpoints (.cu:4684-4714)   the endpoint file itself;
  find_MLP_path_GPU_tabulated (.cu:5502-5660) on the reference's tables
                                       (.cu:4786-4911): rows of the first n
                                       recon histories;
  the CPU block loop (.cu:7525-7560) with DROP_blocks / DROP_update, DROP_blocks_red
  and DROP_blocks_robust2 / DROP_update_robust2 (.cu:7871-8055): the binary32
                                       iterate after `iterations` passes over
                                       the first n histories' reference rows.
Here the endpoint file is parsed by its documented layout and must hold the
recon histories of the same fixture bit for bit; the oracle's tabulated rows
of those histories must equal the reference's; and the oracle's binary64 DROP
loops must match the reference's binary32 ones within 1e-6 relative L2.
"""
import glob
import hashlib
import os

import numpy as np
import pytest

from oracle import oracle
from pct_gb300 import phantoms

HERE = os.path.dirname(os.path.abspath(__file__))
TOL = 1e-6
FIELDS = ("WEPL", "x_entry", "y_entry", "z_entry", "x_exit", "y_exit", "z_exit", "xy_entry_angle", "xz_entry_angle",
          "xy_exit_angle", "xz_exit_angle")


def pin_fixtures():
    out = []
    for p in sorted(glob.glob(os.path.join(HERE, "golden", "*.npz"))):
        with np.load(p, allow_pickle=False) as z:
            if "full:pin.MLP_endpoints_file" in z.files:
                out.append(p)
    return out


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def parse_endpoint_file(raw, columns, rows):
    """uint32 N, then int32 voxel_x/y/z, int32 bin, float32 WEPL, entry, exit and angles (N each)."""
    n = int(np.frombuffer(raw[:4], "<u4")[0])
    assert len(raw) == 4 + 60 * n
    ints = np.frombuffer(raw[4:4 + 16 * n], "<i4").reshape(4, n)
    floats = np.frombuffer(raw[4 + 16 * n:], "<f4").reshape(11, n)
    h = {f: floats[k].copy() for k, f in enumerate(FIELDS)}
    h["bin_num"] = ints[3].copy()
    h["first_voxel"] = (ints[0] + columns * ints[1] + columns * rows * ints[2]).astype(np.uint32)
    return h


@pytest.fixture(scope="module", params=pin_fixtures(), ids=lambda p: os.path.basename(p)[:-4])
def pinned(request):
    with np.load(request.param, allow_pickle=False) as z:
        fx = {k: z[k] for k in z.files}
    w = phantoms.tiny(num_histories=int(fx["num_histories"]), seed=int(fx["seed"]), v_extent=float(fx["v_extent"]))
    assert str(fx["workload"]) == "tiny"
    cfg = phantoms.make_config(w.config)
    h = parse_endpoint_file(fx["full:pin.MLP_endpoints_file"].tobytes(), cfg.columns, cfg.rows)
    return fx, cfg, h


def first(h, n):
    return {k: v[:n] for k, v in h.items()}


def test_endpoint_file_holds_the_recon_histories(pinned):
    fx, cfg, h = pinned
    assert len(h["WEPL"]) == int(fx["full:reconstruction_histories"][0])
    for f in FIELDS + ("bin_num",):
        assert sha(h[f]) == str(fx["sha:recon." + f]), f
    assert sha(h["first_voxel"]) == str(fx["sha:recon.first_MLP_voxel"])


def test_tabulated_rows_equal_the_reference(pinned):
    fx, cfg, h = pinned
    n = int(fx["full:pin.drop.setup"][0])
    offs, rows, _ = oracle.mlp_rows(cfg, first(h, n), tabulated=True)
    assert np.array_equal(offs, fx["full:pin.tab.offsets"])
    assert sha(rows) == str(fx["sha:pin.tab.rows"])


@pytest.mark.parametrize("variant", [0, 1, 2])
def test_drop_loops_within_tolerance(pinned, variant):
    fx, cfg, h = pinned
    n, block_size, iterations = (int(v) for v in fx["full:pin.drop.setup"])
    offs, rows, _ = oracle.mlp_rows(cfg, first(h, n))
    assert sha(offs) == str(fx["sha:mlp.offsets"]) and sha(rows) == str(fx["sha:mlp.rows"])
    chord = fx["full:mlp.chord"].astype(np.float64)
    eta = float(fx["full:pin.drop.eta"][variant])
    lam = float(np.float32(0.1))
    x = oracle.drop_variant(cfg, offs, rows, chord, h["WEPL"], fx["full:x_0"], iterations, block_size, lam,
                            variant, eta, 1)
    ref = fx["full:pin.drop.v%d" % variant].astype(np.float64)
    err = np.linalg.norm(x - ref) / np.linalg.norm(ref)
    assert err <= TOL, "variant %d: relative L2 %.3e" % (variant, err)
    if variant:
        # the variant's own effect is far above the tolerance
        std = fx["full:pin.drop.v0"].astype(np.float64)
        assert np.linalg.norm(ref - std) / np.linalg.norm(std) > 100 * TOL
