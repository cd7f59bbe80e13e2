"""The CUDA path against reference functions outside the driver sequence (needs a GPU).

The fixtures with "pin.*" entries (tests/golden/make_golden.py, scenario
`pins`) hold the endpoint file the reference's write_MLP_endpoints
(src/pCT_Reconstruction_Data_Segments.cu:4684-4714) wrote, the rows of
find_MLP_path_GPU_tabulated (.cu:5502-5660) on the reference's tables
(.cu:4786-4911), and the binary32 iterates of the CPU reconstruction's block
loop (.cu:7525-7560) with DROP_blocks, DROP_blocks_red and
DROP_blocks_robust2 / DROP_update_robust2 (.cu:7871-8055).  Here:
  - pct_read_mlp_endpoints reads the reference's file: every history array and
    first voxel bit for bit;
  - pct_write_mlp_endpoints, after the library's own pipeline on the same
    scan, writes the same bytes;
  - from the first n histories of that file (the same layout, cut to n), the
    analytic and the tabulated MLP rows equal the reference's bit for bit;
  - DROP from x_0 on those rows, block size and variant as the reference loop,
    within 1e-4 relative L2 of the reference's iterate (scatter and sorted
    forms), and each variant's own effect more than 10x that distance.
"""
import ast
import glob
import hashlib
import os

import numpy as np
import pytest

from pct_gb300 import phantoms, recon

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
DROP_TOL = 1e-4
HIST = [("bin_num", "H_BIN_NUM"), ("WEPL", "H_WEPL"), ("x_entry", "H_X_ENTRY"), ("y_entry", "H_Y_ENTRY"),
        ("z_entry", "H_Z_ENTRY"), ("x_exit", "H_X_EXIT"), ("y_exit", "H_Y_EXIT"), ("z_exit", "H_Z_EXIT"),
        ("xy_entry_angle", "H_XY_ENTRY_ANGLE"), ("xz_entry_angle", "H_XZ_ENTRY_ANGLE"),
        ("xy_exit_angle", "H_XY_EXIT_ANGLE"), ("xz_exit_angle", "H_XZ_EXIT_ANGLE")]


def pin_fixtures():
    out = []
    for p in sorted(glob.glob(os.path.join(HERE, "golden", "*.npz"))):
        with np.load(p, allow_pickle=False) as z:
            if "full:pin.MLP_endpoints_file" in z.files:
                out.append(p)
    return out


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def cut_endpoint_file(raw, n):
    """The first n histories of an endpoint file, in the same layout."""
    total = int(np.frombuffer(raw[:4], "<u4")[0])
    ints = np.frombuffer(raw[4:4 + 16 * total], "<i4").reshape(4, total)[:, :n]
    floats = np.frombuffer(raw[4 + 16 * total:], "<f4").reshape(11, total)[:, :n]
    return np.array([n], "<u4").tobytes() + np.ascontiguousarray(ints).tobytes() + np.ascontiguousarray(floats).tobytes()


def config(fx, **over):
    w = phantoms.tiny(num_histories=int(fx["num_histories"]), seed=int(fx["seed"]), v_extent=float(fx["v_extent"]))
    c = dict(w.config)
    run = ast.literal_eval(str(fx["run_config"]))
    for k in ("msc_on", "sm_on", "sc_on", "mlp_hull"):
        if k in run:
            c[k] = run[k]
    c.update(over)
    return w, phantoms.make_config(c)


@pytest.fixture(scope="module", params=pin_fixtures(), ids=lambda p: os.path.basename(p)[:-4])
def pinned(request, tmp_path_factory):
    with np.load(request.param, allow_pickle=False) as z:
        fx = {k: z[k] for k in z.files}
    assert str(fx["workload"]) == "tiny"
    d = tmp_path_factory.mktemp("pins")
    raw = fx["full:pin.MLP_endpoints_file"].tobytes()
    (d / "reference.bin").write_bytes(raw)
    n = int(fx["full:pin.drop.setup"][0])
    (d / "first.bin").write_bytes(cut_endpoint_file(raw, n))
    return fx, d


def test_reads_the_reference_endpoint_file(pinned):
    fx, d = pinned
    w, cfg = config(fx)
    r = recon.Reconstruction(cfg)
    try:
        r.read_mlp_endpoints(d / "reference.bin")
        for f, k in HIST:
            assert sha(r.array(k)) == str(fx["sha:recon." + f]), f
        assert sha(r.array("H_FIRST_VOXEL")) == str(fx["sha:recon.first_MLP_voxel"])
    finally:
        r.close()


def test_writes_the_reference_endpoint_file(pinned):
    fx, d = pinned
    w, cfg = config(fx)
    data, angles = phantoms.generate(w)
    r = recon.run_full(cfg, data, angles)
    try:
        r.collect_mlp_endpoints()
        r.write_mlp_endpoints(d / "library.bin")
    finally:
        r.close()
    assert (d / "library.bin").read_bytes() == fx["full:pin.MLP_endpoints_file"].tobytes()


@pytest.mark.parametrize("tabulated", [0, 1])
def test_rows_from_the_reference_file(pinned, tabulated):
    fx, d = pinned
    n = int(fx["full:pin.drop.setup"][0])
    w, cfg = config(fx, mlp_tabulated=tabulated)
    r = recon.Reconstruction(cfg)
    try:
        r.read_mlp_endpoints(d / "first.bin")
        r.set_image(fx["full:x_0"])
        r.mlp_rows()
        offs = r.array("ROW_OFFSETS")[: n + 1]
        rows = r.array("ROWS")[: offs[-1]]
        chord = r.array("CHORD")[:n]
    finally:
        r.close()
    if tabulated:
        assert np.array_equal(offs, fx["full:pin.tab.offsets"])
        assert sha(rows) == str(fx["sha:pin.tab.rows"])
    else:
        assert sha(offs) == str(fx["sha:mlp.offsets"]) and sha(rows) == str(fx["sha:mlp.rows"])
        assert chord.tobytes() == fx["full:mlp.chord"].astype(np.float32).tobytes()


@pytest.mark.parametrize("form", [0, 1])
@pytest.mark.parametrize("variant", [0, 1, 2])
def test_drop_loops_within_tolerance(pinned, variant, form):
    fx, d = pinned
    n, block_size, iterations = (int(v) for v in fx["full:pin.drop.setup"])
    eta = float(fx["full:pin.drop.eta"][variant])
    w, cfg = config(fx, drop_variant=variant, drop_form=form, eta=eta, psi_sign=1, block_size=block_size,
                    lambda_=0.1)
    r = recon.Reconstruction(cfg)
    try:
        r.read_mlp_endpoints(d / "first.bin")
        r.set_image(fx["full:x_0"])
        r.mlp_rows()
        st = r.drop(iterations)
        x = r.array("X").astype(np.float64)
    finally:
        r.close()
    assert st.drop_form == form
    ref = fx["full:pin.drop.v%d" % variant].astype(np.float64)
    err = np.linalg.norm(x - ref) / np.linalg.norm(ref)
    assert err <= DROP_TOL, "variant %d: relative L2 %.3e" % (variant, err)
    if variant:
        std = fx["full:pin.drop.v0"].astype(np.float64)
        change = np.linalg.norm(ref - std) / np.linalg.norm(std)
        assert change > 10 * err, "variant effect %.3e vs error %.3e" % (change, err)
