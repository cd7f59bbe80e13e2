"""CUDA path vs the reference's own outputs, stage by stage (needs a GPU).

tests/golden/*.npz hold digests (and heads or full copies) of every stage of
the unmodified reference driver sequence, run on seeded synthetic scans by
tests/golden/make_golden.py.  Here each scan is regenerated, driven through the
library's reference-order stage calls (in three chunks of unequal size) and
every captured stage is compared with the fixture: bit for bit for the
history store after binning, cuts and endpoints, the bin counts, means,
sigmas, cut masks, sinogram, hulls, FBP image, initial iterate, first MLP
voxels, MLP rows and chords; the DROP iterates within 1e-4 relative L2 of the
reference's binary32 run.
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
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
DROP_TOL = 1e-4
HIST = [("bin_num", "H_BIN_NUM"), ("WEPL", "H_WEPL"), ("x_entry", "H_X_ENTRY"), ("y_entry", "H_Y_ENTRY"),
        ("z_entry", "H_Z_ENTRY"), ("x_exit", "H_X_EXIT"), ("y_exit", "H_Y_EXIT"), ("z_exit", "H_Z_EXIT"),
        ("xy_entry_angle", "H_XY_ENTRY_ANGLE"), ("xz_entry_angle", "H_XZ_ENTRY_ANGLE"),
        ("xy_exit_angle", "H_XY_EXIT_ANGLE"), ("xz_exit_angle", "H_XZ_EXIT_ANGLE")]
BINS = [("bin_counts_h_pre", "BIN_COUNTS_PRE"), ("mean_WEPL_h", "MEAN_WEPL"), ("mean_rel_ut_angle_h", "MEAN_UT"),
        ("mean_rel_uv_angle_h", "MEAN_UV"), ("stddev_WEPL_h", "SD_WEPL"), ("stddev_rel_ut_angle_h", "SD_UT"),
        ("stddev_rel_uv_angle_h", "SD_UV"), ("bin_counts_post", "BIN_COUNTS_POST"),
        ("bin_counts_pre", "BIN_COUNTS_POST"), ("sinogram", "SINOGRAM")]
WORKLOADS = {"tiny": phantoms.tiny, "cfg1": phantoms.cfg1, "cfg2": phantoms.cfg2, "cfg4": phantoms.cfg4}


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def workload_of(fx):
    if str(fx["workload"]).startswith("ellipsoids_"):
        return phantoms.ellipsoids(int(fx["seed"]), num_histories=int(fx["num_histories"]),
                                   cols=int(fx["grid_cols"]), slices=int(fx["grid_slices"]))
    kw = dict(num_histories=int(fx["num_histories"]), seed=int(fx["seed"]))
    if str(fx["workload"]) == "tiny":
        kw["v_extent"] = float(fx["v_extent"])
    return WORKLOADS[str(fx["workload"])](**kw)


@pytest.fixture(scope="module", params=FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def golden(request):
    with np.load(request.param, allow_pickle=False) as z:
        fx = {k: z[k] for k in z.files}
    w = workload_of(fx)
    data, angles = phantoms.generate(w)
    assert sha(data) + sha(angles) == str(fx["input_sha"]), "synthetic inputs differ from the fixture's"
    cfg = phantoms.make_config(w.config)
    cfg.chord_bf16 = 0  # the reference's chords are binary32
    run = ast.literal_eval(str(fx["run_config"]))
    for k in ("msc_on", "sm_on", "sc_on", "mlp_hull"):
        if k in run:
            setattr(cfg, k, run[k])
    cfg.block_size = int(run.get("block_size", 3200))
    cfg.lambda_ = float(np.float32(run.get("lambda_", 0.001)))
    got = {}
    r = recon.Reconstruction(cfg)
    try:
        n = data.shape[1]
        for a, b in zip([0, n // 3, n // 3 + n // 5], [n // 3, n // 3 + n // 5, n]):
            r.process_chunk(data[:, a:b], angles[a:b])
        for f, k in HIST:
            got["binned." + f] = r.array(k)
        r.hull_detection_finish()
        if cfg.msc_on:
            got["MSC_counts_h"], got["x_MSC"] = r.array("MSC_COUNTS"), r.array("MSC_HULL")
        if cfg.sm_on:
            got["SM_counts_h"], got["x_SM"] = r.array("SM_COUNTS"), r.array("SM_HULL")
        r.statistical_cuts()
        for f, k in BINS:
            got[f] = r.array(k)
        for f, k in HIST:
            got["cut." + f] = r.array(k)
        r.FBP()
        got["FBP_image_h"], got["x_FBP"] = r.array("FBP_IMAGE"), r.array("FBP_HULL")
        r.hull_selection()
        got["x_hull"], got["x_hull_filtered"] = r.array("X_HULL"), r.array("X_HULL_FILTERED")
        r.define_initial_iterate()
        got["x_k0"] = got["x_0"] = r.array("X0")
        r.collect_mlp_endpoints()
        for f, k in HIST:
            got["recon." + f] = r.array(k)
        got["recon.first_MLP_voxel"] = r.array("H_FIRST_VOXEL")
        r.mlp_rows()
        m = int(fx["shape:mlp.chord"][0])
        offs = r.array("ROW_OFFSETS")[: m + 1]
        got["mlp.offsets"] = offs
        got["mlp.rows"] = r.array("ROWS")[: offs[-1]]
        got["_chord"] = r.array("CHORD")[:m]
        iters = int(run.get("iterations", 0))
        for it in range(1, iters + 1):
            r.drop(1)
            got["x_%d" % it] = r.array("X")
        c = r.counts()
        for k in ("total_histories", "recon_vol_histories", "post_cut_histories", "reconstruction_histories"):
            got[k] = np.array([c[k]], np.int32)
    finally:
        r.close()
    return os.path.basename(request.param)[:-4], fx, got


def _digest_names(fx):
    return sorted(k[4:] for k in fx if k.startswith("sha:"))


def _first_difference(fx, name, a):
    for pre in ("full:", "head:"):
        if pre + name in fx:
            want = fx[pre + name]
            a = np.asarray(a).ravel()[: want.size].astype(want.dtype)
            d = np.nonzero(a != want)[0]
            if len(d):
                return "first of %s differs at %d: %s vs %s" % (pre[:-1], d[0], a[d[0]], want[d[0]])
    return "digest differs"


def test_every_stage_equals_the_reference(golden):
    name, fx, got = golden
    skip = {"x_final", "sinogram_pre", "mlp.chord"}
    bad, checked = [], 0
    for k in _digest_names(fx):
        if k in skip or k.startswith("pin.") or (k.startswith("x_") and k[2:].isdigit() and k != "x_0"):
            continue
        assert k in got, "stage %s not produced" % k
        want_dtype = str(fx["dtype:" + k])
        a = np.asarray(got[k])
        if str(a.dtype) != want_dtype:
            a = a.astype(want_dtype)
        if tuple(a.shape) != tuple(fx["shape:" + k]) or sha(a) != str(fx["sha:" + k]):
            bad.append("%s (%s)" % (k, _first_difference(fx, k, a)))
        checked += 1
    assert checked >= 60, checked
    assert not bad, "%s: stages differ from the reference: %s" % (name, bad)


def test_chords_equal_the_reference(golden):
    """The reference's chord is binary64 (EffectiveChordLength_GPU, .cu:4974-4995); the
    rows keep it rounded to binary32."""
    name, fx, got = golden
    want = fx["full:mlp.chord"].astype(np.float32)
    assert got["_chord"].tobytes() == want.tobytes()


def test_drop_iterates_within_tolerance(golden):
    name, fx, got = golden
    its = sorted(k for k in _digest_names(fx) if k.startswith("x_") and k[2:].isdigit() and k != "x_0")
    if not its:
        pytest.skip("the fixture's scenario stops before DROP")
    for k in its:
        ref = fx["full:" + k].astype(np.float64)
        err = np.linalg.norm(got[k].astype(np.float64) - ref) / np.linalg.norm(ref)
        assert err <= DROP_TOL, "%s %s: relative L2 %.3e" % (name, k, err)
