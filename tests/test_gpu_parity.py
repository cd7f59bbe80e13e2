"""CUDA path vs the CPU oracle, stage by stage (needs a GPU).

Bit-exact: per-history intersections and bins, hull counts and hulls, bin
means/sigmas (both sides add the reference's binary32 sums in history order),
cut masks, sinogram, filtered sinogram, FBP image, hull selection, initial
iterate, MLP endpoints and MLP voxel rows.  DROP: the binary32 GPU iterate against the oracle's binary64 run
of the same iterations, relative L2 <= 1e-4.
"""
import numpy as np
import pytest

from pct_gb300 import phantoms, recon
from oracle import oracle

pytestmark = pytest.mark.gpu

DROP_TOL = 1e-4
HIST_FIELDS = [("H_BIN_NUM", "bin_num"), ("H_WEPL", "WEPL"), ("H_X_ENTRY", "x_entry"), ("H_Y_ENTRY", "y_entry"),
               ("H_Z_ENTRY", "z_entry"), ("H_X_EXIT", "x_exit"), ("H_Y_EXIT", "y_exit"), ("H_Z_EXIT", "z_exit"),
               ("H_XY_ENTRY_ANGLE", "xy_entry_angle"), ("H_XZ_ENTRY_ANGLE", "xz_entry_angle"),
               ("H_XY_EXIT_ANGLE", "xy_exit_angle"), ("H_XZ_EXIT_ANGLE", "xz_exit_angle")]

CASES = {
    "tiny_clip": lambda: (phantoms.tiny(num_histories=40000, seed=11, v_extent=0.55), {}),
    "tiny_drop": lambda: (phantoms.tiny(num_histories=40000, seed=7, v_extent=0.3), {}),
    "cfg1_sm": lambda: (phantoms.cfg1(num_histories=120000, seed=5), dict(iterations=2)),
    # the benchmark's grid and phantom: 256x256x32 voxels, 180 angles
    "cfg2_grid": lambda: (phantoms.cfg2(num_histories=200000, seed=9), dict(iterations=2, block_size=50000)),
    # config 4's head phantom and grid: 320x320x64 voxels of 0.8 mm, 180 angles (binary32
    # chords here: the oracle's; the bfloat16 chords are checked by test_bf16_chords_error_stated)
    "cfg4_grid": lambda: (phantoms.cfg4(num_histories=200000, seed=9),
                          dict(iterations=2, block_size=50000, chord_bf16=0)),
    # config 3 grids at both ends: ellipsoid phantoms on 128x128x8 and 256x256x48
    "cfg3_128x8": lambda: (phantoms.ellipsoids(31, num_histories=150000, cols=128, slices=8),
                           dict(iterations=2, block_size=50000)),
    "cfg3_256x48": lambda: (phantoms.ellipsoids(32, num_histories=800000, cols=256, slices=48),
                            dict(iterations=2, block_size=50000)),
}


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and a.tobytes() == b.tobytes()


def mismatch(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.shape != b.shape:
        return "shape %s vs %s" % (a.shape, b.shape)
    d = np.nonzero(a.view(np.uint8).reshape(a.size, -1).any(axis=1) != 0)[0] if False else np.nonzero(a != b)[0]
    return "%d of %d differ, first at %s: %s vs %s" % (len(d), a.size, d[:3], a[d[:3]], b[d[:3]])


@pytest.fixture(scope="module", params=sorted(CASES))
def run(request):
    w, over = CASES[request.param]()
    cfg_over = dict(w.config)
    cfg_over.update(over)
    cfg = phantoms.make_config(cfg_over)
    data, angles = phantoms.generate(w)
    ora = oracle.run_pipeline(cfg, data, angles, keep_history=True)
    r = recon.Reconstruction(cfg)
    out = {}
    # three chunks of unequal size: the resident store must come out as one batch would
    n = data.shape[1]
    cuts = [0, n // 3, n // 3 + n // 5, n]
    for a, b in zip(cuts[:-1], cuts[1:]):
        r.process_chunk(data[:, a:b], angles[a:b])
    out["binned"] = {k: r.array(k) for k, _ in HIST_FIELDS}
    r.hull_detection_finish()
    for k in ("MSC_COUNTS", "SM_COUNTS", "MSC_HULL", "SM_HULL"):
        if (k.startswith("MSC") and cfg.msc_on) or (k.startswith("SM") and cfg.sm_on):
            out[k] = r.array(k)
    r.statistical_cuts()
    for k in ("BIN_COUNTS_PRE", "MEAN_WEPL", "MEAN_UT", "MEAN_UV", "SD_WEPL", "SD_UT", "SD_UV", "BIN_COUNTS_POST",
              "SINOGRAM"):
        out[k] = r.array(k)
    out["cut"] = {k: r.array(k) for k, _ in HIST_FIELDS}
    r.FBP()
    out["SINOGRAM_FILTERED"], out["FBP_IMAGE"], out["FBP_HULL"] = (r.array("SINOGRAM_FILTERED"), r.array("FBP_IMAGE"),
                                                                   r.array("FBP_HULL"))
    r.hull_selection()
    out["X_HULL"], out["X_HULL_FILTERED"] = r.array("X_HULL"), r.array("X_HULL_FILTERED")
    r.define_initial_iterate()
    out["X0"] = r.array("X0")
    r.collect_mlp_endpoints()
    out["recon"] = {k: r.array(k) for k, _ in HIST_FIELDS}
    out["recon"]["H_FIRST_VOXEL"] = r.array("H_FIRST_VOXEL")
    r.mlp_rows()
    out["ROW_OFFSETS"], out["ROWS"], out["CHORD"] = r.array("ROW_OFFSETS"), r.array("ROWS"), r.array("CHORD")
    its = cfg.iterations
    stats = r.drop(its)
    out["X"] = r.array("X")
    out["stats"] = stats
    out["counts"] = r.counts()
    r.close()
    return request.param, cfg, ora, out


def test_history_counts(run):
    name, cfg, ora, out = run
    c = out["counts"]
    assert c["total_histories"] == int(ora["total_histories"][0])
    assert c["recon_vol_histories"] == int(ora["recon_vol_histories"][0])
    assert c["post_cut_histories"] == int(ora["post_cut_histories"][0])
    assert c["reconstruction_histories"] == int(ora["reconstruction_histories"][0])
    assert c["walks_capped"] == 0


@pytest.mark.parametrize("stage", ["binned", "cut", "recon"])
def test_history_store_bit_exact(run, stage):
    name, cfg, ora, out = run
    for k, f in HIST_FIELDS:
        assert same(out[stage][k], ora[stage + "." + f]), "%s %s: %s" % (stage, k, mismatch(out[stage][k], ora[stage + "." + f]))
    if stage == "recon":
        assert same(out["recon"]["H_FIRST_VOXEL"], ora["recon.first_MLP_voxel"])


def test_hulls_bit_exact(run):
    name, cfg, ora, out = run
    if cfg.msc_on:
        assert same(out["MSC_COUNTS"], ora["MSC_counts_h"]), mismatch(out["MSC_COUNTS"], ora["MSC_counts_h"])
        assert same(out["MSC_HULL"], ora["x_MSC"])
    if cfg.sm_on:
        assert same(out["SM_COUNTS"], ora["SM_counts_h"]), mismatch(out["SM_COUNTS"], ora["SM_counts_h"])
        assert same(out["SM_HULL"], ora["x_SM"])
    assert same(out["X_HULL"], ora["x_hull"])
    assert same(out["X_HULL_FILTERED"], ora["x_hull_filtered"])


def test_bin_statistics_and_sinogram_bit_exact(run):
    name, cfg, ora, out = run
    pairs = [("BIN_COUNTS_PRE", "bin_counts_h_pre"), ("MEAN_WEPL", "mean_WEPL_h"), ("MEAN_UT", "mean_rel_ut_angle_h"),
             ("MEAN_UV", "mean_rel_uv_angle_h"), ("SD_WEPL", "stddev_WEPL_h"), ("SD_UT", "stddev_rel_ut_angle_h"),
             ("SD_UV", "stddev_rel_uv_angle_h"), ("BIN_COUNTS_POST", "bin_counts_post"), ("SINOGRAM", "sinogram")]
    for k, o in pairs:
        assert same(out[k], ora[o]), "%s: %s" % (k, mismatch(out[k], ora[o]))


def test_fbp_bit_exact(run):
    name, cfg, ora, out = run
    assert same(out["SINOGRAM_FILTERED"], ora["sinogram_filtered"]), mismatch(out["SINOGRAM_FILTERED"], ora["sinogram_filtered"])
    assert same(out["FBP_IMAGE"], ora["FBP_image_h"]), mismatch(out["FBP_IMAGE"], ora["FBP_image_h"])
    assert same(out["FBP_HULL"], ora["x_FBP"])
    assert same(out["X0"], ora["x_k0"])


def test_mlp_rows_bit_exact(run):
    name, cfg, ora, out = run
    offs, rows, chord = oracle.mlp_rows(cfg, ora["_hr"])
    assert same(out["ROW_OFFSETS"], offs), mismatch(out["ROW_OFFSETS"], offs)
    assert same(out["ROWS"], rows), mismatch(out["ROWS"], rows)
    assert same(out["CHORD"], chord.astype(np.float32))


def test_mlp_fast_path_used_and_exact_mode_agrees(run):
    """The binary32 path must do most samples; an all-binary64 run must give the same rows."""
    name, cfg, ora, out = run
    c = out["counts"]
    total_samples = int(out["ROW_OFFSETS"][-1])
    assert c["mlp_fp64_samples"] < 0.2 * max(total_samples, 1), c
    cfg2 = phantoms.make_config({})
    for f, _ in cfg._fields_:
        setattr(cfg2, f, getattr(cfg, f))
    cfg2.mlp_exact = 1
    w, _ = CASES[name]()
    data, angles = phantoms.generate(w)
    r = recon.run_full(cfg2, data, angles)
    r.collect_mlp_endpoints()
    r.mlp_rows()
    rows = r.array("ROWS")
    r.close()
    assert same(rows, out["ROWS"])


def test_drop_within_tolerance_of_fp64(run):
    name, cfg, ora, out = run
    its = cfg.iterations
    if its == 0:
        pytest.skip("no iterations")
    ref = ora["x_%d" % its]
    err = np.linalg.norm(out["X"].astype(np.float64) - ref) / np.linalg.norm(ref)
    assert err <= DROP_TOL, "relative L2 %.3e" % err
    st = out["stats"]
    assert st.iterations_run == its
    assert all(np.isfinite(st.residual[k]) and st.residual[k] > 0 for k in range(its))


def test_drop_fp64_mode_matches_the_binary64_oracle(run):
    """pct_drop_fp64 (binary64 chord, dot, update and iterate on the GPU) against the
    oracle's binary64 DROP of the same iterations: they differ only in the order of
    the binary64 update sums; and the binary32 iterate stays within 1e-4 of it."""
    name, cfg, ora, out = run
    its = cfg.iterations
    if its == 0:
        pytest.skip("no iterations")
    w, _ = CASES[name]()
    data, angles = phantoms.generate(w)
    r = recon.run_full(cfg, data, angles)
    r.collect_mlp_endpoints()
    r.mlp_rows()
    x0 = r.array("X0")
    x64, st = r.drop_fp64(its, x0)
    assert same(r.array("X"), x0), "pct_drop_fp64 changed the binary32 iterate"
    r.close()
    ref = ora["x_%d" % its]
    err = np.linalg.norm(x64 - ref) / np.linalg.norm(ref)
    assert err <= 1e-9, "binary64 GPU vs oracle: relative L2 %.3e" % err
    err32 = np.linalg.norm(out["X"].astype(np.float64) - x64) / np.linalg.norm(x64)
    assert err32 <= DROP_TOL, "binary32 vs binary64 GPU: relative L2 %.3e" % err32
    assert st.iterations_run == its and all(st.residual[k] > 0 for k in range(its))


@pytest.mark.parametrize("form", [1, 2, 3])
def test_drop_other_forms_within_tolerance(run, form):
    """The sorted (1), tiled (2) and gather (3) forms of the DROP block step against the
    same binary64 iterate (the default scatter form is checked above); the form
    asked for is the one that ran."""
    name, cfg, ora, out = run
    its = cfg.iterations
    if its == 0:
        pytest.skip("no iterations")
    cfg2 = phantoms.make_config({})
    for f, _ in cfg._fields_:
        setattr(cfg2, f, getattr(cfg, f))
    cfg2.drop_form = form
    w, _ = CASES[name]()
    data, angles = phantoms.generate(w)
    r = recon.run_full(cfg2, data, angles)
    r.collect_mlp_endpoints()
    r.mlp_rows()
    st = r.drop(its)
    x = r.array("X").astype(np.float64)
    r.close()
    assert st.drop_form == form
    ref = ora["x_%d" % its]
    err = np.linalg.norm(x - ref) / np.linalg.norm(ref)
    assert err <= DROP_TOL, "relative L2 %.3e" % err


def test_drop_tiled_form_is_reproducible(run):
    """The tiled form accumulates the dots and the block updates in integers:
    repeating the same iterations, in this context or a new one, gives the
    same image bit for bit."""
    name, cfg, ora, out = run
    its = cfg.iterations
    if its == 0:
        pytest.skip("no iterations")
    cfg2 = phantoms.make_config({})
    for f, _ in cfg._fields_:
        setattr(cfg2, f, getattr(cfg, f))
    cfg2.drop_form = 2
    w, over = CASES[name]()
    data, angles = phantoms.generate(w)
    images = []
    for rep in range(2):
        r = recon.run_full(cfg2, data, angles)
        r.collect_mlp_endpoints()
        r.mlp_rows()
        for _ in range(2 - rep):
            r.reset_iterate()
            r.drop(its)
            images.append(r.array("X"))
        r.close()
    assert same(images[0], images[1])
    assert same(images[0], images[2])


@pytest.mark.parametrize("form", [0, 1])
@pytest.mark.parametrize("variant", [1, 2])
def test_drop_variants_within_tolerance(run, variant, form):
    """DROP_blocks_red (1) and DROP_blocks_robust2 + DROP_update_robust2 (2) on
    the GPU against the oracle's binary64 run of the same iterations.  The
    variants divide by ||a||^2 + psi (1) or ||A||_j + psi_j (2) with
    psi = (1 - x) eta psi_sign, which passes through zero where the FBP start
    strays from 1 by more than the smallest ||a||^2 (or c^2) over eta; there
    the update is singular and even binary64 runs one ulp apart disagree (the
    reference default eta = 2.5 is such a case).  eta is therefore chosen per
    scan so that |psi| stays below 5% of the smallest denominator, and the
    variant's effect on the image must exceed 10x the GPU's distance to the
    oracle."""
    name, cfg, ora, out = run
    its = cfg.iterations
    if its == 0:
        pytest.skip("no iterations")
    offs, rows, chord = oracle.mlp_rows(cfg, ora["_hr"])
    x0 = ora["x_k0"].astype(np.float64)
    span = max(1e-3, float(np.abs(1.0 - x0).max()))
    denom = float((chord * chord * np.diff(offs)).min()) if variant == 1 else float((chord * chord).min())
    eta = min(0.05 if variant == 1 else 0.005, 0.05 * denom / span)
    cfg2 = phantoms.make_config({})
    for f, _ in cfg._fields_:
        setattr(cfg2, f, getattr(cfg, f))
    cfg2.drop_variant = variant
    cfg2.drop_form = form
    cfg2.eta = eta
    cfg2.psi_sign = 1
    w, _ = CASES[name]()
    data, angles = phantoms.generate(w)
    r = recon.run_full(cfg2, data, angles)
    r.collect_mlp_endpoints()
    r.mlp_rows()
    st = r.drop(its)
    x = r.array("X").astype(np.float64)
    r.close()
    assert st.drop_form == form
    ref = oracle.drop_variant(cfg, offs, rows, chord, ora["_hr"]["WEPL"], ora["x_k0"], its, cfg.block_size,
                              float(np.float32(cfg.lambda_)), variant, eta, 1)
    std = ora["x_%d" % its]
    err = np.linalg.norm(x - ref) / np.linalg.norm(ref)
    change = np.linalg.norm(ref - std) / np.linalg.norm(std)
    assert err <= DROP_TOL, "relative L2 %.3e (eta %.2e)" % (err, eta)
    assert change > 10 * err, "variant effect %.3e vs error %.3e (eta %.2e)" % (change, err, eta)


def test_bf16_chords_error_stated(run):
    """chord_bf16: the chord lengths are the oracle's rounded to bfloat16 bit for
    bit; the DROP iterate is within the DROP tolerance of the binary64 run on
    those chords, and its distance to the binary64 run on binary64 chords is
    the stated cost of bf16 chords (printed, bounded by 2^-8 relative)."""
    name, cfg, ora, out = run
    its = cfg.iterations
    if its == 0:
        pytest.skip("no iterations")
    cfg2 = phantoms.make_config({})
    for f, _ in cfg._fields_:
        setattr(cfg2, f, getattr(cfg, f))
    cfg2.chord_bf16 = 1
    w, _ = CASES[name]()
    data, angles = phantoms.generate(w)
    r = recon.run_full(cfg2, data, angles)
    r.collect_mlp_endpoints()
    r.mlp_rows()
    chord = r.array("CHORD")
    r.drop(its)
    x = r.array("X").astype(np.float64)
    r.close()
    offs, rows, chord64 = oracle.mlp_rows(cfg, ora["_hr"])
    c32 = chord64.astype(np.float32)
    u = c32.view(np.uint32).astype(np.uint64)
    bf = (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16).astype(np.uint32).view(np.float32)  # round to nearest even
    assert chord.tobytes() == bf.tobytes()
    ref_bf = oracle.drop(cfg, offs, rows, bf.astype(np.float64), ora["_hr"]["WEPL"], ora["x_k0"], its, cfg.block_size,
                         float(np.float32(cfg.lambda_)))
    err_bf = np.linalg.norm(x - ref_bf) / np.linalg.norm(ref_bf)
    ref = ora["x_%d" % its]
    err = np.linalg.norm(x - ref) / np.linalg.norm(ref)
    print("%s: bf16 chords, relative L2 vs binary64 on bf16 chords %.2e, vs binary64 on binary64 chords %.2e"
          % (name, err_bf, err))
    assert err_bf <= DROP_TOL
    assert err <= 2.0 ** -8


def test_tabulated_mlp_rows_bit_exact(run):
    """The tabulated MLP (mlp_tabulated = 1, find_MLP_path_GPU_tabulated) against
    the oracle's restatement of it: the same rows bit for bit; the chords are the
    analytic ones in both."""
    name, cfg, ora, out = run
    cfg2 = phantoms.make_config({})
    for f, _ in cfg._fields_:
        setattr(cfg2, f, getattr(cfg, f))
    cfg2.mlp_tabulated = 1
    w, _ = CASES[name]()
    data, angles = phantoms.generate(w)
    r = recon.run_full(cfg2, data, angles)
    r.collect_mlp_endpoints()
    r.mlp_rows()
    offs_g, rows_g, chord_g = r.array("ROW_OFFSETS"), r.array("ROWS"), r.array("CHORD")
    r.close()
    offs, rows, chord = oracle.mlp_rows(cfg, ora["_hr"], tabulated=True)
    assert same(offs_g, offs), mismatch(offs_g, offs)
    assert same(rows_g, rows), mismatch(rows_g, rows)
    assert same(chord_g, chord.astype(np.float32))
