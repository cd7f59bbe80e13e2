"""Python driver for the C oracle (test infrastructure only).

Wraps oracle/_build/libpct_oracle.so and chains its stages in the order of
the reference's main() (src/pCT_Reconstruction_Data_Segments.cu:42-226), with
output names matching the reference harness captures (oracle/refharness.py),
so a test can compare the two stage by stage.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from pct_gb300 import _capi  # noqa: E402
from oracle import build_oracle  # noqa: E402

_lib = None


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


# pct_allreduce_fn (include/pct.h): user, data, count, dtype, on_device -> 0 on success
ALLREDUCE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_int)


def load():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        _lib = C.CDLL(path)
        _lib.ora_mlp_rows.restype = C.c_int64
        _lib.ora_mlp_rows_tab.restype = C.c_int64
        _lib.ora_effective_chord_length.restype = C.c_double
        _lib.ora_effective_chord_length.argtypes = [C.c_void_p, C.c_double, C.c_double]
        _lib.ora_drop.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_int, C.c_int, C.c_double, C.c_void_p]
        _lib.ora_mlp_rows_mt.restype = C.c_int64
        _lib.ora_drop_variant.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_int, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int, C.c_void_p]
        _lib.ora_drop_mt.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_int, C.c_int, C.c_double, C.c_void_p, C.c_int]
        _lib.ora_drop_shard.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_int, C.c_int, C.c_int, C.c_double, C.c_void_p, ALLREDUCE_FN, C.c_void_p]
    return _lib


def _cfgp(cfg):
    return C.byref(cfg)


def geometry(cfg):
    g = _capi.Geometry()
    assert load().ora_geometry(_cfgp(cfg), C.byref(g)) == 0, "invalid geometry"
    return g


def make_config(overrides):
    """pct_config with the reference's defaults and the given overrides (no CUDA library)."""
    cfg = _capi.Config()
    load().ora_config_default(C.byref(cfg))
    for k, v in overrides.items():
        setattr(cfg, k, v)
    return cfg


_gen = None


def generate(w):
    """The seeded histories of workload `w` (pct_gb300.phantoms) from the host-only build of the
    generator: ((13, N) float32 PCTD arrays in mm, (N,) float32 projection angles), the same bits
    as phantoms.generate without mapping the CUDA library."""
    global _gen
    if _gen is None:
        _gen = C.CDLL(build_oracle.build_gen())
        _gen.pct_gen_last_error.restype = C.c_char_p
    n = int(w.num_histories)
    data = np.empty((13, n), dtype=np.float32)
    angles = np.empty(n, dtype=np.float32)
    sp = _capi.ScanParams(seed=w.seed, num_angles=w.num_angles, gantry_angle_interval=w.gantry_angle_interval,
                          t_extent=w.t_extent, v_extent=w.v_extent, source_radius=260.7,
                          angular_spread=w.angular_spread, beam_energy_mev=200.0, wepl_noise=w.wepl_noise,
                          outlier_fraction=w.outlier_fraction, outlier_max=w.outlier_max,
                          scatter_scale=w.scatter_scale)
    objs = (_capi.PhantomObject * max(1, len(w.objects)))()
    for i, o in enumerate(w.objects):
        objs[i] = _capi.PhantomObject(*o)
    ptrs = (C.c_void_p * 13)(*[data[k].ctypes.data for k in range(13)])
    rc = _gen.pct_generate_histories(objs, len(w.objects), C.byref(sp), ptrs, C.c_void_p(angles.ctypes.data),
                                     C.c_int64(n))
    assert rc == 0, _gen.pct_gen_last_error().decode(errors="replace")
    return data, angles


HIST_FIELDS = ["x_entry", "y_entry", "z_entry", "x_exit", "y_exit", "z_exit",
               "xy_entry_angle", "xz_entry_angle", "xy_exit_angle", "xz_exit_angle"]


def preprocess(cfg, data13, proj_angle):
    lib = load()
    n = data13.shape[1]
    data13 = np.ascontiguousarray(data13, dtype=np.float32)
    proj_angle = np.ascontiguousarray(proj_angle, dtype=np.float32)
    out = {"gantry_angle": np.empty(n, np.int32), "missed": np.empty(n, np.uint8), "bin_num": np.empty(n, np.int32),
           "bin_valid": np.empty(n, np.uint8), "WEPL": np.empty(n, np.float32)}
    for f in HIST_FIELDS:
        out[f] = np.empty(n, np.float32)
    ins = (C.c_void_p * 13)(*[data13[k].ctypes.data for k in range(13)])
    rc = lib.ora_preprocess(_cfgp(cfg), C.c_int64(n), ins, _p(proj_angle), _p(out["gantry_angle"]), _p(out["missed"]),
                            _p(out["bin_num"]), _p(out["bin_valid"]), *[_p(out[f]) for f in HIST_FIELDS], _p(out["WEPL"]))
    assert rc == 0
    return out


def bin_statistics(cfg, h):
    lib = load()
    g = geometry(cfg)
    nb = g.num_bins
    r = {k: np.empty(nb, np.float32) for k in ("mean_WEPL", "mean_ut", "mean_uv", "sd_WEPL", "sd_ut", "sd_uv")}
    r["counts"] = np.empty(nb, np.int32)
    n = len(h["bin_num"])
    rc = lib.ora_bin_statistics(_cfgp(cfg), C.c_int64(n), _p(h["bin_num"]), _p(h["bin_valid"]), _p(h["WEPL"]),
                                _p(h["xy_entry_angle"]), _p(h["xz_entry_angle"]), _p(h["xy_exit_angle"]),
                                _p(h["xz_exit_angle"]), _p(r["counts"]), _p(r["mean_WEPL"]),
                                _p(r["mean_ut"]), _p(r["mean_uv"]), _p(r["sd_WEPL"]), _p(r["sd_ut"]), _p(r["sd_uv"]))
    assert rc == 0
    return r


def statistical_cuts(cfg, h, st):
    lib = load()
    g = geometry(cfg)
    n = len(h["bin_num"])
    failed = np.empty(n, np.uint8)
    counts = np.empty(g.num_bins, np.int32)
    sino = np.empty(g.num_bins, np.float32)
    rc = lib.ora_statistical_cuts(_cfgp(cfg), C.c_int64(n), _p(h["bin_num"]), _p(h["WEPL"]), _p(h["xy_entry_angle"]),
                                  _p(h["xz_entry_angle"]), _p(h["xy_exit_angle"]), _p(h["xz_exit_angle"]),
                                  _p(st["mean_WEPL"]), _p(st["mean_ut"]), _p(st["mean_uv"]), _p(st["sd_WEPL"]),
                                  _p(st["sd_ut"]), _p(st["sd_uv"]), _p(failed), _p(counts), _p(sino))
    assert rc == 0
    return failed, counts, sino


def hull_counts(cfg, kind, h):
    lib = load()
    g = geometry(cfg)
    img = np.empty(g.num_voxels, np.int32)
    lib.ora_initialize_hull(_cfgp(cfg), _p(img))
    stats = np.zeros(2, np.int64)
    n = len(h["WEPL"])
    rc = lib.ora_hull_walk(_cfgp(cfg), kind, C.c_int64(n), _p(h["missed"]), _p(h["WEPL"]), _p(h["x_entry"]),
                           _p(h["y_entry"]), _p(h["z_entry"]), _p(h["x_exit"]), _p(h["y_exit"]), _p(h["z_exit"]),
                           _p(img), _p(stats))
    assert rc == 0
    return img, stats


def msc_edge(cfg, counts):
    out = np.empty_like(counts)
    load().ora_msc_edge_detection(_cfgp(cfg), _p(counts), _p(out))
    return out


def sm_edge(cfg, counts):
    g = geometry(cfg)
    out = np.empty_like(counts)
    thr = np.empty(g.slices, np.int32)
    load().ora_sm_edge_detection(_cfgp(cfg), _p(counts), _p(out), _p(thr))
    return out, thr


def averaging_filter(cfg, hull, radius, threshold):
    out = np.empty_like(hull)
    load().ora_averaging_filter_bool(_cfgp(cfg), _p(hull), _p(out), radius, C.c_double(threshold))
    return out


def fbp(cfg, sino):
    g = geometry(cfg)
    filt = np.empty(g.num_bins, np.float32)
    img = np.empty(g.num_voxels, np.float32)
    hull = np.empty(g.num_voxels, np.uint8)
    lib = load()
    lib.ora_filter(_cfgp(cfg), _p(sino), _p(filt))
    lib.ora_backprojection(_cfgp(cfg), _p(filt), _p(img))
    lib.ora_fbp_hull(_cfgp(cfg), _p(img), _p(hull))
    return filt, img, hull


def endpoints(cfg, hull, h):
    n = len(h["x_entry"])
    out = {"intersected": np.empty(n, np.uint8), "first_voxel": np.empty(n, np.uint32)}
    for f in ("x_in", "y_in", "z_in", "x_out", "y_out", "z_out"):
        out[f] = np.empty(n, np.float32)
    order = ("x_entry", "y_entry", "z_entry", "xy_entry_angle", "xz_entry_angle",
             "x_exit", "y_exit", "z_exit", "xy_exit_angle", "xz_exit_angle")
    capped = load().ora_endpoints(_cfgp(cfg), C.c_int64(n), _p(hull), *[_p(h[f]) for f in order],
                                  _p(out["intersected"]), _p(out["first_voxel"]),
                                  *[_p(out[f]) for f in ("x_in", "y_in", "z_in", "x_out", "y_out", "z_out")])
    out["capped"] = capped
    return out


def mlp_rows(cfg, h, capacity=None, threads=None, tabulated=False):
    """h: recon vectors (x_entry.. are the hull entry/exit points). Returns (offsets, rows, chord).
    tabulated: the reference's lookup-table MLP (ora_mlp_rows_tab)."""
    n = len(h["x_entry"])
    g = geometry(cfg)
    if capacity is None:
        capacity = max(16, n * (2 * (g.columns + g.rows + g.slices) + 8))
    offsets = np.empty(n + 1, np.int64)
    rows = np.empty(capacity, np.uint32)
    chord = np.empty(n, np.float64)
    args = [_p(h[f]) for f in ("x_entry", "y_entry", "z_entry", "x_exit", "y_exit", "z_exit", "xy_entry_angle",
                               "xz_entry_angle", "xy_exit_angle", "xz_exit_angle")]
    if tabulated:
        k = load().ora_mlp_rows_tab(_cfgp(cfg), C.c_int64(n), *args, _p(h["first_voxel"]), _p(offsets), _p(rows),
                                    C.c_int64(capacity), _p(chord))
    elif threads:
        k = load().ora_mlp_rows_mt(_cfgp(cfg), C.c_int64(n), *args, _p(h["first_voxel"]), _p(offsets), _p(rows),
                                   C.c_int64(capacity), _p(chord), C.c_int(threads))
    else:
        k = load().ora_mlp_rows(_cfgp(cfg), C.c_int64(n), *args, _p(h["first_voxel"]), _p(offsets), _p(rows),
                                C.c_int64(capacity), _p(chord))
    if k < 0:
        raise RuntimeError("ora_mlp_rows: capacity too small")
    return offsets, rows[:k].copy(), chord


def drop(cfg, offsets, rows, chord, wepl, x0, iterations, block_size, lam, threads=None):
    x = np.ascontiguousarray(x0, dtype=np.float64).copy()
    w = np.ascontiguousarray(wepl, np.float32)
    if threads:
        rc = load().ora_drop_mt(_cfgp(cfg), C.c_int64(len(chord)), _p(offsets), _p(rows), _p(chord), _p(w),
                                iterations, block_size, C.c_double(lam), _p(x), threads)
    else:
        rc = load().ora_drop(_cfgp(cfg), C.c_int64(len(chord)), _p(offsets), _p(rows), _p(chord), _p(w), iterations,
                             block_size, C.c_double(lam), _p(x))
    assert rc == 0
    return x


def drop_shard(cfg, offsets, rows, chord, wepl, x0, iterations, block_size, num_blocks, lam, allreduce):
    """ora_drop on one shard of the rows; allreduce(user, data, count, dtype, on_device) -> 0 sums over ranks."""
    x = np.ascontiguousarray(x0, dtype=np.float64).copy()
    w = np.ascontiguousarray(wepl, np.float32)
    fn = ALLREDUCE_FN(allreduce)
    rc = load().ora_drop_shard(_cfgp(cfg), C.c_int64(len(chord)), _p(offsets), _p(rows), _p(chord), _p(w),
                               iterations, block_size, num_blocks, C.c_double(lam), _p(x), fn, None)
    assert rc == 0, rc
    return x


def drop_variant(cfg, offsets, rows, chord, wepl, x0, iterations, block_size, lam, variant, eta, psi_sign):
    """DROP_blocks_red (variant 1) or DROP_blocks_robust2 + DROP_update_robust2 (variant 2), binary64."""
    x = np.ascontiguousarray(x0, dtype=np.float64).copy()
    w = np.ascontiguousarray(wepl, np.float32)
    rc = load().ora_drop_variant(_cfgp(cfg), C.c_int64(len(chord)), _p(offsets), _p(rows), _p(chord), _p(w),
                                 iterations, block_size, C.c_double(lam), variant, C.c_double(eta), psi_sign, _p(x))
    assert rc == 0
    return x


def _select(h, mask):
    return {k: v[mask] for k, v in h.items() if isinstance(v, np.ndarray) and v.ndim == 1 and len(v) == len(mask)}


def run_pipeline(cfg, data13, proj_angle, iterations=None, block_size=None, lam=None,
                 keep_history=False):
    """The reference's main() sequence on the oracle.  Returns named stage outputs."""
    out = {}
    g = geometry(cfg)
    h = preprocess(cfg, data13, proj_angle)
    out["total_histories"] = np.array([data13.shape[1]], np.int32)
    kept = h["missed"] == 0
    hk = _select(h, kept)
    out["recon_vol_histories"] = np.array([kept.sum()], np.int32)
    for f in ["bin_num", "WEPL"] + HIST_FIELDS:
        out["binned." + f] = hk[f]
    # hull detection on every history of the chunk (.cu:100), finish (.cu:3892)
    if cfg.sc_on:
        sc, _ = hull_counts(cfg, 0, h)
        out["x_SC"] = sc.astype(np.uint8)
    if cfg.msc_on:
        msc, st = hull_counts(cfg, 1, h)
        out["MSC_counts_h"] = msc
        out["x_MSC"] = msc_edge(cfg, msc)
        out["msc_walk_stats"] = st
    if cfg.sm_on:
        sm, st = hull_counts(cfg, 2, h)
        out["SM_counts_h"] = sm
        out["x_SM"], out["sm_thresholds"] = sm_edge(cfg, sm)
        out["sm_walk_stats"] = st
    st = bin_statistics(cfg, hk)
    out["bin_counts_h_pre"] = st["counts"]
    out["mean_WEPL_h"], out["mean_rel_ut_angle_h"], out["mean_rel_uv_angle_h"] = st["mean_WEPL"], st["mean_ut"], st["mean_uv"]
    out["stddev_WEPL_h"], out["stddev_rel_ut_angle_h"], out["stddev_rel_uv_angle_h"] = st["sd_WEPL"], st["sd_ut"], st["sd_uv"]
    failed, counts_post, sino = statistical_cuts(cfg, hk, st)
    out["failed_cuts"] = failed
    passed = failed == 0
    hc = _select(hk, passed)
    out["post_cut_histories"] = np.array([passed.sum()], np.int32)
    for f in ["bin_num", "WEPL"] + HIST_FIELDS:
        out["cut." + f] = hc[f]
    out["bin_counts_post"] = counts_post
    out["sinogram"] = sino
    filt, fbp_img, fbp_hull = fbp(cfg, sino)
    out["sinogram_filtered"], out["FBP_image_h"], out["x_FBP"] = filt, fbp_img, fbp_hull
    sel = {0: out.get("x_SC"), 1: out.get("x_MSC"), 2: out.get("x_SM"), 3: fbp_hull}[cfg.mlp_hull]
    x_hull = (sel != 0).astype(np.uint8)
    out["x_hull"] = x_hull
    if cfg.avg_filter_hull:
        x_hull = averaging_filter(cfg, x_hull, cfg.hull_filter_radius, cfg.hull_filter_threshold)
        out["x_hull_filtered"] = x_hull
    x0 = {0: x_hull.astype(np.float32), 1: fbp_img, 2: fbp_img * x_hull.astype(np.float32),
          3: np.zeros(g.num_voxels, np.float32)}[cfg.x_k0]
    out["x_k0"] = x0
    ep = endpoints(cfg, x_hull, hc)
    keep = ep["intersected"] == 1
    hr = {f: hc[f][keep] for f in ["bin_num", "WEPL", "xy_entry_angle", "xz_entry_angle", "xy_exit_angle", "xz_exit_angle"]}
    for src, dst in (("x_in", "x_entry"), ("y_in", "y_entry"), ("z_in", "z_entry"), ("x_out", "x_exit"),
                     ("y_out", "y_exit"), ("z_out", "z_exit")):
        hr[dst] = ep[src][keep]
    hr["first_voxel"] = ep["first_voxel"][keep]
    out["endpoint_walks_capped"] = np.array([ep["capped"]], np.int32)
    out["reconstruction_histories"] = np.array([keep.sum()], np.int32)
    for f in ["bin_num", "WEPL"] + HIST_FIELDS:
        out["recon." + f] = hr[f]
    out["recon.first_MLP_voxel"] = hr["first_voxel"]
    iterations = cfg.iterations if iterations is None else iterations
    block_size = cfg.block_size if block_size is None else block_size
    lam = float(np.float32(cfg.lambda_)) if lam is None else lam
    if iterations > 0:
        offsets, rows, chord = mlp_rows(cfg, hr)
        out["mlp.offsets"], out["mlp.rows"], out["mlp.chord"] = offsets, rows, chord
        x = x0.astype(np.float64)
        for it in range(1, iterations + 1):
            x = drop(cfg, offsets, rows, chord, hr["WEPL"], x, 1, block_size, lam)
            out["x_%d" % it] = x.copy()
    if keep_history:
        out["_h"], out["_hk"], out["_hc"], out["_hr"] = h, hk, hc, hr
    return out
