#!/usr/bin/env python3
"""Generates the golden fixtures in tests/golden/ from the reference itself.

For each scenario below: seeded synthetic histories (pct_gb300.phantoms) are
written as PCTD v0 files, the reference's own driver sequence runs on them
(oracle/refharness.py: the unmodified reference source compiled for the host
by oracle/build_ref.py, main()'s call order), and every stage output is
stored.  MLP voxel rows come from the reference's find_MLP_path_GPU
(src/pCT_Reconstruction_Data_Segments.cu:5279) run on the recon histories.

Scenarios with `pins` also store (names "pin.*") the outputs of reference
functions that the driver sequence does not call:
  pin.MLP_endpoints_file  the file write_MLP_endpoints (.cu:4684-4714) writes
                          for the histories image_reconstruction_GPU kept;
  pin.tab.*               rows of find_MLP_path_GPU_tabulated (.cu:5502-5660)
                          on the tables of generate_trig_tables,
                          generate_scattering_coefficient_table and
                          generate_polynomial_tables (.cu:4786-4911);
  pin.drop.v0/v1/v2       the CPU reconstruction's block loop (.cu:7525-7560)
                          with DROP_blocks / DROP_update (.cu:8023-8055),
                          DROP_blocks_red (.cu:7998-8021) and
                          DROP_blocks_robust2 / DROP_update_robust2
                          (.cu:7871-7901), from x_0 on the reference's own MLP
                          rows and chords of the first `rows` histories.

Needs the reference checkout (default /root/reference), so it runs in the
development container only; the fixtures are committed.  Large arrays are
stored as SHA-256 digests plus a leading sample, small ones in full.

    python tests/golden/make_golden.py [--ref /root/reference] [scenario ...]
"""
import argparse
import ctypes as C
import hashlib
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from pct_gb300 import pctd, phantoms  # noqa: E402
from oracle import refharness  # noqa: E402

FULL_LIMIT = 20000      # arrays up to this many elements are stored in full
SAMPLE = 512            # leading elements kept for larger arrays


def scenarios():
    return {
        # z-clip branches of the intersection code and MLP rows that leave the slab
        "tiny_clip": dict(geometry="tiny", workload=phantoms.tiny(num_histories=40000, seed=11, v_extent=0.55),
                          run=dict(msc_on=1, mlp_hull=1, iterations=0), mlp_rows=4000),
        # in-slab scan through DROP (2 iterations, block 6000, lambda 0.1)
        "tiny_drop": dict(geometry="tiny", workload=phantoms.tiny(num_histories=40000, seed=7, v_extent=0.3),
                          run=dict(msc_on=1, mlp_hull=1, iterations=2, block_size=6000, lambda_=0.1), mlp_rows=4000),
        # 200x200x8 water-cylinder geometry with the SM hull
        "cfg1_sm": dict(geometry="cfg1", workload=phantoms.cfg1(num_histories=120000, seed=5),
                        run=dict(msc_on=0, sm_on=1, mlp_hull=2, iterations=0), mlp_rows=1500),
        # the benchmark scan's geometry and phantom (256x256x32, 180 angles), through the MLP rows
        "cfg2_grid": dict(geometry="cfg2", workload=phantoms.cfg2(num_histories=200000, seed=9),
                          run=dict(msc_on=0, sm_on=1, mlp_hull=2, iterations=0), mlp_rows=1500),
        # config 4's head phantom and grid (320x320x64, 0.8 mm voxels, 180 angles), through the MLP rows
        "cfg4_grid": dict(geometry="cfg4", workload=phantoms.cfg4(num_histories=200000, seed=9),
                          run=dict(msc_on=0, sm_on=1, mlp_hull=2, iterations=0), mlp_rows=1500),
        # ellipsoid phantom of the batched-scan family on its smallest grid, 180 angles, through DROP
        "cfg3_128x8": dict(geometry="cfg3_128x8",
                           workload=phantoms.ellipsoids(31, num_histories=150000, cols=128, slices=8),
                           run=dict(msc_on=0, sm_on=1, mlp_hull=2, iterations=2, block_size=50000, lambda_=0.1),
                           mlp_rows=1500),
        # the same family on its largest grid (256x256x48), through the MLP rows
        "cfg3_256x48": dict(geometry="cfg3_256x48",
                            workload=phantoms.ellipsoids(32, num_histories=300000, cols=256, slices=48),
                            run=dict(msc_on=0, sm_on=1, mlp_hull=2, iterations=0), mlp_rows=1500),
        # a small in-slab scan whose reference-written endpoint file is stored in full,
        # with the tabulated MLP and the DROP variants of the CPU reconstruction
        "tiny_pins": dict(geometry="tiny", workload=phantoms.tiny(num_histories=16000, seed=13, v_extent=0.3),
                          run=dict(msc_on=1, mlp_hull=1, iterations=1, block_size=2000, lambda_=0.1), mlp_rows=4000,
                          pins=dict(rows=4000, block_size=500, iterations=3), full_limit=4096),
    }


def digest(a):
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.tobytes()).hexdigest()


def pack(name, arr, out, full_limit=FULL_LIMIT, pins=False):
    out["dtype:" + name] = np.array(str(arr.dtype))
    out["shape:" + name] = np.array(arr.shape, dtype=np.int64)
    out["sha:" + name] = np.array(digest(arr))
    # DROP iterates x_1, x_2, ... in full whatever their size: they are compared
    # within a tolerance, not by digest; so are the pinned DROP loops, and (in a
    # scenario with pins) x_0 and the endpoint file, inputs of the pin tests
    if (arr.size <= full_limit or (name.startswith("x_") and name[2:].isdigit() and int(name[2:]) > 0)
            or (pins and name == "x_0") or (name.startswith("pin.") and name != "pin.tab.rows")):
        out["full:" + name] = arr
    else:
        out["head:" + name] = arr.ravel()[:SAMPLE]


def mlp_rows_reference(geometry, res, limit):
    lib = refharness.load(geometry)
    n = min(limit, len(res["recon.x_entry"]))
    x = np.zeros(1 << 22, np.float32)
    path = np.zeros(1 << 14, np.uint32)
    rows, offsets, chord = [], [0], []
    for i in range(n):
        inp = np.array([res["recon." + f][i] for f in ("x_entry", "y_entry", "z_entry", "x_exit", "y_exit", "z_exit",
                                                      "xy_entry_angle", "xz_entry_angle", "xy_exit_angle",
                                                      "xz_exit_angle", "WEPL")], np.float32)
        ch, ad, aa = C.c_double(), C.c_double(), C.c_double()
        k = lib.pctref_mlp_path_gpu(x.ctypes.data, inp.ctypes.data, int(res["recon.first_MLP_voxel"][i]),
                                    path.ctypes.data, C.byref(ch), C.byref(ad), C.byref(aa))
        rows.append(path[:k].copy())
        offsets.append(offsets[-1] + k)
        chord.append(ch.value)
    return np.concatenate(rows), np.array(offsets, np.int64), np.array(chord, np.float64)


def variant_eta(variant, offsets, chord, x0):
    """eta for a DROP variant: |psi| = |1 - x| eta stays below 5% of the smallest
    denominator (||a||^2 for DROP_blocks_red, c^2 for DROP_blocks_robust2), so that
    the update is far from the singularity ||a||^2 + psi = 0 that the reference's
    default eta = 2.5 reaches on these rows."""
    span = max(1e-3, float(np.abs(1.0 - x0.astype(np.float64)).max()))
    if variant == 1:
        return min(0.05, 0.05 * float((chord * chord * np.diff(offsets)).min()) / span)
    return min(0.005, 0.05 * float((chord * chord).min()) / span)


def pins_reference(geometry, res, pins, lam):
    lib = refharness.load(geometry)
    n = pins["rows"]
    fields = ("x_entry", "y_entry", "z_entry", "x_exit", "y_exit", "z_exit", "xy_entry_angle", "xz_entry_angle",
              "xy_exit_angle", "xz_exit_angle", "WEPL")
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        if lib.pctref_mlp_tables(tmp.encode()) != 0:
            raise SystemExit("reference table generation failed")
    x = np.zeros(1 << 22, np.float32)
    path = np.zeros(1 << 14, np.uint32)
    rows, offsets = [], [0]
    upd = C.c_float()
    for i in range(n):
        inp = np.array([res["recon." + f][i] for f in fields], np.float32)
        k = lib.pctref_mlp_path_tab(x.ctypes.data, inp.ctypes.data, int(res["recon.first_MLP_voxel"][i]),
                                    path.ctypes.data, C.byref(upd))
        rows.append(path[:k].copy())
        offsets.append(offsets[-1] + k)
    out["pin.tab.rows"] = np.concatenate(rows)
    out["pin.tab.offsets"] = np.array(offsets, np.int64)
    offs = res["mlp.offsets"][: n + 1].astype(np.int64)
    r = res["mlp.rows"][: offs[-1]].astype(np.uint32)
    chord = res["mlp.chord"][:n].astype(np.float64)
    wepl = res["recon.WEPL"][:n].astype(np.float32)
    x0 = res["x_0"].astype(np.float32)
    if int(r.max()) >= x0.size or n % pins["block_size"]:
        raise SystemExit("pin rows must lie in the image and fill whole blocks")
    etas = []
    for v in (0, 1, 2):
        eta = 2.5 if v == 0 else variant_eta(v, offs, chord, x0)
        xv = x0.copy()
        rc = lib.pctref_drop_cpu(v, n, offs.ctypes.data, r.ctypes.data, chord.ctypes.data, wepl.ctypes.data,
                                 pins["iterations"], pins["block_size"], float(np.float32(lam)), eta, 1, xv.ctypes.data)
        if rc != 0:
            raise SystemExit("reference DROP loop returned %d" % rc)
        out["pin.drop.v%d" % v] = xv
        etas.append(eta)
    out["pin.drop.eta"] = np.array(etas, np.float64)
    out["pin.drop.setup"] = np.array([n, pins["block_size"], pins["iterations"]], np.int64)
    return out


def make(name, sc, ref_root):
    refharness.ensure_built(sc["geometry"], ref_root)
    w = sc["workload"]
    data, angles = phantoms.generate(w)
    with tempfile.TemporaryDirectory() as tmp:
        pctd.write_scan(tmp, "scan", data, angles, w.num_angles, w.gantry_angle_interval)
        res = refharness.run_pipeline(sc["geometry"], os.path.join(tmp, "ref.npz"), input_directory=tmp + "/",
                                      input_folder="scan", endpoints_file=bool(sc.get("pins")), **sc["run"])
    if int(res["__rc"][0]) != 0:
        raise SystemExit("%s: reference run returned %d" % (name, int(res["__rc"][0])))
    rows, offsets, chord = mlp_rows_reference(sc["geometry"], res, sc["mlp_rows"])
    res["mlp.rows"], res["mlp.offsets"], res["mlp.chord"] = rows, offsets, chord
    if sc.get("pins"):
        if "pin.MLP_endpoints_file" not in res:
            raise SystemExit("%s: the reference wrote no endpoint file" % name)
        res.update(pins_reference(sc["geometry"], res, sc["pins"], sc["run"].get("lambda_", 0.001)))
    out = {"scenario": np.array(name), "workload": np.array(w.name), "seed": np.array(w.seed),
           "num_histories": np.array(w.num_histories), "v_extent": np.array(w.v_extent),
           "input_sha": np.array(digest(data) + digest(angles)),
           "grid_cols": np.array(int(w.config["columns"])),
           "grid_slices": np.array(int(round((w.config["ssd_v_size"] - 1.0) / 0.25))),
           "run_config": np.array(repr(sc["run"]))}
    for k, v in res.items():
        if k.startswith("__"):
            continue
        pack(k, v, out, sc.get("full_limit", FULL_LIMIT), pins=bool(sc.get("pins")))
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print("%s: %d arrays, %d bytes" % (path, len(res), os.path.getsize(path)))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("names", nargs="*")
    a = ap.parse_args()
    sc = scenarios()
    for name in (a.names or sorted(sc)):
        make(name, sc[name], a.ref)


if __name__ == "__main__":
    main()
