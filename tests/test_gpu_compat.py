"""The reference-style driver over the compatibility layer, and the PCTD file
upload of the C ABI, reconstruct the same image as the stage API (needs a GPU
and g++).  The tiled DROP form makes the images comparable bit for bit."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from pct_gb300 import phantoms, pctd, recon

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "pct_gb300", "_lib")


@pytest.fixture(scope="module")
def scan(tmp_path_factory):
    w = phantoms.tiny(num_histories=40000, seed=7, v_extent=0.3)
    over = dict(w.config)
    over["drop_form"] = 2
    cfg = phantoms.make_config(over)
    data, angles = phantoms.generate(w)
    d = tmp_path_factory.mktemp("pctd")
    paths = pctd.write_scan(str(d), "scan", data, angles, w.num_angles, w.gantry_angle_interval)
    r = recon.run_full(cfg, data, angles)
    r.image_reconstruction_GPU()
    x = r.array("X")
    c = r.counts()
    r.close()
    return cfg, str(d), paths, x, c


def test_pctd_upload_matches_stage_api(scan):
    cfg, d, paths, x_ref, c_ref = scan
    r = recon.Reconstruction(cfg)
    r.process_pctd_files(paths)
    r.hull_detection_finish()
    r.statistical_cuts()
    r.FBP()
    r.hull_selection()
    r.define_initial_iterate()
    r.image_reconstruction_GPU()
    x = r.array("X")
    c = r.counts()
    r.close()
    assert c["reconstruction_histories"] == c_ref["reconstruction_histories"]
    assert x.tobytes() == x_ref.tobytes()


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_reference_driver_over_compat_layer(scan, tmp_path):
    cfg, d, paths, x_ref, c_ref = scan
    exe = str(tmp_path / "driver")
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "compat", "driver_main.cpp"), "-L", LIBDIR, "-lpct_compat", "-lpct_gb300",
           "-Wl,-rpath," + LIBDIR, "-o", exe]
    subprocess.run(cmd, check=True)
    cfg_bin = tmp_path / "config.bin"
    cfg_bin.write_bytes(bytes(cfg))
    out = tmp_path / "image.bin"
    res = subprocess.run([exe, str(cfg_bin), d, "scan", "15000", str(out)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr + res.stdout
    x = np.fromfile(str(out), dtype=np.float32)
    assert x.tobytes() == x_ref.tobytes()
    assert ("reconstruction %d" % c_ref["reconstruction_histories"]) in res.stdout
