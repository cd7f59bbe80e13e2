"""Configuration defaults and derived sizes on the host (no GPU).

pct_config_default must give the reference's compile-time values
(include/pCT_data.h, include/pCT_config.h), and pct_geometry_from_config must
derive the sizes the reference's macros give for each configuration the
reconstruction path is measured on: NUM_BINS = ANGULAR_BINS x T_BINS x V_BINS
and NUM_VOXELS = COLUMNS x ROWS x SLICES with SLICES from SSD_V_SIZE - 1
(pCT_data.h:227-271)."""
import ctypes as C

import pytest

from pct_gb300 import _capi, phantoms


def default_config():
    lib = _capi.load()
    cfg = _capi.Config()
    assert lib.pct_config_default(C.byref(cfg)) == 0
    return cfg


def test_defaults_are_the_reference_header_values():
    c = default_config()
    expect = {
        "source_radius": 260.7,            # SOURCE_RADIUS, pCT_data.h:222
        "gantry_angle_interval": 4.0,      # GANTRY_ANGLE_INTERVAL, :223
        "ssd_t_size": 35.0,                # SSD_T_SIZE, :227
        "ssd_v_size": 9.0,                 # SSD_V_SIZE, :228
        "t_bin_size": 0.1,                 # T_BIN_SIZE, :237
        "v_bin_size": 0.25,                # V_BIN_SIZE, :239
        "angular_bin_size": 4.0,           # ANGULAR_BIN_SIZE, :241
        "sigmas_to_keep": 3,               # SIGMAS_TO_KEEP, :244
        "fbp_threshold": 0.6,              # FBP_THRESHOLD, :248
        "recon_cyl_radius": 10.0,          # RECON_CYL_RADIUS, :255
        "columns": 200, "rows": 200,       # COLUMNS, ROWS, :264-265
        "slice_thickness": 0.25,           # SLICE_THICKNESS, :271
        "msc_diff_thresh": 50,             # MSC_DIFF_THRESH, :281
        "sc_threshold": 0.0,               # SC_THRESHOLD, :282
        "msc_threshold": 0.0,              # MSC_THRESHOLD, :283
        "sm_lower_threshold": 6.0,         # SM_LOWER_THRESHOLD, :284
        "sm_scale_threshold": 1.0,         # SM_SCALE_THRESHOLD, :286
        "hull_filter_threshold": 0.1,      # HULL_FILTER_THRESHOLD, :287
        "hull_filter_radius": 1,           # HULL_FILTER_RADIUS, :288
        "mlp_hull": 1,                     # MLP_HULL = MSC_HULL, :293
        "iterations": 12,                  # ITERATIONS, pCT_config.h:5
        "block_size": 3200,                # BLOCK_SIZE_RECON, pCT_data.h:377
        "eta": 2.5, "psi_sign": 1,         # ETA, PSI_SIGN, :369-371
    }
    for k, v in expect.items():
        assert getattr(c, k) == pytest.approx(v, rel=0, abs=0), k
    # LAMBDA is a float global (pCT_data.h:374): 0.001 rounded to binary32
    assert c.lambda_ == pytest.approx(float(C.c_float(0.001).value), rel=0, abs=0)


@pytest.mark.parametrize("name, make, bins, voxels, grid", [
    ("cfg1", lambda: phantoms.cfg1(1000), 90 * 350 * 12, 320_000, (200, 200, 8)),
    ("cfg2", lambda: phantoms.cfg2(1000), 180 * 350 * 36, 2_097_152, (256, 256, 32)),
    ("cfg3 128x128x8", lambda: phantoms.ellipsoids(31, 1000, cols=128, slices=8), 180 * 350 * 12, 131_072,
     (128, 128, 8)),
    ("cfg3 256x256x48", lambda: phantoms.ellipsoids(32, 1000, cols=256, slices=48), 180 * 350 * 52, 3_145_728,
     (256, 256, 48)),
    ("cfg4", lambda: phantoms.cfg4(1000), 180 * 350 * 68, 6_553_600, (320, 320, 64)),
])
def test_derived_sizes_of_the_measured_configurations(name, make, bins, voxels, grid):
    w = make()
    g = phantoms.geometry(phantoms.make_config(w.config))
    assert (g.columns, g.rows, g.slices) == grid, name
    assert g.num_voxels == voxels, name
    assert g.num_bins == bins, name
    assert g.t_bins == 350, name
    assert g.voxel_width == pytest.approx(2 * g.recon_cyl_radius / g.columns, rel=0, abs=0)
    assert g.mlp_u_step == g.voxel_width / 2                 # MLP_U_STEP, pCT_data.h:300
    assert g.x_zero == -g.recon_cyl_radius and g.y_zero == g.recon_cyl_radius
    assert g.z_zero == g.recon_cyl_height / 2


@pytest.mark.parametrize("field, value", [("columns", 0), ("rows", -4), ("recon_cyl_radius", 0.0),
                                          ("slice_thickness", 0.0), ("t_bin_size", 0.0),
                                          ("v_bin_size", -1.0), ("angular_bin_size", 0.0),
                                          ("gantry_angle_interval", 0.0), ("ssd_v_size", 1.0)])
def test_invalid_geometry_is_rejected(field, value):
    lib = _capi.load()
    c = default_config()
    setattr(c, field, value)
    g = _capi.Geometry()
    assert lib.pct_geometry_from_config(C.byref(c), C.byref(g)) != 0, field
