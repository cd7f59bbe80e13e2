"""pct_drop_noalloc (static device scratch, no allocation) against pct_drop.

Collected last so that it also runs after every other GPU test has used the
device; it builds its own context and runs on its own in a fresh process too.
Two calls in a row on the same rows must each reproduce pct_drop's image and
sweep residuals within the DROP tolerance (binary32 scatter-add order differs
between runs), and the device's free memory must be the same before and after
a call (after pct_noalloc_setup and a first call).
"""
import ctypes as C

import numpy as np
import pytest

from pct_gb300 import _capi, phantoms, recon

pytestmark = pytest.mark.gpu

TOL = 1e-4
ITERATIONS = 3
MAX_VOXELS = 1 << 21   # PCT_NOALLOC_MAX_VOXELS in include/pct.h


def _lib():
    lib = _capi.load()
    lib.pct_noalloc_setup.restype = C.c_int
    lib.pct_noalloc_setup.argtypes = []
    lib.pct_drop_noalloc.restype = C.c_int
    lib.pct_drop_noalloc.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                     C.c_float, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    return lib


@pytest.fixture(scope="module")
def ctx():
    w = phantoms.tiny(num_histories=40000, seed=7, v_extent=0.3)
    cfg = phantoms.make_config(w.config)
    data, angles = phantoms.generate(w)
    r = recon.run_full(cfg, data, angles)
    r.collect_mlp_endpoints()
    r.mlp_rows()
    yield cfg, r
    r.close()


def test_noalloc_matches_pct_drop_on_two_calls(ctx):
    import torch
    cfg, r = ctx
    lib = _lib()
    r.reset_iterate()
    st = r.drop(ITERATIONS)
    x_ref = r.array("X").astype(np.float64)
    b2 = float(np.sum(r.array("H_WEPL").astype(np.float64) ** 2))
    n = r.counts()["reconstruction_histories"]
    assert n > 0
    ptr = {k: r.device_ptr(k)[0] for k in ("ROW_OFFSETS", "ROWS", "CHORD", "H_WEPL", "X")}
    nv = phantoms.geometry(cfg).num_voxels
    resid = torch.zeros(ITERATIONS, dtype=torch.float64, device="cuda")
    _capi.check(lib.pct_noalloc_setup(), "pct_noalloc_setup")
    torch.cuda.synchronize()
    for call in range(2):
        r.reset_iterate()
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        s = lib.pct_drop_noalloc(n, ptr["ROW_OFFSETS"], ptr["ROWS"], ptr["CHORD"], ptr["H_WEPL"], nv,
                                 cfg.block_size, cfg.lambda_, ITERATIONS, ptr["X"], resid.data_ptr(), r.stream())
        _capi.check(s, "pct_drop_noalloc")
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        if call == 1:  # the first call may still load the module
            assert free_after == free_before, "device free memory %d -> %d" % (free_before, free_after)
        x = r.array("X").astype(np.float64)
        err = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
        assert err <= TOL, "call %d: relative L2 %.3e" % (call, err)
        rel = np.sqrt(resid.cpu().numpy() / b2)
        ref = np.array(st.residual[:ITERATIONS])
        assert np.all(np.abs(rel - ref) <= TOL * ref), "call %d: residuals %s vs %s" % (call, rel, ref)


def test_noalloc_rejects_images_beyond_scratch():
    lib = _lib()
    s = lib.pct_drop_noalloc(0, None, None, None, None, MAX_VOXELS + 1, 3200, 0.001, 1, None, None, None)
    assert s == 1
    assert b"static scratch" in lib.pct_last_error()
