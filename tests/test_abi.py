"""The C ABI library and the compatibility layer load and export every
function their headers declare (CPU only, no compute calls)."""
import ctypes as C
import os
import re
import shutil
import subprocess

import pytest

from pct_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"\btypedef\b[^;]*;", "", text)  # function-pointer types are not exports
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z_0-9]*\s*\**\s+\**([A-Za-z_][A-Za-z_0-9]*)\s*\(",
                       text, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "return", "sizeof")))


def test_c_abi_exports_every_declared_function():
    lib = _capi.load()
    names = declared_functions("pct.h")
    assert len(names) >= 30, names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_probe_header_is_exported():
    lib = _capi.load()
    names = declared_functions("pct_probe.h")
    assert names == ["pct_probe_l2"]
    assert all(hasattr(lib, n) for n in names)


def test_struct_layouts_match_the_library():
    from pct_gb300 import recon
    lib = _capi.load()
    for which, cls in _capi._STRUCTS + [(4, recon.Counts), (5, recon.DropStats)]:
        assert lib.pct_sizeof(which) == C.sizeof(cls), cls.__name__


@pytest.mark.skipif(shutil.which("nm") is None, reason="nm not available")
def test_compat_layer_exports_the_reference_entry_points():
    lib = os.path.join(ROOT, "pct_gb300", "_lib", "libpct_compat.so")
    assert os.path.exists(lib)
    out = subprocess.run(["nm", "-DC", "--defined-only", lib], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T ([A-Za-z_][A-Za-z_0-9]*)\(", out))
    names = declared_functions("pct_functions_compat.h")
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for ref_name in ("read_data_chunk", "hull_detection", "calculate_means", "FBP", "image_reconstruction_GPU"):
        assert ref_name in exported


def test_cnn_header_is_exported():
    lib = _capi.load()
    names = declared_functions("pct_cnn.h")
    assert "pct_cnn_train_step" in names and "pct_cnn_warm_start" in names, names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    lib.pct_cnn_num_params.restype = C.c_size_t
    assert lib.pct_cnn_num_params() == 27 * (2 * 32 + 6 * 32 * 32 + 32) + 7 * 32 + 1
