"""PCTD version-0 files through the C ABI on the host (no GPU): the library's
reader and writer (pct_pctd_info / pct_pctd_read / pct_pctd_write, the layout
of count_histories_v0 and read_data_chunk_v02,
src/pCT_Reconstruction_Data_Segments.cu:997-1097, 1769-1933) against the
Python reader and writer, and the reader's rejection of malformed files."""
import ctypes as C
import struct

import numpy as np
import pytest

from pct_gb300 import _capi, pctd


@pytest.fixture(scope="module")
def lib():
    lib = _capi.load()
    lib.pct_pctd_info.argtypes = [C.c_char_p, C.POINTER(C.c_int64), C.POINTER(C.c_float), C.POINTER(C.c_float)]
    lib.pct_pctd_read.argtypes = [C.c_char_p, C.POINTER(C.c_void_p), C.c_int64, C.POINTER(C.c_int64),
                                  C.POINTER(C.c_float)]
    lib.pct_pctd_write.argtypes = [C.c_char_p, C.POINTER(C.c_void_p), C.c_int64, C.c_float, C.c_float]
    return lib


def histories(n, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((13, n)).astype(np.float32) * 100.0
    a[12] = np.abs(a[12])
    return a


def c_write(lib, path, a, angle, energy):
    a = np.ascontiguousarray(a, dtype=np.float32)
    ptrs = (C.c_void_p * 13)(*[a[k].ctypes.data for k in range(13)])
    return lib.pct_pctd_write(path.encode(), ptrs, a.shape[1], angle, energy)


def c_read(lib, path, capacity):
    out = np.zeros((13, max(capacity, 1)), np.float32)
    ptrs = (C.c_void_p * 13)(*[out[k].ctypes.data for k in range(13)])
    n, angle = C.c_int64(-1), C.c_float(0)
    st = lib.pct_pctd_read(path.encode(), ptrs, capacity, C.byref(n), C.byref(angle))
    return st, out[:, :max(n.value, 0)], angle.value


def c_info(lib, path):
    n, angle, energy = C.c_int64(-1), C.c_float(0), C.c_float(0)
    st = lib.pct_pctd_info(path.encode(), C.byref(n), C.byref(angle), C.byref(energy))
    return st, n.value, angle.value, energy.value


@pytest.mark.parametrize("n", [0, 1, 4097])
def test_c_writer_python_reader(lib, tmp_path, n):
    a = histories(n, 1 + n)
    path = str(tmp_path / "c.bin")
    assert c_write(lib, path, a, 92.0, 200.0) == 0
    b, angle, energy = pctd.read_file(path)
    assert b.tobytes() == a.tobytes()
    assert (angle, energy) == (92.0, 200.0)


@pytest.mark.parametrize("n", [0, 3, 5000])
def test_python_writer_c_reader(lib, tmp_path, n):
    a = histories(n, 7 + n)
    path = str(tmp_path / "py.bin")
    pctd.write_file(path, a, 270.0, beam_energy=230.0, phantom_name=b"cylinder", data_source=b"",
                    prepared_by=b"x" * 300)
    assert c_info(lib, path) == (0, n, 270.0, 230.0)
    st, b, angle = c_read(lib, path, n)
    assert st == 0 and angle == 270.0
    assert b.tobytes() == a.tobytes()


def test_capacity_too_small(lib, tmp_path):
    a = histories(10, 3)
    path = str(tmp_path / "cap.bin")
    assert c_write(lib, path, a, 0.0, 200.0) == 0
    st, _, _ = c_read(lib, path, 9)
    assert st == _capi.PCT_ERR_OVERFLOW


def _good_bytes(n=5):
    a = histories(n, 11)
    head = b"PCTD" + struct.pack("<ii", 0, n) + struct.pack("<ff", 10.0, 200.0) + struct.pack("<ii", 0, 0)
    for s in (b"p", b"", b"me"):
        head += struct.pack("<i", len(s)) + s
    return head, a.tobytes()


@pytest.mark.parametrize("case", ["magic", "version", "negative_count", "bad_string", "truncated_header",
                                  "truncated_data", "missing"])
def test_malformed_files_are_rejected(lib, tmp_path, case):
    head, body = _good_bytes()
    path = str(tmp_path / ("bad_%s.bin" % case))
    if case == "magic":
        data = b"PCTX" + head[4:] + body
    elif case == "version":
        data = head[:4] + struct.pack("<i", 1) + head[8:] + body
    elif case == "negative_count":
        data = head[:8] + struct.pack("<i", -5) + head[12:] + body
    elif case == "bad_string":
        data = head[:28] + struct.pack("<i", 1 << 30) + head[32:] + body
    elif case == "truncated_header":
        data = head[:30]
    elif case == "truncated_data":
        data = head + body[:-4]
    else:
        data = None
    if data is not None:
        with open(path, "wb") as f:
            f.write(data)
    st, _, _, _ = c_info(lib, path)
    assert st == _capi.PCT_ERR_IO, case
    st, _, _ = c_read(lib, path, 100)
    assert st == _capi.PCT_ERR_IO, case
    if data is not None:
        with pytest.raises(ValueError):
            pctd.read_file(path)


def test_scan_layout_round_trip(lib, tmp_path):
    """write_scan's per-angle files, read back through the C reader: the header
    angle maps to the gantry angle as (int(angle) + 270) % 360 (.cu:1921)."""
    n_angles, interval = 6, 60.0
    data = histories(600, 5)
    gantry_of = np.repeat(np.arange(n_angles) * int(interval), 100)
    proj = ((gantry_of + 90) % 360).astype(np.float32)  # the header angle of each history
    pctd.write_scan(str(tmp_path), "scan", data, proj, n_angles, interval)
    seen = 0
    for k in range(n_angles):
        gantry = int(k * interval)
        path = pctd.file_name(str(tmp_path), "scan", gantry)
        st, n, angle, _ = c_info(lib, path)
        assert st == 0
        assert (int(angle) + 270) % 360 == gantry
        st, b, _ = c_read(lib, path, n)
        assert st == 0
        sel = gantry_of == gantry
        assert b.tobytes() == np.ascontiguousarray(data[:, sel]).tobytes()
        seen += n
    assert seen == data.shape[1]
