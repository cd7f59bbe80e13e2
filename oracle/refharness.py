"""ctypes driver for the reference harness in oracle/_ref (test infrastructure only).

Runs the unmodified reference driver sequence (see oracle/ref/ref_harness.inc)
in a child process, so that the reference's global state starts clean on
every run and a reference fault cannot take the test process with it.  The
child writes every captured array to an .npz file.

Only tests/golden/make_golden.py uses this, in the container that has the
reference checkout; the GPU tests read the committed fixtures instead.
"""
import ctypes as C
import multiprocessing as mp
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
DTYPES = {0: np.float32, 1: np.int32, 2: np.uint8, 3: np.uint32}


class RefRun(C.Structure):
    _fields_ = [("input_directory", C.c_char_p), ("input_folder", C.c_char_p),
                ("sc_on", C.c_int), ("msc_on", C.c_int), ("sm_on", C.c_int), ("avg_filter_hull", C.c_int),
                ("mlp_hull", C.c_int), ("x_k0", C.c_int), ("fbp_filter", C.c_int),
                ("iterations", C.c_int), ("block_size", C.c_int), ("lambda_", C.c_float),
                ("stop_after", C.c_int)]


def lib_path(geometry):
    return os.path.join(REF_DIR, "libpctref_%s.so" % geometry)


def ensure_built(geometry, ref_root="/root/reference"):
    p = lib_path(geometry)
    if not os.path.exists(p):
        subprocess.run([sys.executable, os.path.join(HERE, "build_ref.py"), "--ref", ref_root, geometry], check=True)
    return p


def load(geometry):
    lib = C.CDLL(lib_path(geometry))
    lib.pctref_run.argtypes = [C.POINTER(RefRun)]
    lib.pctref_capture_name.restype = C.c_char_p
    lib.pctref_capture_bytes.restype = C.c_long
    lib.pctref_capture_copy.argtypes = [C.c_int, C.c_void_p]
    lib.pctref_geometry.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_double)]
    lib.pctref_mlp_path_gpu.argtypes = [C.c_void_p, C.c_void_p, C.c_uint, C.c_void_p,
                                        C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.pctref_mlp_path_host.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
    lib.pctref_endpoints.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    lib.pctref_chord_host.restype = C.c_double
    lib.pctref_chord_host.argtypes = [C.c_double, C.c_double]
    lib.pctref_chord_gpu.restype = C.c_double
    lib.pctref_chord_gpu.argtypes = [C.c_double, C.c_double]
    lib.pctref_write_endpoints.argtypes = [C.c_char_p, C.c_char_p]
    lib.pctref_mlp_tables.argtypes = [C.c_char_p]
    lib.pctref_mlp_path_tab.argtypes = [C.c_void_p, C.c_void_p, C.c_uint, C.c_void_p, C.POINTER(C.c_float)]
    lib.pctref_drop_cpu.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                    C.c_int, C.c_float, C.c_double, C.c_int, C.c_void_p]
    return lib


def geometry_of(geometry):
    lib = load(geometry)
    gi = (C.c_int * 16)()
    gd = (C.c_double * 32)()
    lib.pctref_geometry(gi, gd)
    return list(gi[:10]), list(gd[:21])


def _child(geometry, kw, out_path):
    lib = load(geometry)
    run = RefRun(input_directory=kw["input_directory"].encode(), input_folder=kw["input_folder"].encode(),
                 sc_on=kw.get("sc_on", 0), msc_on=kw.get("msc_on", 1), sm_on=kw.get("sm_on", 0),
                 avg_filter_hull=kw.get("avg_filter_hull", 1), mlp_hull=kw.get("mlp_hull", 1),
                 x_k0=kw.get("x_k0", 2), fbp_filter=kw.get("fbp_filter", 1), iterations=kw.get("iterations", 1),
                 block_size=kw.get("block_size", 3200), lambda_=kw.get("lambda_", 0.001),
                 stop_after=kw.get("stop_after", 0))
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)
    rc = lib.pctref_run(C.byref(run))
    arrays = {}
    if rc == 0 and kw.get("endpoints_file"):
        # write_MLP_endpoints on the histories the run kept
        d = os.path.dirname(out_path)
        os.makedirs(os.path.join(d, "endpoints"), exist_ok=True)
        if lib.pctref_write_endpoints((d + "/").encode(), b"endpoints") == 0:
            with open(os.path.join(d, "endpoints", "MLP_endpoints_r=1.bin"), "rb") as f:
                arrays["pin.MLP_endpoints_file"] = np.frombuffer(f.read(), np.uint8).copy()
    for i in range(lib.pctref_capture_count()):
        name = lib.pctref_capture_name(i).decode()
        nbytes = lib.pctref_capture_bytes(i)
        dt = DTYPES[lib.pctref_capture_type(i)]
        a = np.empty(nbytes // np.dtype(dt).itemsize, dtype=dt)
        if nbytes:
            lib.pctref_capture_copy(i, a.ctypes.data)
        key = name
        k = 1
        while key in arrays:
            k += 1
            key = "%s#%d" % (name, k)
        arrays[key] = a
    arrays["__rc"] = np.array([rc], dtype=np.int32)
    np.savez(out_path, **arrays)


def run_pipeline(geometry, out_path, timeout=3600, **kw):
    """Runs the reference pipeline in a spawned child; returns the captured arrays."""
    ctx = mp.get_context("spawn")
    p = ctx.Process(target=_child, args=(geometry, kw, out_path))
    p.start()
    p.join(timeout)
    if p.is_alive():
        p.kill()
        p.join()
        raise RuntimeError("reference pipeline timed out after %ss" % timeout)
    if p.exitcode != 0:
        raise RuntimeError("reference pipeline child exited with %s" % p.exitcode)
    with np.load(out_path) as z:
        return {k: z[k] for k in z.files}
