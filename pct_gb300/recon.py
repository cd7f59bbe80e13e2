"""Host-side mirror of the reference's reconstruction sequence.

`Reconstruction` drives one pct_ctx through the stages in the order of the
reference's main() (src/pCT_Reconstruction_Data_Segments.cu:42-226).  Method
names follow include/pCT_functions.h so a reference driver reads the same:

    r = Reconstruction(config)
    for chunk in chunks:  r.process_chunk(data13, projection_angle)
        # read_data_chunk + recon_volume_intersections + binning + hull_detection
    r.hull_detection_finish()
    r.statistical_cuts()      # calculate_means .. statistical_cuts, construct_sinogram
    r.FBP()
    r.hull_selection()
    r.define_initial_iterate()
    r.image_reconstruction_GPU()   # endpoints, MLP rows, DROP iterations

Every call goes through the C ABI of libpct_gb300.so (include/pct.h); the
library must be built, and on a machine without a CUDA device pct_create()
fails with PCT_ERR_CUDA.  There is no CPU fallback.
"""
import ctypes as C

import numpy as np

from . import _capi
from .phantoms import make_config


class Counts(C.Structure):
    _fields_ = [("total_histories", C.c_int64), ("recon_vol_histories", C.c_int64),
                ("post_cut_histories", C.c_int64), ("reconstruction_histories", C.c_int64),
                ("row_entries", C.c_int64), ("rows_outside_image", C.c_int64), ("walks_capped", C.c_int64),
                ("mlp_fp64_samples", C.c_int64), ("walk_fp64_steps", C.c_int64), ("kernel_launches", C.c_int64),
                ("drop_list_entries", C.c_int64)]


class DropStats(C.Structure):
    _fields_ = [("iterations_run", C.c_int), ("residual", C.c_double * 64), ("seconds", C.c_double),
                ("drop_form", C.c_int)]


ARRAYS = ["MSC_COUNTS", "SM_COUNTS", "SC_HULL", "MSC_HULL", "SM_HULL", "BIN_COUNTS_PRE", "MEAN_WEPL", "MEAN_UT",
          "MEAN_UV", "SD_WEPL", "SD_UT", "SD_UV", "BIN_COUNTS_POST", "SINOGRAM", "SINOGRAM_FILTERED", "FBP_IMAGE",
          "FBP_HULL", "X_HULL", "X_HULL_FILTERED", "X0", "X", "H_BIN_NUM", "H_WEPL", "H_X_ENTRY", "H_Y_ENTRY",
          "H_Z_ENTRY", "H_X_EXIT", "H_Y_EXIT", "H_Z_EXIT", "H_XY_ENTRY_ANGLE", "H_XZ_ENTRY_ANGLE", "H_XY_EXIT_ANGLE",
          "H_XZ_EXIT_ANGLE", "H_FIRST_VOXEL", "H_FAILED_CUTS", "ROW_OFFSETS", "ROWS", "CHORD"]
ARRAY_ID = {name: k for k, name in enumerate(ARRAYS)}
_DTYPES = {"MSC_COUNTS": np.int32, "SM_COUNTS": np.int32, "SC_HULL": np.int32, "MSC_HULL": np.int32,
           "SM_HULL": np.int32, "BIN_COUNTS_PRE": np.int32, "BIN_COUNTS_POST": np.int32, "FBP_HULL": np.uint8,
           "X_HULL": np.uint8, "X_HULL_FILTERED": np.uint8, "H_BIN_NUM": np.int32, "H_FIRST_VOXEL": np.uint32,
           "H_FAILED_CUTS": np.uint8, "ROW_OFFSETS": np.int64, "ROWS": np.uint32}


@_capi.register
def _declare(lib):
    vp, i64, ci = C.c_void_p, C.c_int64, C.c_int
    lib.pct_create.argtypes = [C.POINTER(_capi.Config), ci, C.POINTER(vp)]
    lib.pct_destroy.argtypes = [vp]
    lib.pct_reserve.argtypes = [vp, i64]
    lib.pct_process_chunk.argtypes = [vp, C.POINTER(vp), vp, i64, ci]
    for name in ("pct_hull_detection_finish", "pct_statistical_cuts", "pct_fbp", "pct_hull_selection",
                 "pct_define_initial_iterate", "pct_collect_mlp_endpoints", "pct_mlp_rows"):
        getattr(lib, name).argtypes = [vp]
    lib.pct_drop.argtypes = [vp, ci, C.POINTER(DropStats)]
    lib.pct_image_reconstruction.argtypes = [vp, C.POINTER(DropStats)]
    lib.pct_drop_fp64.argtypes = [vp, ci, C.c_void_p, C.POINTER(DropStats)]
    lib.pct_get_counts.argtypes = [vp, C.POINTER(Counts)]
    lib.pct_get_array.argtypes = [vp, ci, vp, C.POINTER(C.c_size_t)]
    lib.pct_array_device_ptr.argtypes = [vp, ci, C.POINTER(vp), C.POINTER(C.c_size_t)]
    lib.pct_set_image.argtypes = [vp, vp]
    lib.pct_reset_iterate.argtypes = [vp]
    lib.pct_stream.restype = vp
    lib.pct_stream.argtypes = [vp]
    lib.pct_process_pctd_files.argtypes = [vp, C.POINTER(C.c_char_p), ci]
    for name in ("pct_write_mlp_endpoints", "pct_read_mlp_endpoints", "pct_write_mlp_paths", "pct_read_mlp_paths",
                 "pct_read_image"):
        getattr(lib, name).argtypes = [vp, C.c_char_p]
    lib.pct_write_image.argtypes = [vp, ci, C.c_char_p]
    lib.pct_select_shard.argtypes = [vp, ci, ci]
    lib.pct_set_allreduce.argtypes = [vp, _capi.ALLREDUCE_FN, vp]
    lib.pct_memcpy.argtypes = [vp, vp, i64]
    lib.pct_set_block_size.argtypes = [vp, ci]
    lib.pct_drop_many.argtypes = [C.POINTER(vp), ci, ci, C.POINTER(DropStats)]
    lib.pct_compact_rows.argtypes = [vp]


class Reconstruction:
    """One reconstruction context on one CUDA device."""

    def __init__(self, config, device=0):
        self.lib = _capi.load()
        self.cfg = make_config(config) if isinstance(config, dict) else config
        h = C.c_void_p()
        _capi.check(self.lib.pct_create(C.byref(self.cfg), device, C.byref(h)), "pct_create")
        self.h = h
        self._keep = []

    def close(self):
        if self.h:
            self.lib.pct_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _call(self, name, *args):
        _capi.check(getattr(self.lib, name)(self.h, *args), name)

    # ---- stages (reference entry-point names) ---------------------------------
    def reserve(self, n):
        self._call("pct_reserve", int(n))

    def process_chunk(self, data13, projection_angle):
        """Host arrays: (13, n) float32 PCTD data in mm, (n,) float32 header angles.
        Each of the 13 rows must be contiguous, not the whole array: a column
        slice of a larger (pinned) array is uploaded from where it lies."""
        rows = [np.ascontiguousarray(data13[k], dtype=np.float32) for k in range(13)]
        projection_angle = np.ascontiguousarray(projection_angle, dtype=np.float32)
        n = rows[0].shape[0]
        if any(r.shape != (n,) for r in rows) or projection_angle.shape != (n,):
            raise ValueError("process_chunk: 13 rows and the angles must have the same length")
        ptrs = (C.c_void_p * 13)(*[r.ctypes.data for r in rows])
        self._call("pct_process_chunk", ptrs, projection_angle.ctypes.data, n, 0)

    def process_pctd_files(self, paths):
        """Reads PCTD v0 files (one per gantry angle) and uploads each as a chunk."""
        arr = (C.c_char_p * len(paths))(*[p.encode() for p in paths])
        self._call("pct_process_pctd_files", arr, len(paths))

    # ---- files (write/read_MLP_endpoints, MLP path files, image checkpoints) -----
    def write_mlp_endpoints(self, path):
        self._call("pct_write_mlp_endpoints", str(path).encode())

    def read_mlp_endpoints(self, path):
        self._call("pct_read_mlp_endpoints", str(path).encode())

    def write_mlp_paths(self, path):
        self._call("pct_write_mlp_paths", str(path).encode())

    def read_mlp_paths(self, path):
        self._call("pct_read_mlp_paths", str(path).encode())

    def write_image(self, path, name="X"):
        self._call("pct_write_image", ARRAY_ID[name], str(path).encode())

    def read_image(self, path):
        self._call("pct_read_image", str(path).encode())

    def process_chunk_device(self, ptrs13, angle_ptr, n):
        """Device pointers (ints) to the 13 PCTD arrays and the angles."""
        ptrs = (C.c_void_p * 13)(*ptrs13)
        self._call("pct_process_chunk", ptrs, angle_ptr, int(n), 1)

    def hull_detection_finish(self):
        self._call("pct_hull_detection_finish")

    def statistical_cuts(self):
        self._call("pct_statistical_cuts")

    def FBP(self):
        self._call("pct_fbp")

    def hull_selection(self):
        self._call("pct_hull_selection")

    def define_initial_iterate(self):
        self._call("pct_define_initial_iterate")

    def collect_mlp_endpoints(self):
        self._call("pct_collect_mlp_endpoints")

    def mlp_rows(self):
        self._call("pct_mlp_rows")

    def drop(self, iterations):
        st = DropStats()
        self._call("pct_drop", int(iterations), C.byref(st))
        return st

    def compact_rows(self):
        """Packs the MLP rows back to back (pct_compact_rows)."""
        self._call("pct_compact_rows")

    def drop_fp64(self, iterations, x):
        """Binary64 DROP iterations from image x (NUM_VOXELS values, linear order); returns
        (the binary64 image, stats).  The binary32 iterate is not touched (pct_drop_fp64)."""
        xd = np.array(x, dtype=np.float64, copy=True)
        st = DropStats()
        self._call("pct_drop_fp64", int(iterations), C.c_void_p(xd.ctypes.data), C.byref(st))
        return xd, st

    def image_reconstruction_GPU(self):
        st = DropStats()
        self._call("pct_image_reconstruction", C.byref(st))
        return st

    def reset_iterate(self):
        self._call("pct_reset_iterate")

    def set_block_size(self, block_size):
        """DROP block size for the next drop() (pct_set_block_size)."""
        self._call("pct_set_block_size", int(block_size))
        self.cfg.block_size = int(block_size)

    def select_shard(self, shard, num_shards):
        """Keeps this rank's share of every DROP block (pct_select_shard)."""
        self._call("pct_select_shard", int(shard), int(num_shards))

    def set_allreduce(self, fn):
        """fn(user, data, count, dtype, on_device) -> 0 sums `data` over the ranks; None clears it."""
        self._allreduce_fn = _capi.ALLREDUCE_FN(fn) if fn is not None else None
        self._call("pct_set_allreduce", self._allreduce_fn if fn is not None else _capi.ALLREDUCE_FN(), None)

    def set_image(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        self._call("pct_set_image", x.ctypes.data)

    # ---- results ------------------------------------------------------------------
    def counts(self):
        c = Counts()
        self._call("pct_get_counts", C.byref(c))
        return {k: getattr(c, k) for k, _ in Counts._fields_}

    def array(self, name):
        which = ARRAY_ID[name]
        nbytes = C.c_size_t(0)
        self._call("pct_get_array", which, None, C.byref(nbytes))
        dt = np.dtype(_DTYPES.get(name, np.float32))
        out = np.empty(nbytes.value // dt.itemsize, dtype=dt)
        if nbytes.value:
            self._call("pct_get_array", which, out.ctypes.data, C.byref(nbytes))
        return out

    def device_ptr(self, name):
        p = C.c_void_p()
        nbytes = C.c_size_t(0)
        self._call("pct_array_device_ptr", ARRAY_ID[name], C.byref(p), C.byref(nbytes))
        return p.value, nbytes.value

    def stream(self):
        return self.lib.pct_stream(self.h)


def drop_many(recons, iterations):
    """DROP iterations of several reconstructions (each after mlp_rows, with its
    own block size) in one persistent launch per iteration (pct_drop_many);
    returns their DropStats."""
    recons = list(recons)
    if not recons:
        return []
    lib = recons[0].lib
    handles = (C.c_void_p * len(recons))(*[r.h for r in recons])
    stats = (DropStats * len(recons))()
    _capi.check(lib.pct_drop_many(handles, len(recons), int(iterations), stats), "pct_drop_many")
    return list(stats)


def run_full(config, data13, projection_angle, chunk=None, device=0):
    """The whole reference sequence on one host dataset; returns the context."""
    r = Reconstruction(config, device=device)
    n = data13.shape[1]
    r.reserve(n)
    chunk = chunk or n
    for s in range(0, n, chunk):
        r.process_chunk(data13[:, s:s + chunk], projection_angle[s:s + chunk])
    r.hull_detection_finish()
    r.statistical_cuts()
    r.FBP()
    r.hull_selection()
    r.define_initial_iterate()
    return r
