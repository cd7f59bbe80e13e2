"""ctypes view of include/pct.h.

Loads the in-tree pct_gb300/_lib/libpct_gb300.so and declares the C ABI.  The
struct layouts below mirror include/pct.h field for field; load() checks their
sizes against pct_sizeof() so a header change without a binding change fails
loudly instead of passing garbage.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libpct_gb300.so")

PCT_OK = 0
(PCT_ERR_ARGUMENT, PCT_ERR_CUDA, PCT_ERR_ALLOC, PCT_ERR_STATE, PCT_ERR_OVERFLOW, PCT_ERR_TIMEOUT, PCT_ERR_IO,
 PCT_ERR_NUMERIC) = range(1, 9)


class PctError(RuntimeError):
    """A pct_* call returned a non-OK status."""

    def __init__(self, status, message):
        super().__init__("%s (status %d)" % (message, status))
        self.status = status


class Config(C.Structure):
    _fields_ = [
        ("source_radius", C.c_double), ("gantry_angle_interval", C.c_double),
        ("ssd_t_size", C.c_double), ("ssd_v_size", C.c_double),
        ("t_bin_size", C.c_double), ("v_bin_size", C.c_double),
        ("angular_bin_size", C.c_double), ("sigmas_to_keep", C.c_int), ("sample_std_dev", C.c_int),
        ("recon_cyl_radius", C.c_double), ("columns", C.c_int), ("rows", C.c_int),
        ("slice_thickness", C.c_double),
        ("sc_on", C.c_int), ("msc_on", C.c_int), ("sm_on", C.c_int),
        ("avg_filter_hull", C.c_int), ("mlp_hull", C.c_int), ("msc_diff_thresh", C.c_int),
        ("sc_threshold", C.c_double), ("msc_threshold", C.c_double),
        ("sm_lower_threshold", C.c_double), ("sm_scale_threshold", C.c_double),
        ("hull_filter_threshold", C.c_double), ("hull_filter_radius", C.c_int),
        ("fbp_on", C.c_int), ("fbp_filter", C.c_int), ("fbp_threshold", C.c_double),
        ("x_k0", C.c_int), ("iterations", C.c_int), ("block_size", C.c_int), ("lambda_", C.c_float),
        ("residual_tol", C.c_double), ("chord_bf16", C.c_int), ("mlp_exact", C.c_int),
        ("mlp_face_margin", C.c_double), ("drop_form", C.c_int), ("walk_exact", C.c_int),
        ("voxel_order", C.c_int), ("drop_variant", C.c_int), ("eta", C.c_double), ("psi_sign", C.c_int),
        ("mlp_tabulated", C.c_int),
    ]


class Geometry(C.Structure):
    _fields_ = [
        ("columns", C.c_int), ("rows", C.c_int), ("slices", C.c_int), ("num_voxels", C.c_int),
        ("t_bins", C.c_int), ("v_bins", C.c_int), ("angular_bins", C.c_int), ("num_bins", C.c_int),
        ("gantry_angles", C.c_int),
        ("recon_cyl_radius", C.c_double), ("recon_cyl_height", C.c_double),
        ("voxel_width", C.c_double), ("voxel_height", C.c_double), ("voxel_thickness", C.c_double),
        ("x_zero", C.c_double), ("y_zero", C.c_double), ("z_zero", C.c_double),
        ("mlp_u_step", C.c_double),
    ]


class PhantomObject(C.Structure):
    _fields_ = [("kind", C.c_int), ("cx", C.c_double), ("cy", C.c_double), ("cz", C.c_double),
                ("a", C.c_double), ("b", C.c_double), ("c", C.c_double), ("phi", C.c_double),
                ("rsp", C.c_double)]


class ScanParams(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("num_angles", C.c_int), ("gantry_angle_interval", C.c_double),
                ("t_extent", C.c_double), ("v_extent", C.c_double), ("source_radius", C.c_double),
                ("angular_spread", C.c_double), ("beam_energy_mev", C.c_double), ("wepl_noise", C.c_double),
                ("outlier_fraction", C.c_double), ("outlier_max", C.c_double), ("scatter_scale", C.c_double)]


_STRUCTS = [(0, Config), (1, Geometry), (2, PhantomObject), (3, ScanParams)]
_lib = None


# pct_allreduce_fn: (user, data, count, dtype, on_device) -> 0 on success
ALLREDUCE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_int)
PCT_DT_F32, PCT_DT_U32, PCT_DT_F64 = 0, 1, 2


def load():
    """Returns the loaded library; raises if it was never built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libpct_gb300.so is not built (run __graft_entry__.build() or "
                           "python pct_gb300/build.py): %s" % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    lib.pct_sizeof.restype = C.c_size_t
    lib.pct_sizeof.argtypes = [C.c_int]
    for which, cls in _STRUCTS:
        n = lib.pct_sizeof(which)
        if n != C.sizeof(cls):
            raise RuntimeError("ABI mismatch for %s: library %d bytes, binding %d" % (cls.__name__, n, C.sizeof(cls)))
    lib.pct_last_error.restype = C.c_char_p
    lib.pct_status_string.restype = C.c_char_p
    lib.pct_status_string.argtypes = [C.c_int]
    lib.pct_config_default.argtypes = [C.POINTER(Config)]
    lib.pct_geometry_from_config.argtypes = [C.POINTER(Config), C.POINTER(Geometry)]
    lib.pct_generate_histories.argtypes = [C.POINTER(PhantomObject), C.c_int, C.POINTER(ScanParams),
                                           C.POINTER(C.c_void_p), C.c_void_p, C.c_int64]
    lib.pct_phantom_voxelize.argtypes = [C.POINTER(PhantomObject), C.c_int, C.POINTER(Config), C.c_int, C.c_void_p]
    _declare_extra(lib)
    _lib = lib
    return lib


_EXTRA = []


def register(fn):
    """Registers a function that adds argtypes for more entry points at load time."""
    _EXTRA.append(fn)
    if _lib is not None:
        fn(_lib)
    return fn


def _declare_extra(lib):
    for fn in _EXTRA:
        fn(lib)


def check(status, what=""):
    if status != PCT_OK:
        lib = load()
        msg = lib.pct_last_error().decode(errors="replace")
        raise PctError(status, "%s: %s" % (what, msg) if what else msg)
    return status
