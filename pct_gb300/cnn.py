"""ctypes view of include/pct_cnn.h: the learned DROP warm start.

Net wraps a pct_cnn (3D residual CNN, tcgen05 tensor-core convolutions in
libpct_gb300.so).  Volumes are numpy arrays in the voxel order of
Reconstruction.array(): [z][y][x] flattened, x extent 128.
"""
import ctypes as C

import numpy as np

from . import _capi

LAYERS = [(2, 32)] + [(32, 32)] * 6 + [(32, 1)]  # (c_in, c_out) per layer
TAPS = 27


@_capi.register
def _declare(lib):
    vp, ci = C.c_void_p, C.c_int
    lib.pct_cnn_create.argtypes = [ci, ci, ci, ci, C.POINTER(vp)]
    lib.pct_cnn_destroy.argtypes = [vp]
    lib.pct_cnn_num_params.restype = C.c_size_t
    lib.pct_cnn_init.argtypes = [vp, C.c_uint64]
    lib.pct_cnn_set_params.argtypes = [vp, vp, C.c_size_t]
    lib.pct_cnn_get_params.argtypes = [vp, vp, C.c_size_t]
    lib.pct_cnn_forward.argtypes = [vp, vp, vp, vp, ci]
    lib.pct_cnn_gradients.argtypes = [vp, vp, vp, vp, ci, C.POINTER(C.c_double), vp]
    lib.pct_cnn_train_step.argtypes = [vp, vp, vp, vp, ci, C.c_float, C.POINTER(C.c_double)]
    lib.pct_cnn_inspect.argtypes = [vp, ci, ci, vp, C.c_size_t]
    lib.pct_cnn_counts.argtypes = [vp, C.POINTER(C.c_int64)]
    lib.pct_cnn_warm_start.argtypes = [vp, vp]


def param_slices():
    """(weight slice, weight shape [27, c_out, c_in], bias slice) per layer in the parameter vector."""
    out, off = [], 0
    for cin, cout in LAYERS:
        nw = TAPS * cout * cin
        out.append((slice(off, off + nw), (TAPS, cout, cin), slice(off + nw, off + nw + cout)))
        off += nw + cout
    return out


class Net:
    def __init__(self, depth, height, width=128, device=0):
        self.lib = _capi.load()
        self.shape = (depth, height, width)
        self.nv = depth * height * width
        h = C.c_void_p()
        _capi.check(self.lib.pct_cnn_create(device, depth, height, width, C.byref(h)), "pct_cnn_create")
        self.h = h
        self.nparams = int(self.lib.pct_cnn_num_params())

    def close(self):
        if getattr(self, "h", None):
            self.lib.pct_cnn_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _call(self, name, *args):
        _capi.check(getattr(self.lib, name)(self.h, *args), name)

    def init(self, seed):
        self._call("pct_cnn_init", int(seed))

    def params(self):
        p = np.empty(self.nparams, np.float32)
        self._call("pct_cnn_get_params", p.ctypes.data, p.size)
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._call("pct_cnn_set_params", p.ctypes.data, p.size)

    def _in(self, x0, hull, target=None):
        x0 = np.ascontiguousarray(x0, dtype=np.float32).ravel()
        hull = np.ascontiguousarray(hull, dtype=np.uint8).ravel()
        t = None if target is None else np.ascontiguousarray(target, dtype=np.float32).ravel()
        assert x0.size == self.nv and hull.size == self.nv and (t is None or t.size == self.nv)
        return x0, hull, t

    def forward(self, x0, hull):
        x0, hull, _ = self._in(x0, hull)
        out = np.empty(self.nv, np.float32)
        self._call("pct_cnn_forward", x0.ctypes.data, hull.ctypes.data, out.ctypes.data, 0)
        return out

    def forward_device(self, x0_ptr, hull_ptr, out_ptr):
        """network(x0, hull) on device pointers (nv floats, nv bytes, nv floats)."""
        self._call("pct_cnn_forward", C.c_void_p(x0_ptr), C.c_void_p(hull_ptr), C.c_void_p(out_ptr), 1)

    def gradients(self, x0, hull, target):
        x0, hull, t = self._in(x0, hull, target)
        g = np.empty(self.nparams, np.float32)
        loss = C.c_double(0.0)
        self._call("pct_cnn_gradients", x0.ctypes.data, hull.ctypes.data, t.ctypes.data, 0, C.byref(loss),
                   g.ctypes.data)
        return float(loss.value), g

    def train_step(self, x0, hull, target, lr):
        x0, hull, t = self._in(x0, hull, target)
        loss = C.c_double(0.0)
        self._call("pct_cnn_train_step", x0.ctypes.data, hull.ctypes.data, t.ctypes.data, 0, C.c_float(lr),
                   C.byref(loss))
        return float(loss.value)

    def train_step_device(self, x0_ptr, hull_ptr, target_ptr, lr):
        loss = C.c_double(0.0)
        self._call("pct_cnn_train_step", C.c_void_p(x0_ptr), C.c_void_p(hull_ptr), C.c_void_p(target_ptr), 1,
                   C.c_float(lr), C.byref(loss))
        return float(loss.value)

    def inspect(self, kind, layer):
        c = 16 if (kind == 1 and layer == 7) else 32
        a = np.empty(self.nv * c, np.float32)
        self._call("pct_cnn_inspect", int(kind), int(layer), a.ctypes.data, a.size)
        return a.reshape(self.shape + (c,))

    def launches(self):
        n = C.c_int64(0)
        self._call("pct_cnn_counts", C.byref(n))
        return int(n.value)

    def warm_start(self, reconstruction):
        """x0 and the iterate of a Reconstruction (after define_initial_iterate) := network(x0, hull)."""
        _capi.check(self.lib.pct_cnn_warm_start(reconstruction.h, self.h), "pct_cnn_warm_start")


def _main():
    """Runs the network on random data: `reps` forward passes and one gradient pass, with
    their host-timed durations (a self-check of the tensor-core kernels and a profiling
    target)."""
    import argparse
    import time
    ap = argparse.ArgumentParser(description=_main.__doc__)
    ap.add_argument("--depth", type=int, default=16)
    ap.add_argument("--height", type=int, default=128)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args()
    rng = np.random.default_rng(0)
    net = Net(a.depth, a.height, 128)
    net.init(1)
    x0 = rng.uniform(0, 1.5, net.nv).astype(np.float32)
    hull = (x0 > 0.2).astype(np.uint8)
    t0 = time.perf_counter()
    for _ in range(a.reps):
        out = net.forward(x0, hull)
    t_fwd = (time.perf_counter() - t0) / max(a.reps, 1)
    t0 = time.perf_counter()
    loss, g = net.gradients(x0, hull, 0.9 * x0)
    t_grad = time.perf_counter() - t0
    net.close()
    print("forward %.3f ms, forward + gradients %.3f ms, loss %.6g, |out| %.6g, |grad| %.6g"
          % (t_fwd * 1e3, t_grad * 1e3, loss, float(np.abs(out).sum()), float(np.abs(g).sum())))


if __name__ == "__main__":
    _main()
