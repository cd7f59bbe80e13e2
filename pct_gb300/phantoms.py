"""Synthetic workloads: reconstruction config + phantom + seeded scan parameters.

The reference ships no benchmark data; these seeded synthetic scans stand in
for its CTP404-style PCTD inputs (same file layout, same geometry knobs).
Each workload names the configuration it reproduces:

  tiny   64x64x4 grid (r = 3.2 cm), 90 angles: golden vectors and fast tests.
  cfg1   water cylinder r = 8 cm with 4 inserts (RSP 0.9/1.05/1.2/1.6),
         2M histories, 90 angles / 4 deg, 200x200x8 at 1x1x2.5 mm, SM hull,
         Shepp-Logan FBP, 6 DROP iterations, block 60000, lambda 0.1.
  cfg2   r = 10 cm cylinder with 8 inserts (RSP 0.3-1.8), 30M histories,
         180 angles / 2 deg, 256x256x32, 12 iterations, block 200000, lambda 0.1.
  cfg4   head phantom (skull 1.6, brain 1.04, ventricles 1.0, 6 lesions
         0.95-1.1), 60M histories, 180 angles, 320x320x64 at 0.8x0.8x2.5 mm.
  ellipsoids(seed)  random 3-12 ellipsoid phantom (RSP 0.2-1.9) on a grid
         between 128x128x8 and 256x256x48, for the batched-scan workload.
"""
import ctypes as C
import dataclasses
import math
import random

import numpy as np

from . import _capi


@dataclasses.dataclass
class Workload:
    name: str
    config: dict                  # pct_config fields that differ from the reference defaults
    objects: list                 # (kind, cx, cy, cz, a, b, c, phi, rsp)
    num_histories: int
    num_angles: int
    gantry_angle_interval: float
    t_extent: float
    v_extent: float
    seed: int = 1
    wepl_noise: float = 0.02
    outlier_fraction: float = 0.03
    outlier_max: float = 40.0
    angular_spread: float = 0.002
    scatter_scale: float = 1.0

    def scaled(self, num_histories, seed=None):
        w = dataclasses.replace(self, num_histories=int(num_histories))
        if seed is not None:
            w.seed = seed
        return w


CYL, ELL = 0, 1


def _cylinder_with_inserts(r_body, half_height, insert_ring, insert_r, insert_rsps, body_rsp=1.0):
    objs = [(CYL, 0.0, 0.0, 0.0, r_body, r_body, half_height, 0.0, body_rsp)]
    n = len(insert_rsps)
    for k, rsp in enumerate(insert_rsps):
        a = 2 * math.pi * k / n
        objs.append((CYL, insert_ring * math.cos(a), insert_ring * math.sin(a), 0.0,
                     insert_r, insert_r, half_height, 0.0, rsp - body_rsp))
    return objs


def tiny(num_histories=60000, seed=7, v_extent=0.3):
    return Workload(
        name="tiny",
        config=dict(recon_cyl_radius=3.2, columns=64, rows=64, ssd_v_size=2.0, ssd_t_size=12.0,
                    gantry_angle_interval=4.0, angular_bin_size=4.0, iterations=2, block_size=6000,
                    lambda_=0.1),
        objects=_cylinder_with_inserts(2.4, 3.0, 1.1, 0.55, [0.5, 1.5]),
        num_histories=num_histories, num_angles=90, gantry_angle_interval=4.0,
        t_extent=3.0, v_extent=v_extent, seed=seed, outlier_max=8.0)


def cfg1(num_histories=2_000_000, seed=1):
    return Workload(
        name="cfg1",
        config=dict(recon_cyl_radius=10.0, columns=200, rows=200, ssd_v_size=3.0,
                    gantry_angle_interval=4.0, angular_bin_size=4.0, sm_on=1, msc_on=0,
                    mlp_hull=2, iterations=6, block_size=60000, lambda_=0.1),
        objects=_cylinder_with_inserts(8.0, 5.0, 4.0, 1.0, [0.9, 1.05, 1.2, 1.6]),
        num_histories=num_histories, num_angles=90, gantry_angle_interval=4.0,
        t_extent=9.5, v_extent=1.05, seed=seed)


def cfg2(num_histories=30_000_000, seed=2):
    return Workload(
        name="cfg2",
        config=dict(recon_cyl_radius=12.8, columns=256, rows=256, ssd_v_size=9.0,
                    gantry_angle_interval=2.0, angular_bin_size=2.0, sm_on=1, msc_on=0,
                    mlp_hull=2, iterations=12, block_size=200000, lambda_=0.1),
        objects=_cylinder_with_inserts(10.0, 6.0, 5.5, 1.1, [0.3, 0.5, 0.8, 1.04, 1.2, 1.4, 1.6, 1.8]),
        num_histories=num_histories, num_angles=180, gantry_angle_interval=2.0,
        t_extent=11.8, v_extent=4.05, seed=seed)


def cfg4(num_histories=60_000_000, seed=4):
    objs = [
        (ELL, 0.0, 0.0, 0.0, 9.0, 11.0, 10.0, 0.0, 1.6),        # skull outer
        (ELL, 0.0, 0.0, 0.0, 8.4, 10.4, 9.4, 0.0, 1.04 - 1.6),  # brain replaces skull inside
        (ELL, -1.2, 0.5, 0.0, 0.8, 2.5, 3.0, 0.3, 1.0 - 1.04),  # ventricles
        (ELL, 1.2, 0.5, 0.0, 0.8, 2.5, 3.0, -0.3, 1.0 - 1.04),
    ]
    for k, rsp in enumerate([0.95, 0.98, 1.02, 1.06, 1.08, 1.1]):
        a = 2 * math.pi * k / 6
        objs.append((ELL, 5.0 * math.cos(a), 6.0 * math.sin(a), 0.5 * (k % 3 - 1), 0.7, 0.7, 0.7, 0.0, rsp - 1.04))
    return Workload(
        name="cfg4",
        config=dict(recon_cyl_radius=12.8, columns=320, rows=320, ssd_v_size=17.0,
                    gantry_angle_interval=2.0, angular_bin_size=2.0, sm_on=1, msc_on=0,
                    mlp_hull=2, iterations=12, block_size=200000, lambda_=0.1, chord_bf16=1),
        objects=objs, num_histories=num_histories, num_angles=180, gantry_angle_interval=2.0,
        t_extent=12.2, v_extent=8.05, seed=seed)


def ellipsoids(seed, num_histories=None, cols=None, slices=None):
    """Random ellipsoid phantom of the batched-scan workload (3-12 ellipsoids, RSP 0.2-1.9);
    the grid (128-256 columns, 8-48 slices) is drawn from the seed unless given."""
    rng = random.Random(seed)
    cols_drawn = rng.choice([128, 160, 192, 224, 256])
    slices_drawn = rng.choice([8, 16, 24, 32, 40, 48])
    cols = cols_drawn if cols is None else cols
    slices = slices_drawn if slices is None else slices
    r_cyl = cols * 0.1 / 2
    body_a = r_cyl * rng.uniform(0.55, 0.75)
    body_b = r_cyl * rng.uniform(0.55, 0.75)
    height = slices * 0.25
    objs = [(ELL, 0.0, 0.0, 0.0, body_a, body_b, height, 0.0, 1.0)]
    for _ in range(rng.randint(3, 12) - 1):
        a = rng.uniform(0.05, 0.3) * body_a
        b = rng.uniform(0.05, 0.3) * body_b
        c = rng.uniform(0.2, 0.6) * height
        cx = rng.uniform(-0.5, 0.5) * body_a
        cy = rng.uniform(-0.5, 0.5) * body_b
        objs.append((ELL, cx, cy, 0.0, a, b, c, rng.uniform(0, math.pi), rng.uniform(0.2, 1.9) - 1.0))
    if num_histories is None:
        num_histories = int(round(math.exp(rng.uniform(math.log(2e6), math.log(40e6)))))
    return Workload(
        name="ellipsoids_%d" % seed,
        config=dict(recon_cyl_radius=r_cyl, columns=cols, rows=cols, ssd_v_size=height + 1.0,
                    gantry_angle_interval=2.0, angular_bin_size=2.0, sm_on=1, msc_on=0, mlp_hull=2,
                    iterations=12, block_size=200000, lambda_=0.1),
        objects=objs, num_histories=num_histories, num_angles=180, gantry_angle_interval=2.0,
        t_extent=r_cyl * 0.92, v_extent=height / 2 * 0.98, seed=seed)


WORKLOADS = {"tiny": tiny, "cfg1": cfg1, "cfg2": cfg2, "cfg4": cfg4}


def make_config(overrides):
    lib = _capi.load()
    cfg = _capi.Config()
    _capi.check(lib.pct_config_default(C.byref(cfg)), "pct_config_default")
    for k, v in overrides.items():
        setattr(cfg, k, v)
    return cfg


def geometry(cfg):
    lib = _capi.load()
    g = _capi.Geometry()
    _capi.check(lib.pct_geometry_from_config(C.byref(cfg), C.byref(g)), "pct_geometry_from_config")
    return g


def _objects_array(objs):
    arr = (_capi.PhantomObject * max(1, len(objs)))()
    for i, o in enumerate(objs):
        arr[i] = _capi.PhantomObject(*o)
    return arr


def generate(w):
    """Returns ((13, N) float32 PCTD arrays in mm, (N,) float32 projection angles)."""
    lib = _capi.load()
    n = int(w.num_histories)
    data = np.empty((13, n), dtype=np.float32)
    angles = np.empty(n, dtype=np.float32)
    sp = _capi.ScanParams(seed=w.seed, num_angles=w.num_angles, gantry_angle_interval=w.gantry_angle_interval,
                          t_extent=w.t_extent, v_extent=w.v_extent, source_radius=260.7,
                          angular_spread=w.angular_spread, beam_energy_mev=200.0, wepl_noise=w.wepl_noise,
                          outlier_fraction=w.outlier_fraction, outlier_max=w.outlier_max,
                          scatter_scale=w.scatter_scale)
    ptrs = (C.c_void_p * 13)(*[data[k].ctypes.data for k in range(13)])
    objs = _objects_array(w.objects)
    _capi.check(lib.pct_generate_histories(objs, len(w.objects), C.byref(sp), ptrs, angles.ctypes.data, n),
                "pct_generate_histories")
    return data, angles


def voxelize(w, supersample=3):
    lib = _capi.load()
    cfg = make_config(w.config)
    g = geometry(cfg)
    img = np.empty(g.num_voxels, dtype=np.float32)
    objs = _objects_array(w.objects)
    _capi.check(lib.pct_phantom_voxelize(objs, len(w.objects), C.byref(cfg), supersample, img.ctypes.data),
                "pct_phantom_voxelize")
    return img
