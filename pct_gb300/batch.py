"""Batched scans on one GPU and a DROP block-size search.

Many small scans do not fill a GB300 one at a time: for a 2M-history scan on a
128x128x8 grid a DROP block step lasts tens of microseconds and the MLP pass a
few milliseconds.  reconstruct_many() runs each scan in its own context, with
its own CUDA stream, from its own host thread (every C ABI call releases the
interpreter lock), so the kernels of different scans overlap on the device.

autotune_block_size() picks the DROP block size (BLOCK_SIZE_RECON, the
reference's block loop, src/pCT_Reconstruction_Data_Segments.cu:6803-6844) of
one scan by measured time to a residual: the block size changes the iteration
itself (smaller blocks relax more often per iteration but put fewer rows in
each launch), so the iteration rate alone is not the criterion.
"""
import math
import threading
import time

from . import recon


def reconstruct_many(scans, device=0, concurrent=True):
    """scans: list of (config, data13, projection_angles).  Runs the reference
    sequence and image_reconstruction_GPU on each scan; returns the images
    (linear voxel order) and the wall time in seconds."""
    images = [None] * len(scans)
    errors = [None] * len(scans)

    def one(k):
        try:
            cfg, data, angles = scans[k]
            r = recon.run_full(cfg, data, angles, device=device)
            r.image_reconstruction_GPU()
            images[k] = r.array("X")
            r.close()
        except Exception as e:  # re-raised in the caller's thread
            errors[k] = e

    t0 = time.perf_counter()
    if concurrent:
        threads = [threading.Thread(target=one, args=(k,)) for k in range(len(scans))]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
    else:
        for k in range(len(scans)):
            one(k)
    seconds = time.perf_counter() - t0
    for e in errors:
        if e is not None:
            raise e
    return images, seconds


def autotune_block_size(r, candidates=(20000, 50000, 100000, 200000, 400000), iterations=None, target=None):
    """Block size of scan `r` (a Reconstruction after mlp_rows()) with the
    shortest time to reach a relative residual.

    Each candidate runs `iterations` DROP iterations from the initial iterate;
    its time to the target is its time per iteration times the iterations
    until the residual of an iteration is at or below the target (infinite if
    it never is).  The target defaults to the residual the context's current
    block size reaches in its last iteration.  Returns (best block size,
    [(block size, seconds per iteration, residuals, seconds to target)]); `r`
    is left with the best block size and the initial iterate."""
    its = int(iterations or r.cfg.iterations)
    current = int(r.cfg.block_size)
    sizes = [current] + [int(b) for b in candidates if int(b) != current]
    table = []
    for b in sizes:
        r.set_block_size(b)
        r.reset_iterate()
        st = r.drop(its)
        res = [float(st.residual[k]) for k in range(st.iterations_run)]
        table.append([b, st.seconds / max(st.iterations_run, 1), res, None])
    goal = float(target) if target is not None else table[0][2][-1]
    for row in table:
        hit = next((k + 1 for k, v in enumerate(row[2]) if v <= goal), None)
        row[3] = hit * row[1] if hit is not None else math.inf
    best = min(table, key=lambda t: (t[3], t[0]))
    r.set_block_size(best[0])
    r.reset_iterate()
    return best[0], [tuple(t) for t in table]


def main():
    """Measurement on the batched-scan workload: K ellipsoid scans (seeded,
    histories log-uniform in [--min, --max]), one after another and then
    concurrently, after one warm-up scan; then the block-size search on the
    largest scan.  Prints one JSON line."""
    import argparse
    import json
    import random

    import numpy as np

    from . import phantoms

    ap = argparse.ArgumentParser()
    ap.add_argument("--scans", type=int, default=8)
    ap.add_argument("--min", type=float, default=2e6)
    ap.add_argument("--max", type=float, default=10e6)
    ap.add_argument("--seed", type=int, default=100)
    a = ap.parse_args()
    rng = random.Random(a.seed)
    scans, recon_hist = [], []
    for k in range(a.scans):
        n = int(round(math.exp(rng.uniform(math.log(a.min), math.log(a.max)))))
        w = phantoms.ellipsoids(a.seed + k, num_histories=n)
        data, angles = phantoms.generate(w)
        scans.append((phantoms.make_config(w.config), data, angles))
    reconstruct_many(scans[:1], concurrent=False)  # warm-up: module load, first allocations
    seq, t_seq = reconstruct_many(scans, concurrent=False)
    con, t_con = reconstruct_many(scans, concurrent=True)
    worst = max(float(np.linalg.norm(x - y) / max(np.linalg.norm(x), 1e-30)) for x, y in zip(seq, con))
    iters = sum(c.iterations for c, _, _ in scans)
    for cfg, data, angles in scans:
        r = recon.run_full(cfg, data, angles)
        r.collect_mlp_endpoints()
        recon_hist.append(r.counts()["reconstruction_histories"])
        r.close()
    units = sum(h * c.iterations for h, (c, _, _) in zip(recon_hist, scans))
    big = max(range(a.scans), key=lambda k: recon_hist[k])
    cfg, data, angles = scans[big]
    r = recon.run_full(cfg, data, angles)
    r.collect_mlp_endpoints()
    r.mlp_rows()
    best, table = autotune_block_size(r)
    r.close()
    g = [phantoms.geometry(c) for c, _, _ in scans]
    print(json.dumps({
        "workload": "%d ellipsoid scans, %d-%d histories, grids %s" % (
            a.scans, min(d.shape[1] for _, d, _ in scans), max(d.shape[1] for _, d, _ in scans),
            sorted({"%dx%dx%d" % (x.columns, x.rows, x.slices) for x in g})),
        "reconstruction_histories": recon_hist, "iterations": iters,
        "sequential_seconds": t_seq, "concurrent_seconds": t_con,
        "histories_iterations_per_second": {"sequential": units / t_seq, "concurrent": units / t_con},
        "max_relative_l2_concurrent_vs_sequential": worst,
        "block_size_search": {"scan": big, "best": best,
                              "table": [{"block": t[0], "ms_per_iteration": t[1] * 1e3,
                                         "ms_to_target": (t[3] * 1e3 if math.isfinite(t[3]) else None)}
                                        for t in table]}}))


if __name__ == "__main__":
    main()
