"""Batched scans on one GPU and a DROP block-size search.

Many small scans do not fill a GB300 one at a time: for a 2M-history scan on a
128x128x8 grid a DROP block step lasts tens of microseconds and the MLP pass a
few milliseconds.  reconstruct_many() runs each scan in its own context, with
its own CUDA stream, from its own host thread (every C ABI call releases the
interpreter lock), so the kernels of different scans overlap on the device.
prepare_scans() + recon.drop_many() run the DROP iterations of all scans in
one persistent launch per iteration instead (pct_drop_many: the blocks of
every scan, each with its own block size, as one work queue).

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


def prepare_scans(scans, device=0, compact=True):
    """The reference sequence through the MLP rows for every scan, one after
    another (contexts stay open; with `compact` each scan's rows are packed
    before the next scan starts, pct_compact_rows).  Returns the contexts."""
    rs = []
    try:
        for cfg, data, angles in scans:
            r = recon.run_full(cfg, data, angles, device=device)
            rs.append(r)
            r.collect_mlp_endpoints()
            r.mlp_rows()
            if compact:
                r.compact_rows()
    except Exception:
        for r in rs:
            r.close()
        raise
    return rs


def drop_phase(rs, iterations, mode):
    """DROP iterations of every prepared context from its initial iterate:
    "sequential" (one context after another), "concurrent" (one host thread
    per context, each on its own stream) or "persistent" (recon.drop_many).
    Returns (wall seconds, images)."""
    import torch

    for r in rs:
        r.reset_iterate()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    if mode == "persistent":
        recon.drop_many(rs, iterations)
    elif mode == "concurrent":
        errors = [None] * len(rs)

        def one(k):
            try:
                rs[k].drop(iterations)
            except Exception as e:  # re-raised in the caller's thread
                errors[k] = e

        threads = [threading.Thread(target=one, args=(k,)) for k in range(len(rs))]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        for e in errors:
            if e is not None:
                raise e
    else:
        for r in rs:
            r.drop(iterations)
    torch.cuda.synchronize()
    seconds = time.perf_counter() - t0
    return seconds, [r.array("X") for r in rs]


def main():
    """Measurement on the batched-scan workload: K ellipsoid scans (seeded,
    histories log-uniform in [--min, --max], grids drawn per seed from
    128-256 columns and 8-48 slices).  Every scan is prepared through its MLP
    rows (rows packed), its DROP block size is searched (autotune_block_size,
    20000-400000), and then the DROP phase (all scans, `iterations` each, from
    their initial iterates) is timed three ways: contexts one after another,
    concurrent contexts (a host thread and stream each), and one persistent
    launch per iteration (pct_drop_many).  Prints one JSON line."""
    import argparse
    import json
    import random

    import numpy as np
    import torch

    from . import phantoms

    ap = argparse.ArgumentParser()
    ap.add_argument("--scans", type=int, default=16)
    ap.add_argument("--min", type=float, default=2e6)
    ap.add_argument("--max", type=float, default=40e6)
    ap.add_argument("--seed", type=int, default=100)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--reps", type=int, default=2)
    a = ap.parse_args()
    rng = random.Random(a.seed)
    scans_meta = []
    rs = []
    t0 = time.perf_counter()
    try:
        for k in range(a.scans):
            n = int(round(math.exp(rng.uniform(math.log(a.min), math.log(a.max)))))
            w = phantoms.ellipsoids(a.seed + k, num_histories=n)
            data, angles = phantoms.generate(w)
            cfg = phantoms.make_config(w.config)
            rs += prepare_scans([(cfg, data, angles)])
            del data, angles
            g = phantoms.geometry(cfg)
            scans_meta.append({"seed": a.seed + k, "histories": n, "grid": "%dx%dx%d" % (g.columns, g.rows, g.slices),
                               "recon_histories": rs[-1].counts()["reconstruction_histories"]})
        t_prep = time.perf_counter() - t0
        free, total = torch.cuda.mem_get_info()
        t0 = time.perf_counter()
        for m, r in zip(scans_meta, rs):
            if a.no_autotune:
                m["block_size"] = int(r.cfg.block_size)
            else:
                best, table = autotune_block_size(r)
                m["block_size"] = best
                m["block_search_ms_per_iteration"] = {t[0]: round(t[1] * 1e3, 3) for t in table}
        t_tune = time.perf_counter() - t0
        iters = int(rs[0].cfg.iterations)
        assert all(int(r.cfg.iterations) == iters for r in rs)
        units = sum(m["recon_histories"] for m in scans_meta) * iters
        out = {}
        images = {}
        for mode in ("sequential", "concurrent", "persistent"):
            best = None
            for _ in range(a.reps):
                sec, im = drop_phase(rs, iters, mode)
                best = sec if best is None else min(best, sec)
            images[mode] = im
            out[mode] = {"seconds": best, "histories_iterations_per_second": units / best}
        worst = max(float(np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-30))
                    for x, y in zip(images["persistent"], images["concurrent"]))
    finally:
        for r in rs:
            r.close()
    print(json.dumps({
        "workload": "%d ellipsoid scans (seeds %d-%d), %d-%d histories log-uniform, grids %s, %d DROP iterations"
                    % (a.scans, a.seed, a.seed + a.scans - 1, min(m["histories"] for m in scans_meta),
                       max(m["histories"] for m in scans_meta), sorted({m["grid"] for m in scans_meta}), iters),
        "scans": scans_meta, "total_histories": sum(m["histories"] for m in scans_meta),
        "prepare_seconds": t_prep, "block_search_seconds": t_tune,
        "device_memory_in_use_gb": (total - free) / 1e9,
        "drop_phase": out, "timing": "best of %d wall-clock runs of the whole DROP phase (all scans)" % a.reps,
        "max_relative_l2_persistent_vs_concurrent": worst}))

if __name__ == "__main__":
    main()
