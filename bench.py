#!/usr/bin/env python3
"""Benchmark: histories/s per MLP+DROP iteration on the production-size scan.

Workload (the reference's production configuration on one GB300): a seeded
synthetic scan of a 10 cm-radius water cylinder with 8 inserts (RSP 0.3-1.8),
30M proton histories over 180 gantry angles, 256x256x32 voxels of
1x1x2.5 mm, 12 DROP iterations with block size 200000 and lambda 0.1.  The
synthetic generator stands in for the reference's PCTD scans (none ship).

A step is one pass of the hot path over the resident histories: the MLP
voxel rows of every recon history, then 12 DROP iterations (the iterate is
reset to x0 first).  `value` = recon histories x 12 / step time, with the
histories already in HBM.  `e2e` is the same metric for the whole
reference-facing call sequence on a fresh context (pct_process_chunk from
pinned host buffers through preprocessing, hulls, FBP, endpoints, MLP and
DROP, then reading the image back), per step.

  python bench.py [--steps K] [--warmup W] [--histories N] [--impl reference]

With --impl reference the step is the reference algorithm on the CPU (the C
restatement in oracle/, all host threads) on one full DROP block of the same
workload: its MLP rows and the 12 DROP iterations over it.
Under torchrun (N > 1) every rank runs the same workload on its own GPU
(replicas: the path has no cross-GPU exchange here) and `value` sums them.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "histories/s per MLP+DROP iteration"
UNIT = "histories*iterations/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--histories", type=int, default=None,
                    help="scan size (default: 30M for cfg2, 60M for cfg4)")
    ap.add_argument("--workload", default="cfg2", choices=["cfg2", "cfg3", "cfg4", "cfg5"],
                    help="cfg2 (the bench line: 256x256x32, 8-insert cylinder), cfg3 (16 batched ellipsoid scans, "
                         "2M-40M histories, DROP of all of them in one persistent launch per iteration), cfg4 "
                         "(320x320x64 head phantom) or cfg5 (learned warm start: train the CNN, compare FBP-start "
                         "and learned-start DROP)")
    ap.add_argument("--scans", type=int, default=16, help="cfg3: number of scans")
    ap.add_argument("--train-phantoms", type=int, default=64, help="cfg5: training phantoms")
    ap.add_argument("--eval-phantoms", type=int, default=8, help="cfg5: held-out phantoms")
    ap.add_argument("--train-steps", type=int, default=3000, help="cfg5: Adam steps")
    ap.add_argument("--warmstart-target", default="drop", choices=["drop", "truth"],
                    help="cfg5: train towards the pairs' 20-iteration plain DROP images (drop) or, as an extra "
                         "measurement, towards the phantoms' RSP maps (truth)")
    ap.add_argument("--chord-bf16", type=int, default=None, choices=[0, 1],
                    help="round chords to bfloat16 (default: the workload's setting; cfg4 uses bf16)")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--cpu-sample", type=int, default=60000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--drop-form", type=int, default=0, choices=[0, 1, 2, 3],
                    help="DROP block step: 0 scatter (default), 1 sorted, 2 tiled, 3 gather")
    ap.add_argument("--voxel-order", type=int, default=0, choices=[0, 1],
                    help="internal voxel order: 0 bricks where the grid allows (default), 1 linear")
    a = ap.parse_args()
    if a.histories is None:
        a.histories = 60_000_000 if a.workload == "cfg4" else 30_000_000
    return a


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    def __init__(self, gpu):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        self.f = os.fdopen(fd, "w")
        self.gpu = gpu
        self.p = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + q, "--format=csv,noheader",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:  # no nvidia-smi: the line reports no clock samples
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait()
        self.f.close()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1].split()[0]))
                    mx = max(mx, float(f[2].split()[0]))
                except ValueError:
                    continue
                for name, v in zip(["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"], f[5:9]):
                    if v.lower() == "active":
                        reasons.add(name)
        except OSError:
            pass
        finally:
            try:
                os.unlink(self.path)
            except OSError:
                pass
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx or None, "reasons": sorted(reasons),
                "samples": len(sm)}


def reduce_across_ranks(seconds, units, dist=None, device="cpu"):
    """Replica aggregation: the slowest rank's time and the work of all ranks
    (each rank runs its own scan; there is no data-path exchange)."""
    if dist is None:
        return float(seconds), float(units)
    import torch
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


def host_info():
    cpu = "unknown"
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                cpu = line.split(":", 1)[1].strip()
                break
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                cpu = line.split(":", 1)[1].strip()
    except Exception:
        pass
    return cpu, os.cpu_count()


def cpu_baseline(cfg, r, sample, iterations, threads):
    """The reference path (C restatement) on `sample` recon histories of the resident store."""
    from oracle import oracle
    keys = {"x_entry": "H_X_ENTRY", "y_entry": "H_Y_ENTRY", "z_entry": "H_Z_ENTRY", "x_exit": "H_X_EXIT",
            "y_exit": "H_Y_EXIT", "z_exit": "H_Z_EXIT", "xy_entry_angle": "H_XY_ENTRY_ANGLE",
            "xz_entry_angle": "H_XZ_ENTRY_ANGLE", "xy_exit_angle": "H_XY_EXIT_ANGLE", "xz_exit_angle": "H_XZ_EXIT_ANGLE",
            "WEPL": "H_WEPL", "first_voxel": "H_FIRST_VOXEL"}
    h = {k: r.array(v)[:sample].copy() for k, v in keys.items()}
    x0 = r.array("X0").astype(np.float64)
    return time_oracle(cfg, h, x0, iterations, threads)


def time_oracle(cfg, h, x0, iterations, threads):
    from oracle import oracle
    os.environ["OMP_NUM_THREADS"] = str(threads)
    n = len(h["WEPL"])
    t0 = time.perf_counter()
    offs, rows, chord = oracle.mlp_rows(cfg, h, threads=threads)
    x = x0.copy()
    x = oracle.drop(cfg, offs, rows, chord, h["WEPL"], x, iterations, cfg.block_size, float(np.float32(cfg.lambda_)),
                    threads=threads)
    dt = time.perf_counter() - t0
    return n * iterations / dt, dt, n


def mapped_repo_libraries():
    """Shared libraries of this repository mapped into the process (from /proc/self/maps)."""
    found = set()
    try:
        for line in open("/proc/self/maps"):
            path = line.split()[-1] if len(line.split()) >= 6 else ""
            if path.endswith(".so") and path.startswith(ROOT):
                found.add(os.path.relpath(path, ROOT))
    except OSError:
        pass
    return sorted(found)


def workload(a, rank):
    """The scan of this run (seeded per rank) and its configuration overrides."""
    from pct_gb300 import phantoms  # workload definitions (no library is mapped)
    make_workload = phantoms.cfg4 if a.workload == "cfg4" else phantoms.cfg2
    w = make_workload(num_histories=a.histories, seed=(4 if a.workload == "cfg4" else 2) + rank)
    over = dict(w.config)
    if a.chord_bf16 is not None:
        over["chord_bf16"] = a.chord_bf16
    over["drop_form"] = a.drop_form
    over["voxel_order"] = a.voxel_order
    return w, over


def describe(a, w, cfg, g, n, R):
    return ("%s: %d histories, %d recon histories, %d angles, %dx%dx%d, %d DROP iterations, block %d, lambda %.2g,"
            " %s chords" % (a.workload, n, R, w.num_angles, g.columns, g.rows, g.slices, cfg.iterations,
                            cfg.block_size, cfg.lambda_, "bf16" if cfg.chord_bf16 else "binary32"))


def run_reference_arm(a, ws, rank):
    """--impl reference: the reference algorithm on the host cores, on this bench's workload.

    Setup, untimed: the C restatement of the reference's main() sequence (oracle/) on the
    whole scan: preprocessing, hulls, cuts, FBP, initial iterate, hull endpoints.  A step:
    the MLP rows of the first DROP block (block_size recon histories, one full block) and
    the DROP iterations over that block, on all host threads.  The histories come from the
    host build of the seeded generator, so no CUDA library is mapped by this arm."""
    if rank != 0:
        return
    from oracle import oracle
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    w, over = workload(a, 0)
    cfg = oracle.make_config(over)
    g = oracle.geometry(cfg)
    data, angles = oracle.generate(w)
    n = data.shape[1]
    t0 = time.perf_counter()
    ora = oracle.run_pipeline(cfg, data, angles, iterations=0, keep_history=True)
    setup_s = time.perf_counter() - t0
    del data, angles
    hr = ora["_hr"]
    R = len(hr["WEPL"])
    sample = min(R, cfg.block_size)
    h = {k: v[:sample].copy() for k, v in hr.items()}
    x0 = ora["x_k0"].astype(np.float64)
    del ora, hr
    iters = cfg.iterations
    for _ in range(a.warmup):
        time_oracle(cfg, h, x0, iters, threads)
    times = []
    for _ in range(a.steps):
        v, dt, _ = time_oracle(cfg, h, x0, iters, threads)
        times.append(dt)
    value = sample * iters * a.steps / sum(times)
    cpu, ncores = host_info()
    sample_text = ("the first DROP block (%d of %d recon histories) per step: its MLP rows and %d DROP iterations "
                   "over it, on %d threads of %s; setup (preprocessing .. endpoints of the whole scan) %.1f s, "
                   "untimed" % (sample, R, iters, threads, cpu, setup_s))
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
           "ms_per_step": 1e3 * sum(times) / a.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded phantom generator, PCTD layout)",
           "impl": "reference",
           "config": {"workload": describe(a, w, cfg, g, n, R), "sample": sample_text},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample_text},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "libraries_mapped": mapped_repo_libraries()}
    print(json.dumps(out))


def run_warmstart(a, ws, rank):
    """--workload cfg5: the learned warm start.  Trains the CNN on FBP -> 20-iteration-DROP pairs
    of seeded ellipsoid phantoms (128 x 128 x 16 grid) with the library's tensor-core kernels,
    then runs DROP from the FBP start and from the learned start on held-out phantoms.
    `value` = mean over held-out phantoms of (FBP-start seconds / learned-start seconds) to reach
    a voxel RSP RMSE at or below the lowest the FBP start reaches in 30 iterations; the line
    also gives the region-mean targets and the residual stop."""
    if rank != 0:
        return
    from pct_gb300 import warmstart
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    with Clocks(0) as clk:
        res = warmstart.experiment(a.train_phantoms, range(1001, 1001 + a.eval_phantoms), steps=a.train_steps,
                                   target=a.warmstart_target)
    evaluated = len(res["eval_seeds"])
    nv = warmstart.COLS * warmstart.COLS * warmstart.SLICES
    real, padded = warmstart.conv_flops(nv)
    tf = padded / res["forward_seconds"] / 1e12
    peak = peaks.get("bf16_tflops", 1900.0)
    summary = {}
    for target in ("voxel_rmse_at_plain_best", "0.5pct", "within_10pct_of_plain_best", "residual_stop"):
        rows = res["per_seed"]
        it = {st: [r["%s_%s_iterations" % (st, target)] for r in rows] for st in ("fbp", "learned")}
        sec = {st: [r["%s_%s_seconds" % (st, target)] for r in rows] for st in ("fbp", "learned")}
        both = [(f, l) for f, l in zip(sec["fbp"], sec["learned"]) if f is not None and l is not None and l > 0]
        summary[target] = {"iterations": it, "seconds": sec,
                           "mean_time_ratio_fbp_over_learned": float(np.mean([f / l for f, l in both])) if both else None,
                           "reached": {st: sum(v is not None for v in it[st]) for st in it}}
    rows = res["per_seed"]
    start = {st: {"region_error_pct": float(np.mean([r[st]["region_error_pct"][0] for r in rows])),
                  "voxel_rmse_pct": float(np.mean([r[st]["voxel_rmse_pct"][0] for r in rows]))}
             for st in ("fbp", "learned")}
    value = summary["voxel_rmse_at_plain_best"]["mean_time_ratio_fbp_over_learned"]
    out = {"metric": "wall time to RSP RMSE target (the lowest voxel RMSE plain DROP reaches): FBP start / learned "
                     "start", "value": value, "unit": "x",
           "n_gpus": ws, "steps": res["steps"], "warmup": 0, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "bf16 (network), f32 (DROP)",
           "data": "synthetic (seeded ellipsoid phantoms of the batched-scan generator)",
           "config": {"workload": "cfg5: %d training (of %d seeds tried: targets where plain DROP diverged are "
                                  "skipped) / %d of %d held-out phantoms (the same rule), 128x128x16, %d histories "
                                  "each, DROP block %d, lambda %.2g, training targets = %s, %d Adam steps"
                                  % (len(res["train_seeds"]), res["seeds_tried"], evaluated, a.eval_phantoms,
                                     res["histories"],
                                     res["block_size"], res["lambda"],
                                     "the phantoms' RSP maps (an extra measurement: known for synthetic phantoms "
                                     "only)" if a.warmstart_target == "truth" else "20 plain DROP iterations",
                                     res["steps"])},
           "targets": summary, "start_error": start,
           "training": {"pairs_seconds": res["pairs_seconds"], "train_seconds": res["train_seconds"],
                        "seconds_per_step": res["train_seconds"] / res["steps"],
                        "loss_first_50": float(np.mean(res["losses"][:50])),
                        "loss_last_50": float(np.mean(res["losses"][-50:]))},
           "network_forward": {"seconds": res["forward_seconds"], "voxels": nv, "flops_real": real,
                               "flops_tensor_core": padded, "tflops": tf,
                               "frac_of_bf16_peak": tf / peak,
                               "note": "host-timed pct_cnn_forward on device-resident input and output (the "
                                       "call returns after its stream finishes)"},
           "per_seed_region_error_pct": {str(r["seed"]): {"fbp": r["fbp"]["region_error_pct"][:16],
                                                          "learned": r["learned"]["region_error_pct"][:16]}
                                         for r in rows},
           "clocks": clk.summary()}
    print(json.dumps(out))


def run_batched(a, ws, rank):
    """--workload cfg3: many uneven scans on one GPU.  `--scans` seeded ellipsoid scans (histories
    log-uniform in 2M-40M, grids drawn per seed) are prepared through their MLP rows (rows packed),
    each gets its DROP block size from autotune_block_size, and a step is the DROP phase of all of
    them: 12 iterations of every scan from its initial iterate in one persistent cooperative launch
    per iteration, one captured graph per iteration (pct_drop_many).  The step time is the
    library's CUDA-event time on the launching stream; `value` = recon histories of all scans x 12
    / step time.  The same phase with one context after another and with concurrent contexts (a
    host thread and stream each; wall clock) is given beside it."""
    if rank != 0:
        return
    import math
    import random

    import torch
    from pct_gb300 import batch, phantoms, recon
    torch.cuda.set_device(0)
    rng = random.Random(100)
    rs, meta = [], []
    try:
        for k in range(a.scans):
            n = int(round(math.exp(rng.uniform(math.log(2e6), math.log(40e6)))))
            w = phantoms.ellipsoids(100 + k, num_histories=n)
            data, angles = phantoms.generate(w)
            cfg = phantoms.make_config(w.config)
            rs += batch.prepare_scans([(cfg, data, angles)])
            del data, angles
            g = phantoms.geometry(cfg)
            best, _ = batch.autotune_block_size(rs[-1])
            meta.append({"seed": 100 + k, "histories": n, "grid": "%dx%dx%d" % (g.columns, g.rows, g.slices),
                         "recon_histories": rs[-1].counts()["reconstruction_histories"], "block_size": best})
        iters = int(rs[0].cfg.iterations)
        units = sum(m["recon_histories"] for m in meta) * iters

        def step():
            for r in rs:
                r.reset_iterate()
            st = recon.drop_many(rs, iters)
            return st[0].seconds

        for _ in range(a.warmup):
            step()
        with Clocks(0) as clk:
            times = [step() for _ in range(a.steps)]
        launches = a.steps * iters * 2  # per iteration: k_drop_many and k_many_store_resid
        sec = float(np.mean(times))
        other = {}
        for mode in ("sequential", "concurrent"):
            t, _ = batch.drop_phase(rs, iters, mode)
            other[mode] = {"seconds_wall": t, "histories_iterations_per_second": units / t}
    finally:
        for r in rs:
            r.close()
    out = {"metric": "histories/s per DROP iteration (all scans)", "value": units / sec, "unit": UNIT,
           "n_gpus": 1, "steps": a.steps, "warmup": a.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded ellipsoid phantoms)",
           "config": {"workload": "cfg3: %d ellipsoid scans (seeds 100-%d), %d-%d histories log-uniform in 2M-40M, "
                                  "%d recon histories in all, grids %s, %d DROP iterations, block size per scan by "
                                  "autotune_block_size" % (a.scans, 99 + a.scans, min(m["histories"] for m in meta),
                                                           max(m["histories"] for m in meta), units // iters,
                                                           sorted({m["grid"] for m in meta}), iters),
                      "l2": "inputs larger than L2 (rows of all scans resident)",
                      "step": "pct_drop_many: one cooperative launch per iteration over every scan's blocks, one "
                              "captured graph per iteration; CUDA events on the launching stream",
                      "scans": meta},
           "other_modes": other, "gpu_launches": int(launches), "clocks": clk.summary()}
    print(json.dumps(out))


def main():
    a = parse()
    ws, rank, local = dist_env()
    if a.workload == "cfg3":
        if a.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference runs one scan per block loop; "
                                                                      "no batched form to time"}))
            return
        run_batched(a, ws, rank)
        return
    if a.workload == "cfg5":
        if a.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference has no learned warm start"}))
            return
        run_warmstart(a, ws, rank)
        return
    if a.impl == "reference":
        run_reference_arm(a, ws, rank)
        return
    import torch
    from pct_gb300 import phantoms, recon
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    w, over = workload(a, rank)
    cfg = phantoms.make_config(over)
    iters = cfg.iterations
    data, angles = phantoms.generate(w)
    n = data.shape[1]

    # ---- setup: everything before the hot path, through the public API -------------
    r = recon.Reconstruction(cfg, device=local)
    r.reserve(n)
    r.process_chunk(data, angles)
    r.hull_detection_finish()
    r.statistical_cuts()
    r.FBP()
    r.hull_selection()
    r.define_initial_iterate()
    r.collect_mlp_endpoints()
    R = r.counts()["reconstruction_histories"]
    stream = torch.cuda.ExternalStream(r.stream(), device=dev)

    def step():
        r.reset_iterate()
        r.mlp_rows()
        return r.drop(iters)

    for _ in range(a.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    c0 = r.counts()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        drop_s = 0.0
        for _ in range(a.steps):
            st = step()
            drop_s += st.seconds
            form_ran = st.drop_form
        ev1.record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t_local = ev0.elapsed_time(ev1) * 1e-3
    t, units = reduce_across_ranks(t_local, R * iters * a.steps, dist, dev)
    c1 = r.counts()
    launches = c1["kernel_launches"] - c0["kernel_launches"]
    rows = c1["row_entries"]
    value = units / t
    mlp_s = t - drop_s
    drop_iter_s = drop_s / (a.steps * iters)

    # ---- roofline of the dominant kernel ----------------------------------------------
    # One DROP iteration (the dominant part of a step: 12 of them per MLP pass).
    # Algorithmic bytes per recon history and iteration: 4 B WEPL + 8 B row start
    # + 4 B row length + 4 B chord + 4 B row scale 1/(c |a_i|) + 4 B per row
    # entry (voxel index); the image
    # gathers and update reductions stay in L2 and are not counted.  The launch
    # timed is one DROP iteration (all blocks: k_drop_rows + k_drop_relax per
    # block in the scatter form) with CUDA events on the context stream.
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    drop_bytes = R * 24 + rows * 4
    achieved = drop_bytes / drop_iter_s / 1e9
    # the gather form also streams its column lists (4 B per stored entry) and
    # their slice offsets (8 B per 32 voxels per block) every iteration
    list_entries = c1["drop_list_entries"]
    nblocks = (R + cfg.block_size - 1) // cfg.block_size
    stream_bytes = drop_bytes + (list_entries * 4 + nblocks * ((phantoms.geometry(cfg).num_voxels + 31) // 32) * 8
                                 if list_entries else 0)
    forms = {0: "k_drop_rows + k_drop_relax (scatter)", 1: "k_drop_rows + k_drop_relax (sorted)",
             2: "k_tile_fwd + k_tile_rows + k_tile_bwd (tiled)", 3: "k_gather_rows + k_gather_cols (gather)"}
    dom = "one DROP iteration: %s" % forms[a.drop_form]
    traffic = None
    tr = {}
    try:
        tr = json.load(open(os.path.join(ROOT, "profiles", "roofline_traffic.json")))
        tm = tr.get("drop_form_%d" % a.drop_form)
        if tm:  # DRAM bytes of one iteration, scaled from a smaller ncu capture
            nblocks = (R + cfg.block_size - 1) // cfg.block_size
            traffic = tm["ratio_to_algorithmic"] * drop_bytes + tm["per_block_bytes"] * nblocks
    except Exception:
        pass

    # The bound that applies: L2 reduction sectors.  The sectors per row entry
    # (reductions into x_update, reads of the row stream and of the iterate)
    # come from an ncu capture of a full block; the ceiling is measured here by
    # pct_probe_l2 (pseudo-random float reductions into an 8 MB L2-resident
    # array, and the same with a gather before each reduction).
    roofline_l2 = None
    try:
        from pct_gb300 import _capi
        lib = _capi.load()
        lib.pct_probe_l2.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double)]
        red_peak, pair_peak = C.c_double(0.0), C.c_double(0.0)
        if lib.pct_probe_l2(local, 0, C.byref(red_peak)) == 0 and lib.pct_probe_l2(local, 1, C.byref(pair_peak)) == 0:
            tm = tr.get("drop_form_0", {}) if a.drop_form == 0 and a.voxel_order == 0 else {}
            spe = tm.get("l2_reduction_sectors_per_entry")
            rpe = tm.get("l2_read_sectors_per_entry")
            if spe and rpe:
                red_rate = rows * spe / drop_iter_s
                roofline_l2 = {
                    "bound": "l2 reduction sectors", "kernel": dom, "achieved": red_rate / 1e9,
                    "peak": red_peak.value / 1e9, "unit": "G sectors/s", "frac": red_rate / red_peak.value,
                    "read_sectors_achieved": rows * rpe / drop_iter_s / 1e9,
                    "peak_with_gather_before_each_reduction": pair_peak.value / 1e9,
                    "sectors_per_entry": {"reductions": spe, "reads": rpe, "source": tm.get("l2_source")},
                    "peak_source": "measured live: pct_probe_l2, pseudo-random red.global.add.f32 into an 8 MB "
                                   "L2-resident array, one element per 32-byte sector"}
    except Exception as ex:  # the probe is optional evidence; the bench line stands without it
        roofline_l2 = {"unavailable": str(ex)[:200]}

    # MLP row generation, once per step: 48 B per recon history read (10 float
    # endpoint values, WEPL, first voxel) + 4 B per row entry and 4 B row length
    # written.
    mlp_bytes = R * 52 + rows * 4
    mlp_achieved = mlp_bytes / (mlp_s / a.steps) / 1e9

    # ---- convergence: RSP error against the phantom per iteration (not timed) --------
    # FBP x hull start, the same rows, one DROP iteration per call.  Regions: voxels
    # whose 7x7 in-slice neighbourhood is one phantom material (3 voxels away from
    # any boundary), grouped by material.  Reported: the RMS over materials of the
    # relative error of the region mean RSP, and the per-voxel RMSE (noise included).
    g = phantoms.geometry(cfg)
    t3 = phantoms.voxelize(w).reshape(g.slices, g.rows, g.columns)
    k = 3
    pad = np.pad(t3, ((0, 0), (k, k), (k, k)), mode="edge")
    same = t3 > 0
    for dy in range(2 * k + 1):
        for dx in range(2 * k + 1):
            same &= pad[:, dy:dy + g.rows, dx:dx + g.columns] == t3
    truth = t3.ravel()
    roi = same.ravel()
    mats = [(float(v), roi & (truth == v)) for v in np.unique(truth[roi])]
    mats = [(v, m) for v, m in mats if m.sum() >= 200]

    def errors(x):
        region = [(x[m].mean() - v) / v for v, m in mats]
        return (float(np.sqrt(np.mean(np.square(region))) * 100),
                float(np.sqrt(np.mean((x[roi] - truth[roi]) ** 2)) * 100))

    r.reset_iterate()
    r.mlp_rows()
    xs = [r.array("X")]
    errs = [errors(xs[0])]
    for _ in range(iters):
        r.drop(1)
        xs.append(r.array("X"))
        errs.append(errors(xs[-1]))
    # the binary32 iterates against a binary64 run of the same iterations on the same rows
    x64 = xs[0].astype(np.float64)
    fp64_err = []
    for k in range(iters):
        x64, _ = r.drop_fp64(1, x64)
        fp64_err.append(float(np.linalg.norm(xs[k + 1] - x64) / np.linalg.norm(x64)))
    del xs
    hit = next((k for k, e in enumerate(errs) if e[0] <= 0.5), None)
    accuracy = {"region_mean_rsp_error_pct_per_iteration": [e[0] for e in errs],
                "voxel_rsp_rmse_pct_per_iteration": [e[1] for e in errs],
                "regions": "%d materials, %d voxels at least 3 voxels (in-slice) from a material boundary"
                           % (len(mats), int(sum(m.sum() for _, m in mats))),
                "start": "FBP x hull (iteration 0)",
                "seconds_to_region_error_0.5pct": (mlp_s / a.steps + hit * drop_iter_s) if hit is not None else None,
                "fp64_rel_l2_per_iteration": fp64_err,
                "fp64_reference": "pct_drop_fp64: the same iterations on the same rows with binary64 chord, dot, "
                                  "update sums and iterate (relative L2 of the binary32 iterate against it)"}

    # ---- end to end through the public API with host buffers --------------------------
    pinned = torch.empty((13, n), dtype=torch.float32, pin_memory=True)
    pinned.numpy()[:] = data
    pang = torch.empty(n, dtype=torch.float32, pin_memory=True)
    pang.numpy()[:] = angles
    e2e_t = 0.0
    nv = phantoms.geometry(cfg).num_voxels
    xhost = torch.empty(nv, dtype=torch.float32, pin_memory=True)
    for _ in range(a.e2e_steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        q = recon.Reconstruction(cfg, device=local)
        q.reserve(n)
        q.process_chunk(pinned.numpy(), pang.numpy())
        q.hull_detection_finish()
        q.statistical_cuts()
        q.FBP()
        q.hull_selection()
        q.define_initial_iterate()
        q.image_reconstruction_GPU()
        nb = C.c_size_t(nv * 4)
        q._call("pct_get_array", recon.ARRAY_ID["X"], C.c_void_p(xhost.data_ptr()), C.byref(nb))
        e2e_t += time.perf_counter() - t0
        q.close()
    e2e_t, e2e_units = reduce_across_ranks(e2e_t, R * iters * a.e2e_steps, dist, dev)
    e2e_value = e2e_units / e2e_t

    # ---- CPU baseline (rank 0, bounded sample) -------------------------------------------
    cpu_b = None
    if rank == 0 and not a.no_cpu_baseline:
        cpu, ncores = host_info()
        v, dt, ns = cpu_baseline(cfg, r, a.cpu_sample, iters, 1)
        cpu_b = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
                 "sample": "%d recon histories x %d iterations (MLP rows + DROP) on 1 core of %s (%d cores), %.1f s"
                           % (ns, iters, cpu, ncores, dt)}
    r.close()
    clocks = clk.summary()
    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": t / a.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded phantom generator, PCTD layout)",
            "config": {"workload": describe(a, w, cfg, g, n, R),
                       "row_entries": rows, "parallelism": "replicas" if ws > 1 else "single GPU",
                       "l2": "inputs larger than L2 (MLP rows %.1f GB)" % (rows * 4 / 1e9),
                       "drop_form": forms[a.drop_form], "drop_form_ran": forms.get(form_ran, str(form_ran)),
                       "voxel_order": ["bricks", "linear"][a.voxel_order],
                       "mlp_fp64_samples_per_step": (c1["mlp_fp64_samples"]),
                       "mlp_queue_capacity": max(R, 1 << 20),
                       "rows_ms_per_step": mlp_s / a.steps * 1e3, "drop_ms_per_iteration": drop_iter_s * 1e3},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(n * 14 * 4),
                    "d2h_bytes_per_step": int(nv * 4), "seconds_per_step": e2e_t / a.e2e_steps},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "traffic": traffic,
                         "algorithmic_bytes": drop_bytes, "stream_bytes": stream_bytes,
                         "column_list_entries": list_entries,
                         "peak_source": "of measured (MEASURED_PEAKS.json hbm_gbs)" if peaks else "of fallback"},
            "roofline_l2": roofline_l2,
            "roofline_mlp": {"bound": "hbm", "kernel": "MLP row generation (k_mlp_bound .. k_mlp_dedupe)",
                             "achieved": mlp_achieved, "peak": hbm_peak, "unit": "GB/s",
                             "frac": mlp_achieved / hbm_peak, "algorithmic_bytes": mlp_bytes},
            "accuracy": accuracy,
            "cpu_baseline": cpu_b, "gpu_launches": launches, "clocks": clocks,
        }
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
