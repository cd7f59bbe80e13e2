"""Learned warm start for DROP: training pairs, training and evaluation.

The workload follows the learned-start configuration at a scale one GPU can
run in minutes: seeded ellipsoid phantoms of the batched-scan family
(phantoms.ellipsoids) on a 128 x 128 x 16 grid.  For each seed the reference
sequence runs through define_initial_iterate (x0 = FBP x hull, the hull),
and `target_iterations` plain DROP iterations from x0 give the training
target.  The network (cnn.Net) learns x0, hull -> target; at reconstruction
time pct_cnn_warm_start replaces x0 before the endpoints and DROP (the
reference's X_K0 = IMPORT hook).

Evaluation on held-out seeds runs DROP from both starts on the same rows with
the same block size and lambda, one iteration per call, and records per
iteration the RSP error against the phantom (region means, as in the bench
line), the binary64 relative residual and the device time, so that
iterations and wall time to an error target can be compared.
"""
import time

import numpy as np

from . import cnn, phantoms, recon

COLS, SLICES = 128, 16


def workload(seed, histories):
    return phantoms.ellipsoids(seed, num_histories=histories, cols=COLS, slices=SLICES)


def scan(seed, histories, block_size, lam=0.1):
    """The reference sequence through define_initial_iterate; returns (workload, config, Reconstruction)."""
    w = workload(seed, histories)
    over = dict(w.config)
    over.update(block_size=block_size, lambda_=lam)
    cfg = phantoms.make_config(over)
    data, angles = phantoms.generate(w)
    return w, cfg, recon.run_full(cfg, data, angles)


def regions(w, cfg, k=3):
    """Per material: the voxels whose (2k+1)^2 in-slice neighbourhood is that material only."""
    g = phantoms.geometry(cfg)
    t3 = phantoms.voxelize(w).reshape(g.slices, g.rows, g.columns)
    pad = np.pad(t3, ((0, 0), (k, k), (k, k)), mode="edge")
    same = t3 > 0
    for dy in range(2 * k + 1):
        for dx in range(2 * k + 1):
            same &= pad[:, dy:dy + g.rows, dx:dx + g.columns] == t3
    truth = t3.ravel()
    roi = same.ravel()
    mats = [(float(v), roi & (truth == v)) for v in np.unique(truth[roi])]
    return truth, roi, [(v, m) for v, m in mats if m.sum() >= 50]


def region_error(x, mats):
    """RMS over materials of the relative error of the region-mean RSP, in percent."""
    return float(np.sqrt(np.mean([((x[m].mean() - v) / v) ** 2 for v, m in mats])) * 100)


def make_pair(seed, histories, block_size, target_iterations=20, lam=0.1):
    """(x0, hull, target, truth) of one seed."""
    w, cfg, r = scan(seed, histories, block_size, lam)
    try:
        x0 = r.array("X0")
        hull = r.array("X_HULL_FILTERED")
        r.collect_mlp_endpoints()
        r.mlp_rows()
        r.drop(target_iterations)
        target = r.array("X")
    finally:
        r.close()
    truth = phantoms.voxelize(w)
    return {"x0": x0, "hull": hull, "target": target, "truth": truth, "seed": seed}


def improved(pair):
    """True when the pair's DROP target is closer to the phantom (RMS inside the hull) than
    its FBP start: on some phantoms plain DROP diverges in a few voxels, and such targets
    are not used for training."""
    h = pair["hull"] > 0
    e0 = np.sqrt(np.mean((pair["x0"][h] - pair["truth"][h]) ** 2))
    et = np.sqrt(np.mean((pair["target"][h] - pair["truth"][h]) ** 2))
    return bool(et < e0)


def curated_pairs(first_seed, count, histories, block_size, target_iterations=20, lam=0.1, max_tries=None):
    """`count` training pairs from consecutive seeds, skipping those `improved` rejects;
    returns (pairs, seeds tried)."""
    pairs, s = [], first_seed
    max_tries = max_tries or 4 * count
    while len(pairs) < count and s < first_seed + max_tries:
        p = make_pair(s, histories, block_size, target_iterations, lam)
        if improved(p):
            pairs.append(p)
        s += 1
    return pairs, s - first_seed


def train(net, pairs, steps, lr=1e-3, lr_final=1e-4, seed=0, log_every=0, target_key="target"):
    """Adam over randomly drawn pairs (cosine-decayed learning rate) towards pair[target_key]
    ("target": the pair's plain DROP image; "truth": the phantom's RSP map); returns the loss
    per step."""
    rng = np.random.default_rng(seed)
    losses = []
    for s in range(steps):
        p = pairs[int(rng.integers(len(pairs)))]
        a = lr_final + 0.5 * (lr - lr_final) * (1 + np.cos(np.pi * s / max(steps - 1, 1)))
        losses.append(net.train_step(p["x0"], p["hull"], p[target_key], float(a)))
        if log_every and s % log_every == 0:
            print("step %d loss %.4g" % (s, losses[-1]), flush=True)
    return losses


def run_drop(seed, histories, block_size, iterations, net=None, lam=0.1):
    """DROP from the FBP start (net None) or from the learned start; per iteration (index 0 =
    the start) the region error (%), the voxel RSP RMSE (%), the relative residual and the
    cumulative device seconds (the network's inference included for the learned start)."""
    w, cfg, r = scan(seed, histories, block_size, lam)
    truth, roi, mats = regions(w, cfg)
    try:
        t_net = 0.0
        if net is not None:
            t0 = time.perf_counter()
            net.warm_start(r)
            t_net = time.perf_counter() - t0
        r.collect_mlp_endpoints()
        r.mlp_rows()
        x = r.array("X")
        err = [region_error(x, mats)]
        rmse = [float(np.sqrt(np.mean((x[roi] - truth[roi]) ** 2)) * 100)]
        resid, secs = [None], [t_net]
        for _ in range(iterations):
            st = r.drop(1)
            x = r.array("X")
            err.append(region_error(x, mats))
            rmse.append(float(np.sqrt(np.mean((x[roi] - truth[roi]) ** 2)) * 100))
            resid.append(float(st.residual[0]))
            secs.append(secs[-1] + st.seconds)
    finally:
        r.close()
    return {"region_error_pct": err, "voxel_rmse_pct": rmse, "residual": resid, "seconds": secs,
            "network_seconds": t_net}


def first_at_or_below(values, target):
    return next((k for k, v in enumerate(values) if v is not None and v <= target), None)


def conv_flops(nv):
    """Multiply-add FLOPs of one forward pass over nv voxels: as defined (real channels) and as
    the tensor cores execute them (channels padded to 16)."""
    real = sum(2 * 27 * ci * co for ci, co in cnn.LAYERS) * nv
    padded = sum(2 * 27 * max(ci, 16) * max(co, 16) for ci, co in cnn.LAYERS) * nv
    return real, padded


def time_forward(net, pair, reps=20):
    """Seconds per network forward pass on device-resident input and output (each call
    returns after its stream has finished)."""
    import torch
    x0 = torch.from_numpy(pair["x0"]).cuda()
    hull = torch.from_numpy(pair["hull"]).cuda()
    out = torch.empty_like(x0)
    torch.cuda.synchronize()
    net.forward_device(x0.data_ptr(), hull.data_ptr(), out.data_ptr())
    t0 = time.perf_counter()
    for _ in range(reps):
        net.forward_device(x0.data_ptr(), hull.data_ptr(), out.data_ptr())
    return (time.perf_counter() - t0) / reps


def experiment(n_train, eval_seeds, histories=10_000_000, block_size=200000, lam=0.1, target_iterations=20,
               steps=3000, lr=5e-4, eval_iterations=30, net_seed=1, log=None, first_train_seed=2000,
               curate_eval=True, target="drop"):
    """Trains a network on `n_train` curated pairs (seeds from `first_train_seed` on) and
    compares the two starts on `eval_seeds` (with `curate_eval`, on those whose own plain
    DROP target passes `improved`).  `target`: "drop" trains towards the pairs' plain DROP
    images (the method's own output); "truth" towards the phantoms' RSP maps (known for
    synthetic phantoms only).

    Per held-out seed and start: iterations and wall time (DROP device time, plus the
    network's inference for the learned start) until the voxel RSP RMSE is at or below
    the lowest the FBP start reaches in `eval_iterations`, until the region error is
    <= 0.5%, until it is within 10% of the lowest region error the FBP start reaches, and
    until the
    binary64 relative residual is at or below the FBP start's residual after
    `target_iterations` (the same residual stop for both)."""
    t0 = time.perf_counter()
    pairs, tried = curated_pairs(first_train_seed, n_train, histories, block_size, target_iterations, lam)
    t_pairs = time.perf_counter() - t0
    net = cnn.Net(SLICES, COLS, COLS)
    try:
        net.init(net_seed)
        t0 = time.perf_counter()
        losses = train(net, pairs, steps, lr=lr, lr_final=lr / 10, log_every=log or 0,
                       target_key="truth" if target == "truth" else "target")
        t_train = time.perf_counter() - t0
        t_fwd = time_forward(net, pairs[0])
        per_seed = []
        for s in eval_seeds:
            if curate_eval and not improved(make_pair(s, histories, block_size, target_iterations, lam)):
                continue
            fbp = run_drop(s, histories, block_size, eval_iterations, None, lam)
            lrn = run_drop(s, histories, block_size, eval_iterations, net, lam)
            best_err = min(fbp["region_error_pct"])
            best_rmse = min(fbp["voxel_rmse_pct"])
            ref_res = fbp["residual"][target_iterations]
            row = {"seed": s, "fbp": fbp, "learned": lrn}
            for name, crit in (("voxel_rmse_at_plain_best",
                                lambda r: first_at_or_below(r["voxel_rmse_pct"], best_rmse * (1 + 1e-9))),
                               ("0.5pct", lambda r: first_at_or_below(r["region_error_pct"], 0.5)),
                               ("within_10pct_of_plain_best",
                                lambda r: first_at_or_below(r["region_error_pct"], 1.1 * best_err)),
                               ("residual_stop", lambda r: first_at_or_below(r["residual"], ref_res * (1 + 1e-9)))):
                for start in ("fbp", "learned"):
                    k = crit(row[start])
                    row["%s_%s_iterations" % (start, name)] = k
                    row["%s_%s_seconds" % (start, name)] = row[start]["seconds"][k] if k is not None else None
            per_seed.append(row)
    finally:
        net.close()
    return {"pairs_seconds": t_pairs, "train_seconds": t_train, "forward_seconds": t_fwd, "losses": losses,
            "per_seed": per_seed,
            "histories": histories, "block_size": block_size, "lambda": lam, "steps": steps, "training_target": target,
            "train_seeds": [p["seed"] for p in pairs], "seeds_tried": tried,
            "eval_seeds": [r["seed"] for r in per_seed], "eval_seeds_tried": list(eval_seeds)}
