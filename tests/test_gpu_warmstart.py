"""The learned warm start end to end on the GPU: training pairs from the reference
sequence, training with the tensor-core kernels, and what the trained network
gains over the FBP start on held-out phantoms (needs a GPU).

Training and held-out phantoms are both curated: a scan whose 20-iteration plain
DROP result is further from the phantom than its FBP start (plain DROP diverges
in a few voxels on some random phantoms) is skipped."""
import numpy as np
import pytest

pytest.importorskip("torch")
from pct_gb300 import cnn, warmstart  # noqa: E402

pytestmark = pytest.mark.gpu

HIST, BLOCK = 10_000_000, 200000


@pytest.fixture(scope="module")
def trained():
    pairs, _ = warmstart.curated_pairs(3000, 12, HIST, BLOCK)
    assert len(pairs) == 12
    held_out, _ = warmstart.curated_pairs(3100, 2, HIST, BLOCK)
    net = cnn.Net(warmstart.SLICES, warmstart.COLS, warmstart.COLS)
    net.init(1)
    losses = warmstart.train(net, pairs, 2000, lr=5e-4, lr_final=5e-5)
    yield net, held_out, losses
    net.close()


def test_training_lowers_the_loss(trained):
    net, held_out, losses = trained
    assert np.mean(losses[-100:]) < 0.85 * np.mean(losses[:100]), (np.mean(losses[:100]), np.mean(losses[-100:]))


def test_learned_start_is_closer_to_the_phantom(trained):
    """On held-out phantoms the learned start has a lower voxel RSP error than the FBP
    start it replaces, and DROP from it stays finite (each phantom).  The
    region-mean errors are printed: with 12 training pairs the network's bias in
    the material means is not what it gains (its loss is the voxel distance to
    20-iteration DROP images)."""
    net, held_out, losses = trained
    for seed in [p["seed"] for p in held_out]:
        fbp = warmstart.run_drop(seed, HIST, BLOCK, 2, None)
        lrn = warmstart.run_drop(seed, HIST, BLOCK, 2, net)
        print("seed %d: region-mean error FBP start %.2f%%, learned start %.2f%%; voxel RMSE %.2f%% / %.2f%%"
              % (seed, fbp["region_error_pct"][0], lrn["region_error_pct"][0], fbp["voxel_rmse_pct"][0],
                 lrn["voxel_rmse_pct"][0]))
        assert lrn["voxel_rmse_pct"][0] < fbp["voxel_rmse_pct"][0], (seed, fbp["voxel_rmse_pct"], lrn["voxel_rmse_pct"])
        assert all(np.isfinite(lrn["region_error_pct"])) and lrn["residual"][1] > 0


def test_learned_start_is_closer_to_its_target(trained):
    """What the network is trained for, on held-out phantoms: its output is closer (RMS
    over the hull) to the phantom's 20-iteration plain DROP image than the FBP start
    it is given."""
    net, held_out, losses = trained
    for p in held_out:
        out = net.forward(p["x0"], p["hull"])
        inside = p["hull"] > 0
        d_fbp = float(np.sqrt(np.mean((p["x0"][inside] - p["target"][inside]) ** 2)))
        d_lrn = float(np.sqrt(np.mean((out[inside] - p["target"][inside]) ** 2)))
        assert d_lrn < d_fbp, (p["seed"], d_fbp, d_lrn)
