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
    yield net, [p["seed"] for p in held_out], losses
    net.close()


def test_training_lowers_the_loss(trained):
    net, held_out, losses = trained
    assert np.mean(losses[-100:]) < 0.85 * np.mean(losses[:100]), (np.mean(losses[:100]), np.mean(losses[-100:]))


def test_learned_start_is_closer_to_the_phantom(trained):
    """On held-out phantoms the learned start has a lower voxel RSP error than the FBP
    start it replaces (each phantom) and a lower region-mean error (mean over the
    phantoms), and DROP from it stays finite."""
    net, held_out, losses = trained
    reg_fbp, reg_lrn = [], []
    for seed in held_out:
        fbp = warmstart.run_drop(seed, HIST, BLOCK, 2, None)
        lrn = warmstart.run_drop(seed, HIST, BLOCK, 2, net)
        reg_fbp.append(fbp["region_error_pct"][0])
        reg_lrn.append(lrn["region_error_pct"][0])
        assert lrn["voxel_rmse_pct"][0] < fbp["voxel_rmse_pct"][0], (seed, fbp["voxel_rmse_pct"], lrn["voxel_rmse_pct"])
        assert all(np.isfinite(lrn["region_error_pct"])) and lrn["residual"][1] > 0
    assert np.mean(reg_lrn) < np.mean(reg_fbp), (reg_fbp, reg_lrn)
